/*
 * vk.h -- C ABI of the GB300-native VIKSHOBHA 2D GPE stepper (libvk.so).
 *
 * Drop-in boundary for the reference's Fortran hot path: the Fortran driver
 * (src/driver.f90) keeps reading parameter.txt / parameter_gpe.txt, writing
 * the wf / energy / spectra files and running the solve loop
 * (src/solve.f90); the routines it calls for the state update and the
 * diagnostics reductions come from here through ISO_C_BINDING.
 *
 * Conventions
 *  - Every entry point returns int status: VK_OK (0) or a negative VK_E_*
 *    code; vk_last_error() returns a message for the calling thread.
 *  - All array arguments are HOST pointers owned by the caller.
 *  - Complex arrays are interleaved (re, im) doubles, i.e. Fortran
 *    COMPLEX(C_DOUBLE_COMPLEX).
 *  - Physical layout psi(i1=x, i2=y), x fastest: element (x, y) at y*nx + x.
 *    Fourier layout kpsi(i2=ky, i1=kx), ky fastest: element (kx, ky) at
 *    kx*ny + ky -- the FFTW_MPI_TRANSPOSED_OUT layout of
 *    src/mod_fft.f90:143-146.
 *  - One context = one GPU state = one CUDA stream; a context is used from
 *    one host thread at a time.
 */
#ifndef VK_H
#define VK_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define VK_OK 0
#define VK_E_INVALID (-1)   /* bad argument or parameter value          */
#define VK_E_CUDA (-2)      /* a CUDA runtime call failed               */
#define VK_E_NOMEM (-3)     /* device or host allocation failed          */
#define VK_E_IO (-4)        /* file missing, truncated or malformed     */
#define VK_E_STATE (-5)     /* call out of order (e.g. no psi set yet)  */
#define VK_E_NUMERIC (-6)   /* NaN/Inf or norm blow-up detected          */

#define VK_PREC_FP64 0      /* plain FP64 everywhere                       */
#define VK_PREC_FP32 1      /* FP32 bulk, FP64 twiddles and reductions     */

/* Solver parameters.  Field names follow the Fortran module globals
 * (src/mod_grid.f90, src/mod_2dHD.f90, src/mod_gpparticles.f90) holding the
 * values AFTER set_grid (src/mod_grid.f90:63-101) and the derived-physics
 * block (src/driver.f90:360-396).  vk_params_derive() computes them from
 * the raw namelist values. */
typedef struct vk_params {
  int32_t nx, ny;            /* &resolution Nx, Ny (powers of two, 16..4096) */
  int32_t precision;         /* VK_PREC_FP64 or VK_PREC_FP32                 */
  int32_t otoc;              /* -DGPOTOC: ic_OTOC_gpe after vk_set_psi        */
  double dt;                 /* dt (= dt_fix)                                */
  double alpha;              /* alpha = csound*xi*sqrt(rho_avg/2)            */
  double gstrength;          /* g = csound^2/(2 alpha)                       */
  double omega_chem;         /* Omega (= g without SGLE)                     */
  double disp_factor;        /* &gpparam disp_factor                         */
  double xi;                 /* xi after xi*dx                               */
  double k_otoc_gp;          /* &gpotoc k_otoc_gp                            */
  double eps_otoc_gp;        /* &gpotoc eps_otoc_gp                          */
  int32_t n_particles;       /* &gpparticle gp_N_obj (0 = -DGPPART off)      */
  int32_t argle_renorm;      /* ARGLE renormalisation to Nparticle (new)     */
  double ppot_v0;            /* ppotV0 after *gstrength                      */
  double ppot_d;             /* ppotd  after *xi                             */
  double gp_mass_part;       /* &gpparticle gp_mass_part                     */
  int32_t reserved[8];
} vk_params;

/* Compile-time branches of the reference, selected at run time
 * (vk_set_variant).  Only the ones listed as built are accepted. */
#define VK_VAR_FRCDISP 1     /* -DGPE_FRCDISP: gpe_rhs hypo/hyperviscosity and
                                random-phase shell forcing (src/gpe.f90:623-658) */
#define VK_VAR_ADVECTION 2   /* -DGPE_ADVECTION: ARGLE Taylor-Green advection
                                (src/gpe.f90:78-81, 93-96, 115-131)         */
#define VK_VAR_COUNTERFLOW 4 /* -DGPE_COUNTERFLOW: ARGLE constant counterflow
                                (src/gpe.f90:78-81, 93-96, 135-145)         */
#define VK_VAR_SGLE 8        /* -DGPE_SGLE: ARGLE noise and chemical-potential
                                ODE (src/gpe.f90:149-178, 199-219, 226-274)  */
#define VK_VAR_SELFTRUNC 16  /* -DGPE_SELFTRUNC with SGLE: kpsi = 0 for
                                k^2 > ktrunc^2 (src/gpe.f90:213-217)        */
typedef struct vk_variant {
  int32_t flags;                      /* VK_VAR_* bits                      */
  int32_t pad;
  double vishypo_gp, vishype_gp;      /* &gphypvis (src/driver.f90:68)       */
  double famp_gp, kf1_gp, kf2_gp;     /* &gpforceparam, kf after *kdx
                                         (src/driver.f90:67, :384-387)       */
  double vnx, vny;                    /* &gpcounterflow (src/driver.f90:61)  */
  double oneybeta, nuN, chempot0;     /* &gpfiniteT (src/driver.f90:59)      */
  double ktrunc;                      /* &selftruncation (src/driver.f90:64) */
  uint64_t seed;                      /* counter-based stream of the forcing
                                         phases (stands in for RANDOM_NUMBER) */
  int32_t reserved[8];
} vk_variant;

/* Raw namelist values (src/driver.f90:52-79) -> vk_params, restating
 * set_grid (src/mod_grid.f90:63-101) and src/driver.f90:360-396. */
typedef struct vk_namelist {
  int32_t nx, ny;
  double dt_fix;
  double xi, csound, rho_avg, disp_factor;   /* &gpparam */
  double k_otoc_gp, eps_otoc_gp;            /* &gpotoc  */
  int32_t gp_n_obj;                         /* &gpparticle */
  double gp_mass_part, ppotd, ppotv0, ppotthick;
  int32_t maxiter, fsteps, ssteps, gsteps;  /* &tparam */
  int32_t nrst, sprst;                      /* &ckprst */
  int32_t strst, ststeps;                   /* &ckprst strst, &tparam ststeps (-DGPSTS) */
  /* branches selected by vk_set_variant (src/driver.f90:59-68) */
  double famp_gp, kf1_gp, kf2_gp;           /* &gpforceparam   */
  double vishypo_gp, vishype_gp;            /* &gphypvis       */
  double vnx, vny;                          /* &gpcounterflow  */
  double oneybeta, nun, chempot0;           /* &gpfiniteT      */
  double ktrunc;                            /* &selftruncation */
  int32_t nsplit_orignal, nsplit_current;   /* &fileparam (split restart files) */
} vk_namelist;

/* Replaces: the namelist reads + MPI_BCAST block (src/driver.f90:147-334).
 * Parses parameter.txt and parameter_gpe.txt (either path may be NULL). */
int vk_read_namelists(const char* parameter_txt, const char* parameter_gpe_txt, vk_namelist* out);
/* Replaces: set_grid + derived GPE parameters (src/mod_grid.f90:63-101,
 * src/driver.f90:360-396). */
int vk_params_derive(const vk_namelist* nl, int32_t precision, int32_t otoc, vk_params* out);
/* nshell = int(1.414*Nx/2.0d0)+1 (src/mod_grid.f90:77). */
int32_t vk_nshell(int32_t nx);

/* Replaces: mpi_localsize_estimate + create_state_variables +
 * create_global_array + initialize_fft + global_array
 * (src/mod_fft.f90:122-428, src/mod_2dHD.f90:62-76, src/pspectral.f90:1-35).
 * Allocates the device state on the current CUDA device. */
int vk_init(const vk_params* p, void** ctx);
/* Replaces: clear_fft + free_state_variables + dealloc_global_array
 * (src/mod_fft.f90:201-228,433-465, src/mod_2dHD.f90:78-92). */
int vk_finalize(void* ctx);

/* Replaces: restart_from_argle_data(0) + ic_OTOC_gpe
 * (src/initial_config.f90:630-771, :295-368): psi <- psi_phys,
 * kpsi <- F[psi]; with p->otoc the kpsi modes outside the 2/3 disk are
 * zeroed and psi <- F^-1[kpsi]. */
int vk_set_psi(void* ctx, const double* psi_phys);
/* Sets kpsi directly (transposed Fourier layout); psi <- F^-1[kpsi]. */
int vk_set_kpsi(void* ctx, const double* kpsi);
/* Copies back psi (physical) / kpsi (transposed Fourier). */
int vk_get_psi(void* ctx, double* psi_phys);
int vk_get_kpsi(void* ctx, double* kpsi);

/* Replaces: gpe_rk4 (src/gpe.f90:310-494) with gpe_rhs (:498-671) and, with
 * particles, gp_particle_motion_rk4 (src/gpe_particle.f90:429-531);
 * nsteps consecutive steps.  psi is current on return. */
int vk_gpe_rk4(void* ctx, int32_t nsteps);
/* Replaces: ARGLE(time) (src/gpe.f90:5-224), nsteps consecutive steps.
 * As in the reference, psi on return is the field at the START of the last
 * step.  residual_out (may be NULL) receives the new convergence measure
 * ||kpsi_new-kpsi_old||_2 / (dt ||kpsi_old||_2) of the last step. */
int vk_argle(void* ctx, int32_t nsteps, double* residual_out);

/* Replaces: diagnostics_gpe (src/diagnostics.f90:4-571) reductions.
 * scalars[10] = momx, momy, egrad, echem, eintr, etot, norm, eppot,
 *               eobj_kin, esrep (reference scalings, :105-239).
 * spec[(nshell+1)*6] in Fortran order spec_gp(0:nshell,1:6) (:394-399).
 * nvort[2] (may be NULL) = (# of +1, # of -1) plaquette windings (new). */
int vk_diagnostics(void* ctx, double* scalars, double* spec, int32_t* nvort);

/* Particle state, Fortran (1:2,1:P) order: [p][d] (src/mod_gpparticles.f90:24-30).
 * vk_particles_set also runs particle_potential (src/gpe_particle.f90:3-90). */
int vk_particles_set(void* ctx, const double* pos, const double* vel, const double* f0ext);
/* frc = gp_frc_obj as diagnostics_gpe leaves it (src/diagnostics.f90:528-533). */
int vk_particles_get(void* ctx, double* pos, double* vel, double* frc);

/* The context's CUDA stream (cudaStream_t), for callers that time or order
 * work against it. */
int vk_get_stream(void* ctx, void** stream);
/* Number of kernels this context has launched so far. */
int vk_kernel_launches(void* ctx, int64_t* count);

/* New (no reference counterpart): the vk_ic_vortices state computed on the
 * GPU in FP64 (for large grids), then loaded as by vk_set_psi.  pos_out
 * [2*n_vort] may be NULL. */
int vk_set_psi_vortices(void* ctx, int32_t n_vort, uint64_t seed, double xi0, double min_sep, double* pos_out);

/* Ensembles (new, no reference counterpart): n
 * independent fields of uneven sizes (nx, ny in {128, 256, 512, 1024}, one
 * precision, no particles) stepped together.  Each RK4 pass is one
 * persistent kernel over all members' row tiles; tile heights and grid sizes
 * come from an autotuner run at vk_ens_init (vk_ens_report describes it);
 * steps after the first replay one CUDA graph. */
int vk_ens_init(const vk_params* members, int32_t n, void** ens);
int vk_ens_finalize(void* ens);
int vk_ens_set_psi(void* ens, int32_t member, const double* psi_phys);
int vk_ens_get_psi(void* ens, int32_t member, double* psi_phys);
int vk_ens_gpe_rk4(void* ens, int32_t nsteps);
int vk_ens_report(void* ens, char* buf, int32_t cap);
int vk_ens_get_stream(void* ens, void** stream);
int vk_ens_kernel_launches(void* ens, int64_t* count);

/* Learned ARGLE warm-start network (new, no reference counterpart).  A
 * periodic conv encoder-decoder (levels, channels base*2^l, 3x3 convs) on
 * h x w grids with BF16 weights/activations and FP32 accumulation; every
 * convolution (forward, data and weight gradient) runs on tcgen05 tensor
 * cores.  Tensors passed in are DEVICE FP32 planar arrays: input [3][h][w]
 * (Re/Im of the phase ansatz, signed vortex-charge density), output and
 * target [2][h][w] (Re/Im correction).  Parameters are one FP32 vector,
 * per conv W[cout][9][cin] then b[cout]. */
int vk_nn_create(int32_t h, int32_t w, int32_t base, int32_t levels, uint64_t seed, void** net);
int vk_nn_destroy(void* net);
int vk_nn_num_params(void* net, int64_t* n);
int vk_nn_get_params(void* net, float* host, int64_t n);
int vk_nn_set_params(void* net, const float* host, int64_t n);
int vk_nn_forward(void* net, const float* in_dev, float* out_dev, void* stream);
int vk_nn_loss_grad(void* net, const float* in_dev, const float* target_dev, double* loss_out, float* grad_host);
int vk_nn_train_step(void* net, const float* in_dev, const float* target_dev, float lr, double* loss_out);
/* Batched training and inference (new).  vk_nn_create_batched sizes the
 * activations for up to batch_cap images (1..64); vk_nn_set_batch(net, b),
 * b <= batch_cap, makes vk_nn_forward, vk_nn_loss_grad and vk_nn_train_step
 * take b images: inputs [b][3][h][w], outputs and targets [b][2][h][w]; the
 * loss is the mean over the b images (one Adam step per batch).
 * vk_nn_create is vk_nn_create_batched with batch_cap 1. */
int vk_nn_create_batched(int32_t h, int32_t w, int32_t base, int32_t levels, int32_t batch_cap, uint64_t seed,
                         void** net);
int vk_nn_set_batch(void* net, int32_t batch);
/* Input features of one image on the device (new): out_dev [3][h][w] FP32
 * = Re psi, Im psi and the signed vortex-charge density
 * sum_j q_j exp(-|x - x_j|^2 / (2 width^2)) (periodic distance; q_j = +1 for
 * the first n_vort/2 vortices, -1 for the rest).  psi_host [h][w] complex128
 * (x fastest), pos_host [n_vort][2] (x, y), n_vort <= 4096. */
int vk_nn_features(void* net, const double* psi_host, const double* pos_host, int32_t n_vort, double width,
                   float* out_dev);

/* Per-kernel timing.  Between vk_timing_begin and vk_timing_end every kernel
 * this context launches is bracketed by CUDA events on the context's stream;
 * vk_timing_end synchronises and returns, per kernel tag (NUL-terminated,
 * 24 bytes each), the summed elapsed milliseconds and the launch count.
 * Timing adds one event record per launch; time production runs without it. */
int vk_timing_begin(void* ctx);
int vk_timing_end(void* ctx, int32_t cap, char* tags, double* total_ms, int64_t* counts, int32_t* ntags);

/* Forward 2D FFT that allocates no device memory.  No counterpart in the
 * reference.  For callers that must not call cudaMalloc, such as a Fortran
 * code whose device arrays belong to an OpenACC / OpenMP-offload runtime, or
 * an application with its own device pool.  psi_dev [ny][nx] and kpsi_dev
 * [nx][ny] are DEVICE pointers to complex128 arrays owned by the caller;
 * kpsi = unnormalised F[psi] in the transposed layout (what vk_set_psi puts in
 * kpsi).  The transposed intermediate lives in a built-in device array of
 * 262144 complex points (4 MiB, nx*ny must fit; nx, ny powers of two in
 * [16, 4096]), held by every GPU that loads the library until exit.  The
 * first call on a device resolves that array's address and fills the
 * twiddle tables, so make it before any stream capture.  Calls share the
 * array: calls that overlap on the GPU race.  Work is queued on `stream`
 * (a cudaStream_t; NULL = legacy default stream) and is not synchronised. */
int vk_fft2d_forward_noalloc(const double* psi_dev, double* kpsi_dev, int32_t nx, int32_t ny, void* stream);

/* Selects the compile-time branches of v->flags for this context (0 = the
 * plain equations).  With VK_VAR_FRCDISP every RK4 right-hand side
 * (gpe_rhs, src/gpe.f90:609-669) becomes
 *   prefac((alpha k^2 - Omega) kpsi + N^) - vishypo k^-16 kpsi (k != 0)
 *   - vishype k^16 kpsi + famp exp(i 2 pi u)   (kf1^2 <= k^2 <= kf2^2),
 * then the 2/3 mask; u is uniform [0,1) from (seed, RHS evaluation count,
 * mode kx*ny + ky) -- the reference draws RANDOM_NUMBER per mode and RHS.
 * With VK_VAR_ADVECTION or VK_VAR_COUNTERFLOW (one of them) every ARGLE step
 * adds to N = -g P_G rho psi, with grad psi = F^-1[i k kpsi]:
 *   advection   -i u.grad psi - (1/4)(1/alpha)|u|^2 psi,
 *               u = (sin x cos y, -cos x sin y);
 *   counterflow -i (vnx, vny).grad psi.
 * The flow terms need nx <= 2048 (FP64) and no particles.
 * With VK_VAR_SGLE the chemical potential starts at chempot0 and before
 * every ARGLE update becomes omega - dt nuN/(Lx Ly) (norm - Lx Ly)
 * (finiteT_adhoc_chempot, src/gpe.f90:226-264), and the update adds
 * sqrt(dt) F[noise] (2/3 mask), noise = (v1 + i v2) sqrt(oneybeta/(2 alpha))
 * /sqrt(dvol) with standard normals v1, v2 per point from the same
 * counter-based stream (the reference: the polar method on RANDOM_NUMBER,
 * so parity with it is statistical).  VK_VAR_SELFTRUNC then zeroes
 * k^2 > ktrunc^2.  Unbuilt flags return VK_E_INVALID. */
int vk_set_variant(void* ctx, const vk_variant* v);
/* vk_variant from the raw namelist values for the VK_VAR_* flags: kf1, kf2
 * times kdx (src/driver.f90:384-387), the rest as read. */
int vk_variant_derive(const vk_namelist* nl, int32_t flags, uint64_t seed, vk_variant* out);
/* Current chemical potential omega_chem (changes under VK_VAR_SGLE;
 * write_chempot_for_restart, src/gpe.f90:266-300, writes it). */
int vk_get_chempot(void* ctx, double* omega);

/* ---- spatio-temporal spectra (the -DGPSTS path) ----
 * Replaces: sts_gpe (src/diagnostics.f90:636-695), called every ststeps
 * (src/solve.f90:139-144), which appends kpsi(:,kx=0) and the kpsi plane to
 * files, and the offline post-processor Run/CompSTS/driver.f90:132-265,
 * which Hann-windows each mode's time series (w = (1-cos(2 pi t/(Nt-1)))/2),
 * transforms it along time (FFTW forward), and forms
 *   sts1d[w][ky]   = stsnorm |X(kx=0, ky, w)|^2
 *   sts2d[w][m]    = sum over nint(|k|) = m of stsnorm |X(k, w)|^2, m = 0..nx/3
 * with stsnorm = (1/Nt)^2 (1/(nx ny))^2.  Here the planes stay on the GPU in
 * a ring of nt records (nt * nx * ny * 16 bytes) and the transform and the
 * shell sums run there. */
/* Allocates the ring for nt records (nt a power of two, 16..4096). */
int vk_sts_begin(void* ctx, int32_t nt);
/* Appends the current kpsi (as FP64) to the ring; VK_E_STATE when full. */
int vk_sts_record(void* ctx);
/* Number of records held. */
int vk_sts_count(void* ctx, int32_t* n);
/* With the ring full: sts1d[nt*ny] (row w = 0..nt-1), sts2d[nt*(nx/3+1)].
 * Consumes the records (the ring is empty afterwards). */
int vk_sts_spectra(void* ctx, double* sts1d, double* sts2d);
/* Frees the ring. */
int vk_sts_end(void* ctx);

/* Asynchronous field dump (the io_fields writes of src/io_fields.f90:1-66
 * without stalling the stepping).  vk_dump_begin snapshots psi (as FP64)
 * in step order and starts its copy to pinned host memory on a second
 * stream, then returns; later vk_gpe_rk4 / vk_argle calls proceed meanwhile.
 * vk_dump_wait blocks until that copy is done and copies psi_phys[ny*nx]
 * out; it touches only the dump's event and buffer, so another host thread
 * may call it while this context steps.  One dump in flight at a time. */
int vk_dump_begin(void* ctx);
int vk_dump_wait(void* ctx, double* psi_phys);

/* Thread-local message for the last failing call on this thread. */
const char* vk_last_error(void);

/* ---- host-side I/O in the reference's file formats (no GPU needed) ---- */

/* io_fields (src/io_fields.f90:1-66, -DIOEVERYPROC, one rank): Fortran
 * sequential-unformatted file: record (int32 iopoint, real64 time, real64 dt),
 * then ny records of nx complex128 (x fastest). */
int vk_write_wf(const char* path, int32_t iopoint, double time, double dt,
                int32_t nx, int32_t ny, const double* psi_phys);
/* Reads the same layout (restart_from_argle_data, src/initial_config.f90:727-741). */
int vk_read_wf(const char* path, int32_t nx, int32_t ny, int32_t* iopoint,
               double* time, double* dt, double* psi_phys);

/* Regrouping of a field written as nsplit files (src/io_fields.f90:121-146,
 * -DIOEVERYPROC, nsplit_orignal > nsplit_current = 1): reads
 * <prefix>p1.dat .. <prefix>p<nsplit>.dat, each a header and ny/nsplit rows,
 * into psi_phys[ny*nx] in file order.  prefix e.g. "restart/wf/wf0". */
int vk_read_wf_split(const char* prefix, int32_t nsplit, int32_t nx, int32_t ny, int32_t* iopoint,
                     double* time, double* dt, double* psi_phys);

/* New (no reference counterpart): seeded N-vortex initial state.
 * Positions from SplitMix64(seed), uniform on [0,2pi)^2 with periodic
 * minimum separation min_sep; charges +1 for the first n_vort/2, -1 after.
 * psi = prod_j A(r_j) * exp(i theta), A(r) = (r/xi0)/sqrt(2+(r/xi0)^2),
 * theta the doubly periodic phase of the neutral set.  pos_out[2*n_vort]
 * (may be NULL) receives the positions. */
int vk_ic_vortices(int32_t nx, int32_t ny, int32_t n_vort, uint64_t seed,
                   double xi0, double min_sep, double* psi_phys, double* pos_out);

#ifdef __cplusplus
}
#endif
#endif /* VK_H */
