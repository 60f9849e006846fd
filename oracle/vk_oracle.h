/*
 * vk_oracle.h -- CPU FP64 restatement of the VIKSHOBHA 2D GPE hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA path:
 * only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
 * load it.  The product library (libvk) never links or calls it.
 *
 * PARITY UNPINNED: the reference is Fortran 90 + FFTW 3.3.8 + MPI, none of
 * which exist on these machines, and the reference ships no tests, golden
 * vectors or fixtures.  The restatement is pinned instead by derived
 * known answers (plane-wave RK4 amplification factor, stationary uniform
 * state, linear dispersion, symmetric particle forces) and by an
 * independent numpy restatement in tests/.
 *
 * Layouts follow the reference exactly:
 *   physical  psi(i1=x, i2=y)  -> C index  y*nx + x      (x fastest)
 *   Fourier   kpsi(i2=ky,i1=kx)-> C index  kx*ny + ky    (ky fastest,
 *             i.e. the FFTW_MPI_TRANSPOSED_OUT layout, src/mod_fft.f90:143-146)
 * Complex values are interleaved (re, im) doubles.
 */
#ifndef VK_ORACLE_H
#define VK_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef struct vko_state vko_state;

/* Grid + physics (already-derived values, as the Fortran module globals hold
 * them after src/driver.f90:360-396 and src/mod_grid.f90:63-101). */
typedef struct vko_params {
  int32_t nx, ny;
  int32_t n_particles;      /* gp_N_obj (0 = no particles, i.e. -DGPPART off) */
  int32_t renorm;           /* ARGLE renormalisation (new; not in the reference) */
  double dt, alpha, gstrength, omega_chem, disp_factor;
  double xi;                /* xi after xi*dx (driver.f90:363) */
  double ppot_v0, ppot_d;   /* after V0*g and d*xi (driver.f90:391-392) */
  double gp_mass_part;
} vko_params;

vko_state* vko_create(const vko_params* p);
void vko_destroy(vko_state* s);

/* Derived grid constants (mod_grid.f90:63-101). */
int32_t vko_nshell(int32_t nx);
double vko_kalias(int32_t nx);
int32_t vko_kwn(int32_t n, int32_t i1based);

/* Unnormalised FFTs in the reference layouts (mod_fft.f90:471-542):
 * forward psi[y][x] -> four[kx][ky]; inverse four -> phys then * 1/(nx*ny). */
void vko_fft_forward(vko_state* s, const double* phys, double* four);
void vko_fft_inverse(vko_state* s, const double* four, double* phys);

/* restart_from_argle_data (initial_config.f90:630-771): psi <- field,
 * kpsi <- F[psi]; then ic_OTOC_gpe (initial_config.f90:295-368) if otoc. */
void vko_set_psi(vko_state* s, const double* psi_phys, int32_t otoc, double k_otoc, double eps_otoc);
void vko_get_psi(const vko_state* s, double* out);
void vko_get_kpsi(const vko_state* s, double* out);
void vko_set_kpsi(vko_state* s, const double* kpsi);

/* gpe_rk4 (gpe.f90:310-494) nsteps times. */
void vko_gpe_rk4(vko_state* s, int32_t nsteps);
/* ARGLE (gpe.f90:5-224) nsteps times; residual of the last step
 * ||kpsi_new-kpsi_old||_2 / (dt*||kpsi_old||_2) written to *residual. */
void vko_argle(vko_state* s, int32_t nsteps, double* residual);

/* diagnostics_gpe (diagnostics.f90:4-571).
 * scalars[0..9] = momx, momy, egrad, echem, eintr, etot, norm, eppot,
 *                 eobj_kin, esrep
 * spec[(nshell+1)*6] in Fortran order spec(0:nshell,1:6). */
void vko_diagnostics(vko_state* s, double* scalars, double* spec);

/* Particles (gpe_particle.f90).  Arrays are Fortran (1:2,1:P): [p][d]. */
void vko_particles_set(vko_state* s, const double* pos, const double* vel, const double* f0ext);
void vko_particles_get(const vko_state* s, double* pos, double* vel, double* frc);
/* Force on every particle at the current state (translate_particle_potential(i)
 * for i=1..P, diagnostics.f90:528-533); frc[p][d]. */
void vko_particle_forces(vko_state* s, double* frc);
/* -DGPE_FRCDISP (gpe.f90:623-658): hypo/hyperviscosity and random-phase
 * forcing in the shell kf1^2 <= k^2 <= kf2^2 (phases from frc_uniform). */
void vko_set_frcdisp(vko_state* s, int32_t on, double vishypo, double vishype, double famp, double kf1,
                     double kf2, uint64_t seed);
/* ARGLE flow terms (gpe.f90:78-146): mode 1 = -DGPE_ADVECTION (Taylor-Green
 * u = (sin x cos y, -cos x sin y)), 2 = -DGPE_COUNTERFLOW (u = (vnx, vny)). */
void vko_set_argle_flow(vko_state* s, int32_t mode, double vnx, double vny);
/* -DGPE_SGLE (gpe.f90:149-178, 199-219, 226-274): noise of amplitude
 * noisesigma/sqrt(dvol), noisesigma = sqrt(oneybeta/(2 alpha)), and the
 * chemical potential ODE from chempot0; -DGPE_SELFTRUNC zeroes k^2 > ktrunc^2. */
void vko_set_sgle(vko_state* s, int32_t on, double oneybeta, double nuN, double chempot0, int32_t selftrunc,
                  double ktrunc, uint64_t seed);
double vko_chempot(const vko_state* s);

/* Signed plaquette winding count on the physical grid (new component). */
void vko_count_vortices(const vko_state* s, int32_t* n_plus, int32_t* n_minus);

void vko_set_threads(int32_t n);

/* Seeded neutral vortex state (new component, no reference counterpart):
 * positions from SplitMix64(seed), uniform on [0,2pi)^2 with a periodic
 * minimum separation, charges +1 for the first half and -1 for the rest;
 * amplitude prod_j (r_j/xi0)/sqrt(2 + (r_j/xi0)^2), phase from the odd Jacobi
 * theta function (nome e^{-pi}) with the linear term that makes it periodic.
 * psi[ny*nx] interleaved complex, pos[2*n_vort].  Returns 0, or -1 when the
 * arguments are invalid or the vortices cannot be placed. */
int32_t vko_ic_vortices(int32_t nx, int32_t ny, int32_t n_vort, uint64_t seed, double xi0, double min_sep,
                        double* psi, double* pos);

#ifdef __cplusplus
}
#endif
#endif
