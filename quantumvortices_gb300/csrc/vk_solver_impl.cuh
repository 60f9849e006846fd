// vk_solver_impl.cuh -- Solver<T>: device state and launch sequences.
//
// Included by vk_solver_tu.cu, which is compiled once per (precision, row-length
// class).  Each compilation defines VK_LEN_MASK (bit i set: row length 16 << i
// is instantiated) and VK_SOLVER_NS, a distinct inline namespace that keeps
// every compilation's Solver, with_len and host helpers apart at link time.
// The kernels each one instantiates are those of its own lengths, so the
// classes compile in parallel.
#pragma once
#ifndef VK_LEN_MASK
#define VK_LEN_MASK 511
#endif
#ifndef VK_SOLVER_NS
#error "VK_SOLVER_NS must name this compilation's inline namespace"
#endif
#include <cuda_runtime.h>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <type_traits>
#include <unordered_set>
#include <vector>
#include "vk_kernels.cuh"
#include "vk_particles.cuh"
#include "vk_diag.cuh"
#include "vk_stage.cuh"
#include "vk_solver.h"

namespace vk {
inline namespace VK_SOLVER_NS {

#define VK_CUDA_TRY(expr)                                                              \
  do {                                                                                 \
    cudaError_t e_ = (expr);                                                           \
    if (e_ != cudaSuccess) {                                                           \
      set_error(std::string(#expr) + ": " + cudaGetErrorString(e_));                   \
      return VK_E_CUDA;                                                                \
    }                                                                                  \
  } while (0)

template <int L> using LC = std::integral_constant<int, L>;

// Calls f(LC<n>()) for a row length n of this compilation's class.
template <typename F> bool with_len(int n, F&& f) {
  switch (n) {
    case 16: if constexpr ((VK_LEN_MASK >> 0) & 1) { f(LC<16>()); return true; } else { return false; }
    case 32: if constexpr ((VK_LEN_MASK >> 1) & 1) { f(LC<32>()); return true; } else { return false; }
    case 64: if constexpr ((VK_LEN_MASK >> 2) & 1) { f(LC<64>()); return true; } else { return false; }
    case 128: if constexpr ((VK_LEN_MASK >> 3) & 1) { f(LC<128>()); return true; } else { return false; }
    case 256: if constexpr ((VK_LEN_MASK >> 4) & 1) { f(LC<256>()); return true; } else { return false; }
    case 512: if constexpr ((VK_LEN_MASK >> 5) & 1) { f(LC<512>()); return true; } else { return false; }
    case 1024: if constexpr ((VK_LEN_MASK >> 6) & 1) { f(LC<1024>()); return true; } else { return false; }
    case 2048: if constexpr ((VK_LEN_MASK >> 7) & 1) { f(LC<2048>()); return true; } else { return false; }
    case 4096: if constexpr ((VK_LEN_MASK >> 8) & 1) { f(LC<4096>()); return true; } else { return false; }
    default: return false;
  }
}

template <typename T> __global__ void k_from_f64(const double2* __restrict__ in, cplx<T>* __restrict__ out, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    out[i] = mkc<T>(T(in[i].x), T(in[i].y));
}
template <typename T> __global__ void k_to_f64(const cplx<T>* __restrict__ in, double2* __restrict__ out, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    out[i] = make_double2((double)in[i].x, (double)in[i].y);
}
// One more right-hand side evaluated: advance the forcing-phase counter
// (templated so each precision's translation unit has its own symbol).
template <typename T> __global__ void k_rng_bump(unsigned long long* c) { *c += 1ull; }

template <typename T> __global__ void k_scale_two(cplx<T>* __restrict__ a, cplx<T>* __restrict__ b, size_t n,
                                                  const double* __restrict__ sums, double factor_num) {
  // renormalisation: s = sqrt(Nparticle / norm), norm = factor * sum|kpsi|^2
  const double s = sqrt(factor_num / sums[2]);
  const T st = T(s);
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    a[i] = cscale(a[i], st);
    b[i] = cscale(b[i], st);
  }
}

// vhat[kx][ky] = mask * full[kx][ky] for kx in [0, K] (particle_potential's
// dealiased V^, src/gpe_particle.f90:67-88; V is real, so this half suffices).
template <typename T>
__global__ void k_extract_half(const cplx<T>* __restrict__ full, cplx<T>* __restrict__ half, int K, int nx, int ny,
                               int k2max) {
  const size_t n = (size_t)(K + 1) * ny;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int kx = (int)(i / ny), ky = (int)(i % ny);
    const int k2 = kwn(ky, ny);
    half[i] = (kx * kx + k2 * k2 > k2max) ? mkc<T>(T(0), T(0)) : full[(size_t)kx * ny + ky];
  }
}

enum TaState { TA_INVALID = 0, TA_PRUNED = 1, TA_FULL = 2 };

template <typename T>
class Solver : public SolverBase {
  typedef cplx<T> C;

 public:
  explicit Solver(const vk_params& p) : p_(p) {}
  ~Solver() override { release(); }

  int init() {
    nx_ = p_.nx;
    ny_ = p_.ny;
    n2_ = (size_t)nx_ * ny_;
    k2max_ = k2max_for(nx_);
    K_ = kmax_for(k2max_);
    if (K_ >= nx_ / 2) {
      set_error("grid too small for the 2/3 rule");
      return VK_E_INVALID;
    }
    pk_ = (K_ + 2) & ~1;
    nshell_ = vk_nshell(nx_);
    VK_CUDA_TRY(cudaStreamCreateWithFlags(&st_, cudaStreamNonBlocking));
    const size_t fb = n2_ * sizeof(C);
    VK_CUDA_TRY(cudaMalloc(&psi_, fb));
    VK_CUDA_TRY(cudaMalloc(&kpsi_, fb));
    VK_CUDA_TRY(cudaMalloc(&str1_, fb));
    VK_CUDA_TRY(cudaMalloc(&str2_, fb));
    VK_CUDA_TRY(cudaMalloc(&Ta_, fb));
    VK_CUDA_TRY(cudaMalloc(&Td_, fb));
    VK_CUDA_TRY(cudaMalloc(&Tb_, sizeof(C) * (size_t)(K_ + 1) * ny_));
    VK_CUDA_TRY(cudaMalloc(&Tc_, sizeof(C) * (size_t)ny_ * pk_));
    VK_CUDA_TRY(cudaMalloc(&stage64_, n2_ * sizeof(double2)));
    VK_CUDA_TRY(cudaMemsetAsync(psi_, 0, fb, st_));
    VK_CUDA_TRY(cudaMemsetAsync(kpsi_, 0, fb, st_));
    VK_CUDA_TRY(cudaMemsetAsync(str1_, 0, fb, st_));
    VK_CUDA_TRY(cudaMemsetAsync(str2_, 0, fb, st_));
    VK_CUDA_TRY(cudaMemsetAsync(Ta_, 0, fb, st_));
    VK_CUDA_TRY(cudaMemsetAsync(Td_, 0, fb, st_));
    VK_CUDA_TRY(cudaMemsetAsync(Tb_, 0, sizeof(C) * (size_t)(K_ + 1) * ny_, st_));
    VK_CUDA_TRY(cudaMemsetAsync(Tc_, 0, sizeof(C) * (size_t)ny_ * pk_, st_));
    const int maxblk = std::max(nx_, ny_);
    VK_CUDA_TRY(cudaMalloc(&part_, sizeof(double) * 3 * (size_t)maxblk));
    VK_CUDA_TRY(cudaMalloc(&sums_, sizeof(double) * 8));
    VK_CUDA_TRY(cudaMalloc(&rngc_, sizeof(unsigned long long)));
    VK_CUDA_TRY(cudaMemset(rngc_, 0, sizeof(unsigned long long)));
    c_.frc = 0;
    c_.rng_ctr = rngc_;
    // twiddle tables
    int trc = upload_twiddles(nx_, &twx_);
    if (trc) return trc;
    if (ny_ == nx_) twy_ = twx_;
    else if ((trc = upload_twiddles(ny_, &twy_))) return trc;
    c_.nx = nx_;
    c_.ny = ny_;
    c_.K = K_;
    c_.k2max = k2max_;
    c_.pk = pk_;
    c_.alpha = p_.alpha;
    c_.g = p_.gstrength;
    c_.omega = p_.omega_chem;
    c_.dt = p_.dt;
    // prefacrhs = (one - zi*disp_factor)/zi = (-disp_factor, -1)  (src/gpe.f90:529)
    c_.prefac_re = -p_.disp_factor;
    c_.prefac_im = -1.0;
    c_.scale = 1.0 / ((double)nx_ * (double)ny_);
    c_.rho_bg = std::is_same<T, double>::value ? 0.0 : (p_.gstrength != 0.0 ? p_.omega_chem / p_.gstrength : 0.0);
    // FP64 x passes at nx = 1024 run one row per CTA.  The pass is bound by
    // the FP64 pipe of the busiest SM: 512 row-pair CTAs leave 4 pairs on
    // some SMs and 3 on others (135 us for k_x1 on GB300), while 1024
    // single-row CTAs, 608 resident and the rest taking the SMs that free
    // first, even the rows out (119 us).  At 4096^2 the row pairs stay
    // ahead (6.12e8 against 6.04e8 grid-pt-steps/s).  VK_XSPLIT=0 keeps the
    // row pairs at 1024 too.
    c_.xsingle = 0;
    const char* xs_env = std::getenv("VK_XSPLIT");
    if (std::is_same<T, double>::value && nx_ == 1024 && !(xs_env && xs_env[0] == '0')) c_.xsingle = ny_;
    // VK_XSPLIT=1: single rows in every x pass with nx >= 128 (timing comparisons)
    if (xs_env && xs_env[0] == '1' && nx_ >= 128) c_.xsingle = ny_;
    // FP64: the y passes (y1, RK4 y2) and the single-row CTAs of k_x1 load
    // their rows by bulk copies (cp.async.bulk on an mbarrier, bounded
    // waits); VK_BULK=0 loads element-wise.
    bulk_ = false;
    if (std::is_same<T, double>::value) {
      const char* b = std::getenv("VK_BULK");
      bulk_ = !(b && b[0] == '0');
    }
    if (bulk_) {
      const char* lim = std::getenv("VK_SPIN_LIMIT");
      VK_CUDA_TRY(cudaMalloc(&async_err_, sizeof(int)));
      VK_CUDA_TRY(cudaMemset(async_err_, 0, sizeof(int)));
      c_.async_err = async_err_;
      c_.async_limit = lim ? std::strtoull(lim, nullptr, 10) : (1ull << 24);
    }
    {
      int frc = init_fused();
      if (frc) return frc;
    }
    if (p_.n_particles > 0) {
      int prc = init_particles();
      if (prc) return prc;
    }
    VK_CUDA_TRY(cudaStreamSynchronize(st_));
    return VK_OK;
  }

  int init_particles() {
    np_ = p_.n_particles;
    if (nx_ < 32 || ny_ < 32) {
      set_error("particles need nx, ny >= 32");
      return VK_E_INVALID;
    }
    if (!(p_.gp_mass_part > 0) || !(p_.ppot_d > 0)) {
      set_error("particles need gp_mass_part > 0 and ppotd > 0");
      return VK_E_INVALID;
    }
    const int rp = geo_rows_x(ny_) / 2;
    nblk_pot_ = (K_ + 1 + rp - 1) / rp;
    double* d[10];
    const size_t sz[10] = {2u * (size_t)np_, 2u * (size_t)np_, 2u * (size_t)np_, 2u * (size_t)np_, 8u * (size_t)np_,
                           8u * (size_t)np_, 2u * (size_t)np_, 2u * (size_t)np_,
                           2u * (size_t)np_ * (K_ + 1), 2u * (size_t)np_ * ny_};
    for (int i = 0; i < 10; ++i) VK_CUDA_TRY(cudaMalloc(&d[i], sizeof(double) * sz[i]));
    for (int i = 0; i < 10; ++i) VK_CUDA_TRY(cudaMemsetAsync(d[i], 0, sizeof(double) * sz[i], st_));
    ps_.pos = d[0]; ps_.vel = d[1]; ps_.tpos = d[2]; ps_.tvel = d[3]; ps_.ku = d[4]; ps_.kq = d[5];
    ps_.f0ext = d[6]; ps_.frc = d[7]; ps_.tab_x = d[8]; ps_.tab_y = d[9];
    VK_CUDA_TRY(cudaMalloc(&ps_.fpart, sizeof(double) * 2 * (size_t)np_ * nblk_pot_));
    VK_CUDA_TRY(cudaMalloc(&vhat_, sizeof(C) * (size_t)(K_ + 1) * ny_));
    VK_CUDA_TRY(cudaMemsetAsync(vhat_, 0, sizeof(C) * (size_t)(K_ + 1) * ny_, st_));
    VK_CUDA_TRY(cudaMalloc(&Tv_, sizeof(C) * (size_t)ny_ * pk_));
    VK_CUDA_TRY(cudaMalloc(&vpot_, sizeof(T) * n2_));
    const double two_pi = 6.283185307179586476925286766559, pi = two_pi / 2;
    pc_.np = np_;
    pc_.K = K_;
    pc_.nx = nx_;
    pc_.ny = ny_;
    pc_.nblk = nblk_pot_;
    pc_.dt = p_.dt;
    pc_.mass = p_.gp_mass_part;
    pc_.alpha = p_.alpha;
    pc_.dvol = (two_pi / nx_) * (two_pi / ny_);
    pc_.scale = c_.scale;
    // shortrange_repulsion constants (src/gpe_particle.f90:395-401): gpdeltaE is
    // assigned from a default-real literal, gpr0obj = 4.0*xi.
    const double dE = (double)0.062f, r0 = 4.0 * p_.xi;
    auto ip = [](double x, int n) { double r = 1.0; for (int i = 0; i < n; ++i) r *= x; return r; };
    pc_.rep_factor = 384.0 * dE * ip(pi, 12) * ip(r0, 12) / ip(two_pi, 12);
    erep_factor_ = 64.0 * dE * ip(pi, 12) * ip(r0, 12) / ip(two_pi, 12);
    return VK_OK;
  }

  void* stream() override { return (void*)st_; }
  int field_view(void* out, size_t size) override {
    if (size != sizeof(Field<T>)) {
      set_error("field_view: size mismatch");
      return VK_E_INVALID;
    }
    Field<T> f;
    f.psi = psi_; f.kpsi = kpsi_; f.str1 = str1_; f.str2 = str2_;
    f.Ta = Ta_; f.Tb = Tb_; f.Tc = Tc_; f.Td = Td_;
    f.twx = twx_; f.twy = twy_; f.c = c_;
    std::memcpy(out, &f, sizeof(f));
    return VK_OK;
  }
  int set_variant(const vk_variant* v) override {
    if (v->flags & ~(VK_VAR_FRCDISP | VK_VAR_ADVECTION | VK_VAR_COUNTERFLOW | VK_VAR_SGLE | VK_VAR_SELFTRUNC)) {
      set_error("vk_set_variant: unknown flag");
      return VK_E_INVALID;
    }
    if ((v->flags & VK_VAR_SELFTRUNC) && !(v->flags & VK_VAR_SGLE)) {
      set_error("vk_set_variant: VK_VAR_SELFTRUNC acts inside the SGLE branch only");
      return VK_E_INVALID;
    }
    const int flow = (v->flags & VK_VAR_ADVECTION) ? 1 : ((v->flags & VK_VAR_COUNTERFLOW) ? 2 : 0);
    if ((v->flags & VK_VAR_ADVECTION) && (v->flags & VK_VAR_COUNTERFLOW)) {
      set_error("vk_set_variant: advection and counterflow are exclusive");
      return VK_E_INVALID;
    }
    if (flow && (np_ > 0 || (sizeof(T) == 8 && nx_ > 2048))) {
      set_error("vk_set_variant: the ARGLE flow terms need no particles and nx <= 2048 in FP64");
      return VK_E_INVALID;
    }
    const double vals[] = {v->vishypo_gp, v->vishype_gp, v->famp_gp, v->kf1_gp, v->kf2_gp, v->vnx, v->vny,
                           v->oneybeta, v->nuN, v->chempot0, v->ktrunc};
    for (double x : vals)
      if (!std::isfinite(x)) {
        set_error("vk_set_variant: non-finite parameter");
        return VK_E_INVALID;
      }
    c_.frc = (v->flags & VK_VAR_FRCDISP) ? 1 : 0;
    c_.vishypo = v->vishypo_gp;
    c_.vishype = v->vishype_gp;
    c_.famp = v->famp_gp;
    c_.kf1sq = v->kf1_gp * v->kf1_gp;
    c_.kf2sq = v->kf2_gp * v->kf2_gp;
    c_.seed = v->seed;
    flow_ = flow;
    vnx_ = v->vnx;
    vny_ = v->vny;
    if (flow_ && !Tg_) VK_CUDA_TRY(cudaMalloc(&Tg_, n2_ * sizeof(C)));
    // SGLE (src/driver.f90:368-376): omega_chem = chempot0, noisesigma =
    // sqrt(oneybeta/(2 alpha)), applied with 1/sqrt(dvol) (src/gpe.f90:163)
    sgle_ = (v->flags & VK_VAR_SGLE) ? 1 : 0;
    const double two_pi = 6.283185307179586476925286766559;
    const double dvol = (two_pi / nx_) * (two_pi / ny_);
    c_.sgle_amp = (1.0 / std::sqrt(dvol)) * std::sqrt((1.0 / (2.0 * c_.alpha)) * v->oneybeta);
    c_.sqrt_dt = std::sqrt(c_.dt);
    c_.selftrunc = (v->flags & VK_VAR_SELFTRUNC) ? 1 : 0;
    c_.ktrunc2 = v->ktrunc * v->ktrunc;
    nun_area_ = v->nuN / (two_pi * two_pi);
    if (sgle_) {
      if (!Tn_) VK_CUDA_TRY(cudaMalloc(&Tn_, n2_ * sizeof(C)));
      if (!omega_dev_) VK_CUDA_TRY(cudaMalloc(&omega_dev_, sizeof(double) * (1 + kNormBlocks)));
      c_.omega = v->chempot0;
      VK_CUDA_TRY(cudaMemcpy(omega_dev_, &c_.omega, sizeof(double), cudaMemcpyHostToDevice));
    } else {
      c_.omega = p_.omega_chem;
    }
    c_.omega_dev = omega_dev_;
    // the captured step graphs bake the constants in: capture again
    if (g_rk4_) cudaGraphExecDestroy(g_rk4_);
    if (g_argle_) cudaGraphExecDestroy(g_argle_);
    g_rk4_ = g_argle_ = nullptr;
    VK_CUDA_TRY(cudaMemsetAsync(rngc_, 0, sizeof(unsigned long long), st_));
    return sync_check();
  }
  int dump_begin() override {
    if (!have_psi_) { set_error("vk_dump_begin: no psi set"); return VK_E_STATE; }
    if (dump_pending_) { set_error("vk_dump_begin: the previous dump was not waited for"); return VK_E_STATE; }
    if (!dump_dev_) {
      VK_CUDA_TRY(cudaMalloc(&dump_dev_, n2_ * sizeof(double2)));
      VK_CUDA_TRY(cudaMallocHost(&dump_host_, n2_ * sizeof(double2)));
      VK_CUDA_TRY(cudaStreamCreateWithFlags(&dump_st_, cudaStreamNonBlocking));
      VK_CUDA_TRY(cudaEventCreateWithFlags(&dump_snap_, cudaEventDisableTiming));
      VK_CUDA_TRY(cudaEventCreateWithFlags(&dump_done_, cudaEventDisableTiming));
    }
    // device snapshot in step order on the solver stream (FP64 for the file)
    if (std::is_same<T, double>::value)
      VK_CUDA_TRY(cudaMemcpyAsync(dump_dev_, psi_, n2_ * sizeof(double2), cudaMemcpyDeviceToDevice, st_));
    else
      launch_simple("k_to_f64", k_to_f64<T>, (const C*)psi_, dump_dev_, n2_);
    VK_CUDA_TRY(cudaEventRecord(dump_snap_, st_));
    // the copy to the host runs on its own stream while later steps proceed
    VK_CUDA_TRY(cudaStreamWaitEvent(dump_st_, dump_snap_, 0));
    VK_CUDA_TRY(cudaMemcpyAsync(dump_host_, dump_dev_, n2_ * sizeof(double2), cudaMemcpyDeviceToHost, dump_st_));
    VK_CUDA_TRY(cudaEventRecord(dump_done_, dump_st_));
    dump_pending_ = true;
    return check_launch();
  }
  int dump_wait(double* psi) override {
    if (!dump_pending_) { set_error("vk_dump_wait: no dump in flight"); return VK_E_STATE; }
    VK_CUDA_TRY(cudaEventSynchronize(dump_done_));
    std::memcpy(psi, dump_host_, n2_ * sizeof(double2));
    dump_pending_ = false;
    return VK_OK;
  }
  int get_chempot(double* omega) override {
    *omega = c_.omega;
    return VK_OK;
  }
  int snapshot_kpsi_f64(void* dst) override {
    launch_simple("k_to_f64", k_to_f64<T>, (const C*)kpsi_, (double2*)dst, n2_);
    return check_launch();
  }
  bool kpsi_is_masked() const override { return kpsi_masked_; }
  void mark_rk4_done() override {
    kpsi_masked_ = true;
    ta_ = TA_PRUNED;
  }
  int64_t launches() const override { return launches_; }

  // ---------------------------------------------------------------- I/O --
  int set_psi(const double* psi) override {
    int rc = upload(psi, psi_);
    if (rc) return rc;
    return set_psi_on_device();
  }
  // New (no reference counterpart): the seeded vortex state computed on the
  // device, then the same path as set_psi.
  int set_psi_vortices(int n_vort, uint64_t seed, double xi0, double min_sep, double* pos_out) override {
    if (n_vort < 0 || (n_vort % 2) != 0 || !(xi0 > 0)) {
      set_error("vk_set_psi_vortices: need an even (neutral) vortex count and positive xi0");
      return VK_E_INVALID;
    }
    std::vector<double> px, py;
    std::vector<int> q;
    int rc = vortex_positions(n_vort, seed, min_sep, px, py, q);
    if (rc) return rc;
    double S = 0.0;
    for (int j = 0; j < n_vort; ++j) S += q[j] * px[j];
    double *dx = nullptr, *dy = nullptr;
    int* dq = nullptr;
    const size_t nv = (size_t)std::max(n_vort, 1);
    VK_CUDA_TRY(cudaMalloc(&dx, sizeof(double) * nv));
    VK_CUDA_TRY(cudaMalloc(&dy, sizeof(double) * nv));
    VK_CUDA_TRY(cudaMalloc(&dq, sizeof(int) * nv));
    if (n_vort > 0) {
      VK_CUDA_TRY(cudaMemcpyAsync(dx, px.data(), sizeof(double) * n_vort, cudaMemcpyHostToDevice, st_));
      VK_CUDA_TRY(cudaMemcpyAsync(dy, py.data(), sizeof(double) * n_vort, cudaMemcpyHostToDevice, st_));
      VK_CUDA_TRY(cudaMemcpyAsync(dq, q.data(), sizeof(int) * n_vort, cudaMemcpyHostToDevice, st_));
    }
    launch_raw("k_ic_vortices", k_ic_vortices, 152 * 8, 256, 0, (double2*)stage64_, nx_, ny_, (const double*)dx,
               (const double*)dy, (const int*)dq, n_vort, xi0, S);
    if (std::is_same<T, double>::value)
      VK_CUDA_TRY(cudaMemcpyAsync(psi_, stage64_, n2_ * sizeof(double2), cudaMemcpyDeviceToDevice, st_));
    else
      launch_simple("k_from_f64", k_from_f64<T>, (const double2*)stage64_, psi_, n2_);
    rc = sync_check();
    cudaFree(dx);
    cudaFree(dy);
    cudaFree(dq);
    if (rc) return rc;
    if (pos_out)
      for (int j = 0; j < n_vort; ++j) {
        pos_out[2 * j] = px[j];
        pos_out[2 * j + 1] = py[j];
      }
    return set_psi_on_device();
  }
  int set_psi_on_device() {
    fwd2d(psi_, kpsi_, p_.otoc != 0);
    if (p_.otoc) {
      inv2d(kpsi_, psi_, true);
      kpsi_masked_ = true;
      ta_ = TA_FULL;
    } else {
      kpsi_masked_ = false;
      ta_ = TA_INVALID;
    }
    have_psi_ = true;
    return sync_check();
  }
  int set_kpsi(const double* kpsi) override {
    int rc = upload(kpsi, kpsi_);
    if (rc) return rc;
    inv2d(kpsi_, psi_, false);
    kpsi_masked_ = false;
    ta_ = TA_FULL;
    have_psi_ = true;
    return sync_check();
  }
  int get_psi(double* out) override { return download(psi_, out); }
  int get_kpsi(double* out) override { return download(kpsi_, out); }

  // One RK4 step (gpe_rk4, src/gpe.f90:310-494): four stages of four fused
  // passes, plus the particle tables/update when particles are on.
  void rk4_step(bool from_psi) {
    if (fused_grid_ > 0 && !c_.frc && np_ == 0) {
      for (int stage = 1; stage <= 4; ++stage) stage_fused(stage, from_psi && stage == 1);
      return;
    }
    for (int stage = 1; stage <= 4; ++stage) {
      x1((from_psi && stage == 1) ? 0 : 1, true);
      if (np_ > 0) {
        part_tables();
        y1_pot(true, nullptr);
        x2_pot(+1);
      } else {
        y1();
        x2(+1, true);
      }
      y2_rk4(stage);
      if (c_.frc) launch_raw("k_rng_bump", k_rng_bump<T>, 1, 1, 0, rngc_);
      if (np_ > 0) launch_raw("k_part_update", k_part_update, 1, kPartThreads, part_update_smem(np_), ps_, pc_, stage);
    }
  }

  // Launch `body` through a CUDA graph captured on first use (one graph per
  // kind of step; pointers and constants of a context never change).  Falls
  // back to direct launches if capture is not possible.
  template <typename F> int replay(cudaGraphExec_t& ge, int64_t& nk, F&& body) {
    if (!ge && graphs_ok_) {
      const int64_t l0 = launches_;
      cudaGraph_t g = nullptr;
      if (cudaStreamBeginCapture(st_, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
        body();
        if (cudaStreamEndCapture(st_, &g) == cudaSuccess && g &&
            cudaGraphInstantiate(&ge, g, 0) == cudaSuccess) {
          nk = launches_ - l0;
        } else {
          ge = nullptr;
          graphs_ok_ = false;
        }
        if (g) cudaGraphDestroy(g);
      } else {
        graphs_ok_ = false;
      }
      launches_ = l0;
      cudaGetLastError();
      launch_err_ = cudaSuccess;
    }
    if (!ge) {
      body();
      return VK_OK;
    }
    VK_CUDA_TRY(cudaGraphLaunch(ge, st_));
    launches_ += nk;
    return VK_OK;
  }

  // ---------------------------------------------------------------- RK4 --
  int rk4(int nsteps) override {
    if (!have_psi_) { set_error("vk_gpe_rk4: no psi set"); return VK_E_STATE; }
    if (nsteps <= 0) return VK_OK;
    if (!kpsi_masked_) {
      launch_simple("k_mask_four", k_mask_four<T>, kpsi_, nx_, ny_, k2max_);
      kpsi_masked_ = true;
    }
    if (np_ > 0 && !have_particles_) { set_error("vk_gpe_rk4: particles not set"); return VK_E_STATE; }
    for (int s = 0; s < nsteps; ++s) {
      if (s == 0 || timing_) {
        rk4_step(s == 0);
      } else {
        int rc = replay(g_rk4_, g_rk4_n_, [&]() { rk4_step(false); });
        if (rc) return rc;
      }
    }
    if (np_ > 0) rep_init_ = true;
    xinv_from_ta(true);
    ta_ = TA_PRUNED;
    return check_launch();
  }

  // One ARGLE step (src/gpe.f90:5-224) with the new residual sums when resid.
  void argle_step(bool resid, int nblk) {
    x1(1, false);
    if (sgle_) {  // finiteT_adhoc_chempot on the psi of this step (src/gpe.f90:189), then the noise
      launch_raw("k_sum_abs2", k_sum_abs2<T>, kNormBlocks, 256, 0, (const C*)psi_, n2_, omega_dev_ + 1);
      const double two_pi = 6.283185307179586476925286766559;
      launch_raw("k_chempot", k_chempot, 1, 32, 0, (const double*)(omega_dev_ + 1), kNormBlocks, omega_dev_,
                 c_.dt, nun_area_, (two_pi / nx_) * (two_pi / ny_), two_pi * two_pi);
      with_len(nx_, [&](auto lc) {
        constexpr int L = decltype(lc)::value;
        typedef GeoX<T, L> G;
        launch_raw("k_noise_x", k_noise_x<T, L>, ny_ / G::R, G::NT, sizeof(C) * G::R * G::LP, Tn_, (const C*)twx_, c_);
      });
    }
    if (np_ > 0) {
      y1_pot(false, nullptr);
      x2_pot(-1);
    } else if (flow_) {
      y1();
      x2_flow();
    } else {
      y1();
      x2(-1, false);
    }
    y2_argle(resid);
    if (sgle_) launch_raw("k_rng_bump", k_rng_bump<T>, 1, 1, 0, rngc_);
    if (resid) launch_raw("k_reduce_partials3", k_reduce_partials3, 1, 256, 0, (const double*)part_, nblk, sums_);
    if (p_.argle_renorm) {
      // norm = dvol * (1/(nx ny)) * sum |kpsi|^2; target Nparticle = Lx*Ly
      const double two_pi = 6.283185307179586476925286766559;
      const double dvol = (two_pi / nx_) * (two_pi / ny_);
      const double area = two_pi * two_pi;
      launch_raw("k_scale_two", k_scale_two<T>, 1024, 256, 0, kpsi_, Ta_, n2_, (const double*)sums_,
                 area / (dvol * c_.scale));
    }
  }

  // -------------------------------------------------------------- ARGLE --
  int argle(int nsteps, double* residual) override {
    if (!have_psi_) { set_error("vk_argle: no psi set"); return VK_E_STATE; }
    if (nsteps <= 0) return VK_OK;
    if (np_ > 0 && !have_particles_) { set_error("vk_argle: particles not set"); return VK_E_STATE; }
    if (ta_ != TA_FULL) yinv_to_ta();
    if (flow_) yinv_deriv_to_tg();
    const int nblk = nx_ / geo_rows_y(ny_);
    if (np_ > 0) part_tables();
    for (int s = 0; s < nsteps; ++s) {
      const bool last = (s == nsteps - 1);
      const bool resid = last || p_.argle_renorm;
      if (resid || timing_) {
        argle_step(resid, nblk);
      } else {
        int rc = replay(g_argle_, g_argle_n_, [&]() { argle_step(false, nblk); });
        if (rc) return rc;
      }
    }
    ta_ = TA_FULL;
    kpsi_masked_ = false;
    int rc = check_launch();
    if (rc) return rc;
    if (sgle_) {
      // the host copy feeds the diagnostics (echem) and any later RK4 steps,
      // whose captured graph holds the old value
      VK_CUDA_TRY(cudaMemcpyAsync(&c_.omega, omega_dev_, sizeof(double), cudaMemcpyDeviceToHost, st_));
      VK_CUDA_TRY(cudaStreamSynchronize(st_));
      if (g_rk4_) cudaGraphExecDestroy(g_rk4_);
      g_rk4_ = nullptr;
    }
    if (residual) {
      double h[3];
      VK_CUDA_TRY(cudaMemcpyAsync(h, sums_, sizeof(h), cudaMemcpyDeviceToHost, st_));
      VK_CUDA_TRY(cudaStreamSynchronize(st_));
      // a zero field stays zero: report 0 rather than 0/0
      *residual = h[1] > 0.0 ? std::sqrt(h[0]) / (p_.dt * std::sqrt(h[1])) : (h[0] > 0.0 ? HUGE_VAL : 0.0);
    }
    return VK_OK;
  }

  int diagnostics(double* scalars, double* spec, int32_t* nvort) override {
    if (!have_psi_) { set_error("vk_diagnostics: no psi set"); return VK_E_STATE; }
    return diag_.run(*this, scalars, spec, nvort);
  }

  // particle_potential + initialize_particles (src/gpe_particle.f90:3-141).
  int particles_set(const double* pos, const double* vel, const double* f0ext) override {
    const size_t b = sizeof(double) * 2 * np_;
    VK_CUDA_TRY(cudaMemcpyAsync(ps_.pos, pos, b, cudaMemcpyHostToDevice, st_));
    VK_CUDA_TRY(cudaMemcpyAsync(ps_.vel, vel, b, cudaMemcpyHostToDevice, st_));
    VK_CUDA_TRY(cudaMemcpyAsync(ps_.f0ext, f0ext, b, cudaMemcpyHostToDevice, st_));
    // origin-centred Gaussian on the sin chart x~ = (1/c)(s + s^3/6 + s^5/40),
    // s = sin(c x), c = 2 pi/(2 L)  (src/gpe_particle.f90:34-59)
    const double two_pi = 6.283185307179586476925286766559;
    const double L = two_pi, cc = two_pi / (2.0 * L), dx = L / nx_, dy = L / ny_;
    const double v0 = p_.ppot_v0, d = p_.ppot_d;
    std::vector<double> v((size_t)2 * n2_);
    for (int y = 0; y < ny_; ++y) {
      const double sy = std::sin(cc * (y * dy));
      const double yp = (1.0 / cc) * (sy + (1.0 / 6.0) * (sy * sy * sy) + (1.0 / 40.0) * (sy * sy * sy * sy * sy));
      for (int x = 0; x < nx_; ++x) {
        const double sx = std::sin(cc * (x * dx));
        const double xp = (1.0 / cc) * (sx + (1.0 / 6.0) * (sx * sx * sx) + (1.0 / 40.0) * (sx * sx * sx * sx * sx));
        const double r = std::sqrt(xp * xp + yp * yp);
        v[2 * ((size_t)y * nx_ + x)] = v0 * std::exp(-(r * r) / (2.0 * (d * d)));
        v[2 * ((size_t)y * nx_ + x) + 1] = 0.0;
      }
    }
    int rc = upload(v.data(), Ta_);
    if (rc) return rc;
    ta_ = TA_INVALID;
    fwd2d(Ta_, str1_, false);
    launch_simple("k_extract_half", k_extract_half<T>, (const C*)str1_, vhat_, K_, nx_, ny_, k2max_);
    have_particles_ = true;
    return sync_check();
  }
  int particles_get(double* pos, double* vel, double* frc) override {
    const size_t b = sizeof(double) * 2 * np_;
    if (pos) VK_CUDA_TRY(cudaMemcpyAsync(pos, ps_.pos, b, cudaMemcpyDeviceToHost, st_));
    if (vel) VK_CUDA_TRY(cudaMemcpyAsync(vel, ps_.vel, b, cudaMemcpyDeviceToHost, st_));
    if (frc) VK_CUDA_TRY(cudaMemcpyAsync(frc, ps_.frc, b, cudaMemcpyDeviceToHost, st_));
    VK_CUDA_TRY(cudaStreamSynchronize(st_));
    return VK_OK;
  }
  void part_tables() {
    const int tot = np_ * (K_ + 1 + ny_);
    launch_raw("k_part_tables", k_part_tables, std::min((tot + 255) / 256, 152 * 8), 256, 0, ps_, pc_);
  }
  void y1_pot(bool force, C* rhohat) {
    with_len(ny_, [&](auto lc) {
      constexpr int L = decltype(lc)::value;
      typedef GeoX<T, L> G;
      const size_t sm = sizeof(C) * G::R * G::LP;
      if (force) launch_raw("k_y1_pot", k_y1_pot<T, L, true>, nblk_pot_, G::NT, sm, (const C*)Tb_, (const C*)vhat_, Tc_, Tv_, rhohat, ps_, pc_, (const C*)twy_, c_);
      else launch_raw("k_y1_pot", k_y1_pot<T, L, false>, nblk_pot_, G::NT, sm, (const C*)Tb_, (const C*)vhat_, Tc_, Tv_, rhohat, ps_, pc_, (const C*)twy_, c_);
    });
  }
  void x2_pot(int sign) {
    with_len(nx_, [&](auto lc) {
      constexpr int L = decltype(lc)::value;
      typedef GeoX<T, L> G;
      const size_t sm = sizeof(C) * G::R * G::LP;
      if (sign > 0) launch_raw("k_x2_pot", k_x2_pot<T, L, +1, true>, ny_ / G::R, G::NT, sm, (const C*)Tc_, (const C*)Tv_, (const C*)psi_, Td_, (const C*)twx_, c_);
      else launch_raw("k_x2_pot", k_x2_pot<T, L, -1, false>, ny_ / G::R, G::NT, sm, (const C*)Tc_, (const C*)Tv_, (const C*)psi_, Td_, (const C*)twx_, c_);
    });
  }
  void vtot_phys() {
    with_len(nx_, [&](auto lc) {
      constexpr int L = decltype(lc)::value;
      typedef GeoX<T, L> G;
      launch_raw("k_vtot_x", k_vtot_x<T, L>, ny_ / G::R, G::NT, sizeof(C) * G::R * G::LP, (const C*)Tv_, vpot_, (const C*)twx_, c_);
    });
  }

  // ------------------------------------------------- launch helpers --
  template <typename... KA, typename... A>
  void launch_raw(const char* tag, void (*kern)(KA...), int grid, int block, size_t smem, A... args) {
    ensure_smem_attr((const void*)kern, smem);
    if (timing_ && ev_used_ == 0) record_event(nullptr);
    kern<<<grid, block, smem, st_>>>(args...);
    ++launches_;
    const cudaError_t le = cudaGetLastError();
    if (le != cudaSuccess && launch_err_ == cudaSuccess) {
      launch_err_ = le;
      launch_err_tag_ = tag;
    }
    if (timing_) record_event(tag);
  }
  // Cooperative launch (all CTAs co-resident; capturable in a graph).
  template <typename... KA, typename... A>
  void launch_coop(const char* tag, void (*kern)(KA...), int grid, int block, size_t smem, A... args) {
    ensure_smem_attr((const void*)kern, smem);
    if (timing_ && ev_used_ == 0) record_event(nullptr);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st_;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeCooperative;
    at[0].val.cooperative = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    const cudaError_t le = cudaLaunchKernelEx(&cfg, kern, args...);
    ++launches_;
    if (le != cudaSuccess && launch_err_ == cudaSuccess) {
      launch_err_ = le;
      launch_err_tag_ = tag;
    }
    if (timing_) record_event(tag);
  }

  // ------------------------------------------- persistent stage kernel --
  // FP32 at 1024^2 with VK_FUSED=1: each plain RK4 stage is one cooperative
  // launch of k_stage_rk4 over fused_grid_ CTAs (vk_stage.cuh).  Off by
  // default: on GB300 a stage took 65.9 us against 56.5 us for the four pass
  // kernels (4.17e9 against 6.21e9 grid-pt-steps/s), because the x bodies'
  // registers leave 8 warps per SM for the y passes, which run 16 as
  // separate kernels.  VK_SPIN_LIMIT sets how many polls a CTA waits at a
  // barrier before it gives up (default 2^24, about a second).
  template <int L> static constexpr bool kFusedLen = std::is_same<T, float>::value && L == 1024;
  int init_fused() {
    fused_grid_ = 0;
    const char* env = std::getenv("VK_FUSED");
    if (!(std::is_same<T, float>::value && nx_ == 1024 && ny_ == 1024) || !(env && env[0] == '1')) return VK_OK;
    int dev = 0, coop = 0, nsm = 0;
    VK_CUDA_TRY(cudaGetDevice(&dev));
    VK_CUDA_TRY(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
    VK_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    if (!coop) return VK_OK;
    const char* lim = std::getenv("VK_SPIN_LIMIT");
    spin_limit_ = lim ? std::strtoull(lim, nullptr, 10) : (1ull << 24);
    with_len(nx_, [&](auto lc) {
      constexpr int L = decltype(lc)::value;
      if constexpr (kFusedLen<L>) {
        typedef typename GeoFused<T, L>::X GX;
        typedef typename GeoFused<T, L>::Y GY;
        fused_smem_ = sizeof(C) * std::max(GX::R * GX::LP, GY::R * GY::LP);
        int occ = 1 << 30;
        auto fit = [&](const void* fn) {
          int b = 0;
          ensure_smem_attr(fn, fused_smem_);
          if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, fn, GeoFused<T, L>::NT, fused_smem_) != cudaSuccess)
            b = 0;
          occ = std::min(occ, b);
        };
        fit((const void*)k_stage_rk4<T, L, 1, false>);
        fit((const void*)k_stage_rk4<T, L, 1, true>);
        fit((const void*)k_stage_rk4<T, L, 2, true>);
        fit((const void*)k_stage_rk4<T, L, 3, true>);
        fit((const void*)k_stage_rk4<T, L, 4, true>);
        cudaGetLastError();
        const int tiles = std::max(ny_ / GX::R, (2 * K_ + GY::R) / GY::R);
        if (occ > 0) fused_grid_ = std::min(occ * nsm, tiles);
      }
    });
    if (fused_grid_ <= 0) return VK_OK;
    VK_CUDA_TRY(cudaMalloc(&bar_, sizeof(GridBarrier)));
    VK_CUDA_TRY(cudaMemset(bar_, 0, sizeof(GridBarrier)));
    return VK_OK;
  }
  void stage_fused(int stage, bool from_psi) {
    with_len(nx_, [&](auto lc) {
      constexpr int L = decltype(lc)::value;
      if constexpr (kFusedLen<L>) {
        Field<T> f;
        f.psi = psi_; f.kpsi = kpsi_; f.str1 = str1_; f.str2 = str2_;
        f.Ta = Ta_; f.Tb = Tb_; f.Tc = Tc_; f.Td = Td_;
        f.twx = twx_; f.twy = twy_; f.c = c_;
        const int nt = GeoFused<T, L>::NT;
        const unsigned long long lim = spin_limit_;
        switch (stage) {
          case 1:
            if (from_psi) launch_coop("k_stage_rk4", k_stage_rk4<T, L, 1, false>, fused_grid_, nt, fused_smem_, f, bar_, lim);
            else launch_coop("k_stage_rk4", k_stage_rk4<T, L, 1, true>, fused_grid_, nt, fused_smem_, f, bar_, lim);
            break;
          case 2: launch_coop("k_stage_rk4", k_stage_rk4<T, L, 2, true>, fused_grid_, nt, fused_smem_, f, bar_, lim); break;
          case 3: launch_coop("k_stage_rk4", k_stage_rk4<T, L, 3, true>, fused_grid_, nt, fused_smem_, f, bar_, lim); break;
          default: launch_coop("k_stage_rk4", k_stage_rk4<T, L, 4, true>, fused_grid_, nt, fused_smem_, f, bar_, lim); break;
        }
      }
    });
  }
  // A barrier that timed out leaves err set: report it once, reset the
  // barrier and invalidate the field (its contents are partial).
  int barrier_check() {
    if (!bar_) return VK_OK;
    GridBarrier h;
    VK_CUDA_TRY(cudaMemcpyAsync(&h, bar_, sizeof(h), cudaMemcpyDeviceToHost, st_));
    VK_CUDA_TRY(cudaStreamSynchronize(st_));
    if (h.err == 0) return VK_OK;
    VK_CUDA_TRY(cudaMemsetAsync(bar_, 0, sizeof(GridBarrier), st_));
    VK_CUDA_TRY(cudaStreamSynchronize(st_));
    set_error("vk_gpe_rk4: a CTA of the persistent stage kernel gave up waiting at grid barrier " +
              std::to_string(h.err - 1) + " (the field is not valid; set it again)");
    have_psi_ = false;
    return VK_E_CUDA;
  }

  template <typename... KA, typename... A>
  void launch_simple(const char* tag, void (*kern)(KA...), A... args) {
    const int grid = (int)std::min<size_t>((n2_ + 255) / 256, 152 * 16);
    launch_raw(tag, kern, grid, 256, 0, args...);
  }

  // ------------------------------------------------------ timing --
  void record_event(const char* tag) {
    if (ev_used_ >= (int)ev_.size()) {
      cudaEvent_t e;
      if (cudaEventCreate(&e) != cudaSuccess) return;
      ev_.push_back(e);
      ev_tag_.push_back(nullptr);
    }
    cudaEventRecord(ev_[ev_used_], st_);
    ev_tag_[ev_used_] = tag;
    ++ev_used_;
  }
  int timing_begin() override {
    timing_ = true;
    ev_used_ = 0;
    return VK_OK;
  }
  int timing_end(int cap, char* tags, double* ms, int64_t* counts, int* ntags) override {
    timing_ = false;
    VK_CUDA_TRY(cudaStreamSynchronize(st_));
    std::vector<std::string> names;
    std::vector<double> tot;
    std::vector<int64_t> cnt;
    for (int i = 1; i < ev_used_; ++i) {
      float t = 0.f;
      VK_CUDA_TRY(cudaEventElapsedTime(&t, ev_[i - 1], ev_[i]));
      const std::string nm = ev_tag_[i] ? ev_tag_[i] : "?";
      size_t j = 0;
      while (j < names.size() && names[j] != nm) ++j;
      if (j == names.size()) { names.push_back(nm); tot.push_back(0.0); cnt.push_back(0); }
      tot[j] += t;
      cnt[j] += 1;
    }
    const int n = (int)std::min<size_t>(names.size(), (size_t)std::max(cap, 0));
    for (int j = 0; j < n; ++j) {
      std::memset(tags + 24 * j, 0, 24);
      std::strncpy(tags + 24 * j, names[j].c_str(), 23);
      ms[j] = tot[j];
      counts[j] = cnt[j];
    }
    *ntags = (int)names.size();
    ev_used_ = 0;
    return VK_OK;
  }
  // CTAs of k_x1 / k_x2: row groups of R, then c_.xsingle single rows.
  int x_grid(int R) const { return (ny_ - c_.xsingle) / R + c_.xsingle; }
  static int geo_rows_x(int L) {
    int r = 0;
    with_len(L, [&](auto lc) { r = GeoX<T, decltype(lc)::value>::R; });
    return r;
  }
  static int geo_rows_y(int L) {
    int r = 0;
    with_len(L, [&](auto lc) { r = GeoY<T, decltype(lc)::value>::R; });
    return r;
  }

  // Forward 2D FFT phys[y][x] -> four[kx][ky] (Td as the transposed scratch).
  void fwd2d(const C* phys, C* four, bool otoc) {
    with_len(nx_, [&](auto lc) {
      constexpr int L = decltype(lc)::value;
      typedef GeoX<T, L> G;
      launch_raw("k_xfwd", k_xfwd<T, L>, ny_ / G::R, G::NT, sizeof(C) * G::R * G::LP, phys, Td_, (const C*)twx_, ny_);
    });
    with_len(ny_, [&](auto lc) {
      constexpr int L = decltype(lc)::value;
      typedef GeoY<T, L> G;
      if (otoc)
        launch_raw("k_yfwd", k_yfwd<T, L, true>, nx_ / G::R, G::NT, sizeof(C) * G::R * G::LP, (const C*)Td_, four,
                   (const C*)twy_, nx_, k2max_, p_.k_otoc_gp, p_.eps_otoc_gp);
      else
        launch_raw("k_yfwd", k_yfwd<T, L, false>, nx_ / G::R, G::NT, sizeof(C) * G::R * G::LP, (const C*)Td_, four,
                   (const C*)twy_, nx_, k2max_, 0.0, 0.0);
    });
  }
  // Inverse 2D FFT four[kx][ky] -> phys[y][x] (scaled), through Ta.
  void inv2d(const C* four, C* phys, bool prune) {
    with_len(ny_, [&](auto lc) {
      constexpr int L = decltype(lc)::value;
      typedef GeoY<T, L> G;
      launch_raw("k_yinv", k_yinv<T, L>, nx_ / G::R, G::NT, sizeof(C) * G::R * G::LP, four, Ta_, (const C*)twy_, nx_);
    });
    with_len(nx_, [&](auto lc) {
      constexpr int L = decltype(lc)::value;
      typedef GeoX<T, L> G;
      if (prune)
        launch_raw("k_xinv", k_xinv<T, L, true>, ny_ / G::R, G::NT, sizeof(C) * G::R * G::LP, (const C*)Ta_, phys,
                   (const C*)twx_, T(c_.scale), K_);
      else
        launch_raw("k_xinv", k_xinv<T, L, false>, ny_ / G::R, G::NT, sizeof(C) * G::R * G::LP, (const C*)Ta_, phys,
                   (const C*)twx_, T(c_.scale), K_);
    });
  }
  void yinv_deriv_to_tg() {
    with_len(ny_, [&](auto lc) {
      constexpr int L = decltype(lc)::value;
      typedef GeoY<T, L> G;
      launch_raw("k_yinv", k_yinv<T, L, true>, nx_ / G::R, G::NT, sizeof(C) * G::R * G::LP, (const C*)kpsi_, Tg_, (const C*)twy_, nx_);
    });
  }
  void x2_flow() {
    with_len(nx_, [&](auto lc) {
      constexpr int L = decltype(lc)::value;
      if constexpr (sizeof(T) == 4 || L <= 2048) {
        typedef GeoX<T, L> G;
        const size_t sm = sizeof(C) * 3 * G::R * G::LP;
        if (flow_ == 1)
          launch_raw("k_x2_flow", k_x2_flow<T, L, 1>, ny_ / G::R, G::NT, sm, (const C*)Tc_, (const C*)psi_, (const C*)Ta_,
                     (const C*)Tg_, Td_, (const C*)twx_, c_, vnx_, vny_);
        else
          launch_raw("k_x2_flow", k_x2_flow<T, L, 2>, ny_ / G::R, G::NT, sm, (const C*)Tc_, (const C*)psi_, (const C*)Ta_,
                     (const C*)Tg_, Td_, (const C*)twx_, c_, vnx_, vny_);
      }
    });
  }
  void yinv_to_ta() {
    with_len(ny_, [&](auto lc) {
      constexpr int L = decltype(lc)::value;
      typedef GeoY<T, L> G;
      launch_raw("k_yinv", k_yinv<T, L>, nx_ / G::R, G::NT, sizeof(C) * G::R * G::LP, (const C*)kpsi_, Ta_, (const C*)twy_, nx_);
    });
  }
  void xinv_from_ta(bool prune) {
    with_len(nx_, [&](auto lc) {
      constexpr int L = decltype(lc)::value;
      typedef GeoX<T, L> G;
      if (prune)
        launch_raw("k_xinv", k_xinv<T, L, true>, ny_ / G::R, G::NT, sizeof(C) * G::R * G::LP, (const C*)Ta_, psi_,
                   (const C*)twx_, T(c_.scale), K_);
      else
        launch_raw("k_xinv", k_xinv<T, L, false>, ny_ / G::R, G::NT, sizeof(C) * G::R * G::LP, (const C*)Ta_, psi_,
                   (const C*)twx_, T(c_.scale), K_);
    });
  }
  void x1(int from_t, bool prune) {
    with_len(nx_, [&](auto lc) {
      constexpr int L = decltype(lc)::value;
      typedef GeoX<T, L> G;
      const size_t sm = sizeof(C) * G::R * G::LP;
      const int grid = x_grid(G::R);
      auto go = [&](auto bulk_c) {
        constexpr bool B = decltype(bulk_c)::value;
        if (!from_t) launch_raw("k_x1", k_x1<T, L, false, false, B>, grid, G::NT, sm, (const C*)Ta_, psi_, Tb_, (const C*)twx_, c_);
        else if (prune) launch_raw("k_x1", k_x1<T, L, true, true, B>, grid, G::NT, sm, (const C*)Ta_, psi_, Tb_, (const C*)twx_, c_);
        else launch_raw("k_x1", k_x1<T, L, true, false, B>, grid, G::NT, sm, (const C*)Ta_, psi_, Tb_, (const C*)twx_, c_);
      };
      if constexpr (std::is_same<T, double>::value && L >= 128) {
        if (bulk_ && c_.xsingle > 0) return go(std::true_type());
      }
      go(std::false_type());
    });
  }
  void y1() {
    with_len(ny_, [&](auto lc) {
      constexpr int L = decltype(lc)::value;
      typedef GeoY<T, L> G;
      if constexpr (std::is_same<T, double>::value) {
        if (bulk_) {
          launch_raw("k_y1", k_y1<T, L, true>, (K_ + 1 + G::R - 1) / G::R, G::NT, sizeof(C) * G::R * G::LP,
                     (const C*)Tb_, Tc_, (const C*)twy_, c_);
          return;
        }
      }
      launch_raw("k_y1", k_y1<T, L>, (K_ + 1 + G::R - 1) / G::R, G::NT, sizeof(C) * G::R * G::LP, (const C*)Tb_, Tc_,
                 (const C*)twy_, c_);
    });
  }
  void x2(int sign, bool prune_out) {
    with_len(nx_, [&](auto lc) {
      constexpr int L = decltype(lc)::value;
      typedef GeoX<T, L> G;
      const size_t sm = sizeof(C) * G::R * G::LP;
      const int grid = x_grid(G::R);
      if (sign > 0) launch_raw("k_x2", k_x2<T, L, +1, true, false>, grid, G::NT, sm, (const C*)Tc_, (const C*)psi_, (const T*)nullptr, Td_, (const C*)twx_, c_);
      else launch_raw("k_x2", k_x2<T, L, -1, false, false>, grid, G::NT, sm, (const C*)Tc_, (const C*)psi_, (const T*)nullptr, Td_, (const C*)twx_, c_);
      (void)prune_out;
    });
  }
  void y2_rk4(int stage) {
    with_len(ny_, [&](auto lc) {
      constexpr int L = decltype(lc)::value;
      typedef GeoY<T, L> G;
      const int grid = (2 * K_ + 1 + G::R - 1) / G::R;
      const size_t sm = sizeof(C) * G::R * G::LP;
      auto go = [&](auto frc_c, auto bulk_c) {
        constexpr bool F = decltype(frc_c)::value, B = decltype(bulk_c)::value;
        switch (stage) {
          case 1: launch_raw("k_y2_rk4", k_y2_rk4<T, L, 1, F, B>, grid, G::NT, sm, (const C*)Td_, kpsi_, str1_, str2_, Ta_, (const C*)twy_, c_); break;
          case 2: launch_raw("k_y2_rk4", k_y2_rk4<T, L, 2, F, B>, grid, G::NT, sm, (const C*)Td_, kpsi_, str1_, str2_, Ta_, (const C*)twy_, c_); break;
          case 3: launch_raw("k_y2_rk4", k_y2_rk4<T, L, 3, F, B>, grid, G::NT, sm, (const C*)Td_, kpsi_, str1_, str2_, Ta_, (const C*)twy_, c_); break;
          default: launch_raw("k_y2_rk4", k_y2_rk4<T, L, 4, F, B>, grid, G::NT, sm, (const C*)Td_, kpsi_, str1_, str2_, Ta_, (const C*)twy_, c_); break;
        }
      };
      auto go_b = [&](auto frc_c) {
        if constexpr (std::is_same<T, double>::value) {
          if (bulk_) return go(frc_c, std::true_type());
        }
        go(frc_c, std::false_type());
      };
      if (c_.frc) go_b(std::true_type());
      else go_b(std::false_type());
    });
  }
  void y2_argle(bool resid) {
    with_len(ny_, [&](auto lc) {
      constexpr int L = decltype(lc)::value;
      typedef GeoY<T, L> G;
      const size_t sm = sizeof(C) * G::R * G::LP;
      if (sgle_) {
        auto go = [&](auto rc_, auto dc_) {
          constexpr bool RS = decltype(rc_)::value, DV = decltype(dc_)::value;
          launch_raw("k_y2_argle", k_y2_argle<T, L, RS, DV, true>, nx_ / G::R, G::NT, 2 * sm, (const C*)Td_, kpsi_, Ta_,
                     (const C*)twy_, part_, c_, Tg_, (const C*)Tn_);
        };
        if (resid && flow_) go(std::true_type(), std::true_type());
        else if (resid) go(std::true_type(), std::false_type());
        else if (flow_) go(std::false_type(), std::true_type());
        else go(std::false_type(), std::false_type());
      } else if (flow_) {
        if (resid) launch_raw("k_y2_argle", k_y2_argle<T, L, true, true>, nx_ / G::R, G::NT, 2 * sm, (const C*)Td_, kpsi_, Ta_, (const C*)twy_, part_, c_, Tg_, (const C*)nullptr);
        else launch_raw("k_y2_argle", k_y2_argle<T, L, false, true>, nx_ / G::R, G::NT, 2 * sm, (const C*)Td_, kpsi_, Ta_, (const C*)twy_, part_, c_, Tg_, (const C*)nullptr);
      } else if (resid) launch_raw("k_y2_argle", k_y2_argle<T, L, true>, nx_ / G::R, G::NT, sm, (const C*)Td_, kpsi_, Ta_, (const C*)twy_, part_, c_, (C*)nullptr, (const C*)nullptr);
      else launch_raw("k_y2_argle", k_y2_argle<T, L, false>, nx_ / G::R, G::NT, sm, (const C*)Td_, kpsi_, Ta_, (const C*)twy_, part_, c_, (C*)nullptr, (const C*)nullptr);
    });
  }

  int check_launch() {
    cudaError_t e = launch_err_;
    std::string tag = launch_err_tag_ ? launch_err_tag_ : "";
    launch_err_ = cudaSuccess;
    launch_err_tag_ = nullptr;
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) {
      set_error(std::string("kernel launch ") + tag + ": " + cudaGetErrorString(e));
      return VK_E_CUDA;
    }
    return VK_OK;
  }
  int sync_check() {
    int rc = check_launch();
    if (rc) return rc;
    VK_CUDA_TRY(cudaStreamSynchronize(st_));
    rc = barrier_check();
    return rc ? rc : async_check();
  }
  // A CTA whose wait for its bulk row loads ran out set the error word:
  // report it once, reset it and invalidate the field.
  int async_check() {
    if (!async_err_) return VK_OK;
    int h = 0;
    VK_CUDA_TRY(cudaMemcpyAsync(&h, async_err_, sizeof(int), cudaMemcpyDeviceToHost, st_));
    VK_CUDA_TRY(cudaStreamSynchronize(st_));
    if (h == 0) return VK_OK;
    VK_CUDA_TRY(cudaMemsetAsync(async_err_, 0, sizeof(int), st_));
    VK_CUDA_TRY(cudaStreamSynchronize(st_));
    set_error("vk_gpe_rk4: a CTA of a row pass gave up waiting for its bulk row loads (the field is not valid; "
              "set it again)");
    have_psi_ = false;
    return VK_E_CUDA;
  }

  int upload(const double* host, C* dev) {
    if (std::is_same<T, double>::value) {
      VK_CUDA_TRY(cudaMemcpyAsync(dev, host, n2_ * sizeof(double2), cudaMemcpyHostToDevice, st_));
    } else {
      VK_CUDA_TRY(cudaMemcpyAsync(stage64_, host, n2_ * sizeof(double2), cudaMemcpyHostToDevice, st_));
      launch_simple("k_from_f64", k_from_f64<T>, (const double2*)stage64_, dev, n2_);
    }
    return check_launch();
  }
  int download(const C* dev, double* host) {
    if (std::is_same<T, double>::value) {
      VK_CUDA_TRY(cudaMemcpyAsync(host, dev, n2_ * sizeof(double2), cudaMemcpyDeviceToHost, st_));
    } else {
      launch_simple("k_to_f64", k_to_f64<T>, dev, (double2*)stage64_, n2_);
      VK_CUDA_TRY(cudaMemcpyAsync(host, stage64_, n2_ * sizeof(double2), cudaMemcpyDeviceToHost, st_));
    }
    return sync_check();
  }

  int upload_twiddles(int n, C** dst) {
    std::vector<double> h(2 * (size_t)n);
    twiddle_table(n, h.data());
    std::vector<C> t(n);
    for (int k = 0; k < n; ++k) { t[k].x = T(h[2 * k]); t[k].y = T(h[2 * k + 1]); }
    VK_CUDA_TRY(cudaMalloc(dst, sizeof(C) * n));
    VK_CUDA_TRY(cudaMemcpy(*dst, t.data(), sizeof(C) * n, cudaMemcpyHostToDevice));
    return VK_OK;
  }

  void release() {
    diag_.release();
    if (g_rk4_) cudaGraphExecDestroy(g_rk4_);
    if (g_argle_) cudaGraphExecDestroy(g_argle_);
    g_rk4_ = g_argle_ = nullptr;
    for (auto e : ev_) cudaEventDestroy(e);
    ev_.clear();
    if (twy_ && twy_ != twx_) cudaFree(twy_);
    C* bufs[] = {psi_, kpsi_, str1_, str2_, Ta_, Td_, Tb_, Tc_, twx_};
    for (C* b : bufs)
      if (b) cudaFree(b);
    if (vpot_) cudaFree(vpot_);
    if (vhat_) cudaFree(vhat_);
    if (Tv_) cudaFree(Tv_);
    double* pb[] = {ps_.pos, ps_.vel, ps_.tpos, ps_.tvel, ps_.ku, ps_.kq, ps_.f0ext, ps_.frc, ps_.tab_x, ps_.tab_y, ps_.fpart};
    for (double* b : pb)
      if (b) cudaFree(b);
    ps_ = PartState{};
    vpot_ = nullptr;
    vhat_ = Tv_ = nullptr;
    if (stage64_) cudaFree(stage64_);
    if (part_) cudaFree(part_);
    if (sums_) cudaFree(sums_);
    if (bar_) cudaFree(bar_);
    if (async_err_) cudaFree(async_err_);
    async_err_ = nullptr;
    if (rngc_) cudaFree(rngc_);
    rngc_ = nullptr;
    if (Tg_) cudaFree(Tg_);
    Tg_ = nullptr;
    if (Tn_) cudaFree(Tn_);
    Tn_ = nullptr;
    if (dump_st_) cudaStreamSynchronize(dump_st_);
    if (dump_dev_) cudaFree(dump_dev_);
    if (dump_host_) cudaFreeHost(dump_host_);
    if (dump_st_) cudaStreamDestroy(dump_st_);
    if (dump_snap_) cudaEventDestroy(dump_snap_);
    if (dump_done_) cudaEventDestroy(dump_done_);
    dump_dev_ = nullptr;
    dump_host_ = nullptr;
    dump_st_ = nullptr;
    dump_snap_ = dump_done_ = nullptr;
    if (omega_dev_) cudaFree(omega_dev_);
    omega_dev_ = nullptr;
    if (st_) cudaStreamDestroy(st_);
    psi_ = kpsi_ = str1_ = str2_ = Ta_ = Td_ = Tb_ = Tc_ = twx_ = twy_ = nullptr;
    st_ = nullptr;
  }

  // state (public for the diagnostics helper)
  vk_params p_;
  int nx_ = 0, ny_ = 0, K_ = 0, k2max_ = 0, pk_ = 0, nshell_ = 0;
  size_t n2_ = 0;
  cudaStream_t st_ = nullptr;
  C *psi_ = nullptr, *kpsi_ = nullptr, *str1_ = nullptr, *str2_ = nullptr;
  C *Ta_ = nullptr, *Tb_ = nullptr, *Tc_ = nullptr, *Td_ = nullptr;
  C *twx_ = nullptr, *twy_ = nullptr;
  T* vpot_ = nullptr;   // V_tot(x), real (diagnostics)
  C *vhat_ = nullptr, *Tv_ = nullptr;
  PartState ps_{};
  PartConsts pc_{};
  int np_ = 0, nblk_pot_ = 0;
  bool have_particles_ = false, rep_init_ = false;
  double erep_factor_ = 0.0;
  void* stage64_ = nullptr;
  double* part_ = nullptr;
  double* sums_ = nullptr;
  StepConsts c_{};
  bool kpsi_masked_ = false, have_psi_ = false;
  int ta_ = TA_INVALID;
  int64_t launches_ = 0;
  bool timing_ = false;
  bool graphs_ok_ = true;
  cudaGraphExec_t g_rk4_ = nullptr, g_argle_ = nullptr;
  unsigned long long* rngc_ = nullptr;  // forcing-phase counter (RHS evaluations)
  int flow_ = 0;                          // ARGLE flow terms: 1 advection, 2 counterflow
  int sgle_ = 0;                          // -DGPE_SGLE noise + chemical potential ODE
  double nun_area_ = 0.0;                 // nuN / (Lx Ly)
  static constexpr int kNormBlocks = 152 * 4;
  double* omega_dev_ = nullptr;           // [0] omega_chem, [1..] norm partial sums
  C* Tn_ = nullptr;                       // x-spectrum of the SGLE noise
  double2* dump_dev_ = nullptr;           // asynchronous dump: device snapshot (FP64)
  double2* dump_host_ = nullptr;          //   pinned host copy
  cudaStream_t dump_st_ = nullptr;
  cudaEvent_t dump_snap_ = nullptr, dump_done_ = nullptr;
  bool dump_pending_ = false;
  double vnx_ = 0.0, vny_ = 0.0;
  C* Tg_ = nullptr;                       // F^-1_y[i ky kpsi] for the flow terms
  int64_t g_rk4_n_ = 0, g_argle_n_ = 0;
  cudaError_t launch_err_ = cudaSuccess;
  const char* launch_err_tag_ = nullptr;
  int ev_used_ = 0;
  std::vector<cudaEvent_t> ev_;
  std::vector<const char*> ev_tag_;
  Diagnostics<T> diag_;
  GridBarrier* bar_ = nullptr;            // persistent stage kernel: barrier state
  int fused_grid_ = 0;                    //   its CTAs (0: the four pass kernels)
  size_t fused_smem_ = 0;
  unsigned long long spin_limit_ = 1ull << 24;
  bool bulk_ = false;                     // FP64 bulk row loads
  int* async_err_ = nullptr;              // their error word
};

}  // namespace VK_SOLVER_NS
}  // namespace vk
