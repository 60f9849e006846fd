// vk_diag.cuh -- diagnostics_gpe (src/diagnostics.f90:4-634) on the GPU.
//
// Passes (N^2 grid, K = largest kept |k|):
//   1. F^-1[i kx kpsi], F^-1[i ky kpsi]  (y pass with the multiplier, x pass)
//      -> grad_x psi, grad_y psi                      (diagnostics.f90:55-71)
//   2. rho = |psi|^2 -> F -> 2/3 mask (masked rho^ kept for the interaction
//      spectrum) -> F^-1 -> P_G rho                  (:84-149)
//   3. fused x pass: P_G rho; FP64 partial sums of momentum, |grad psi|^2,
//      |psi|^2, |P_G rho||psi|^2, V P_G rho (:84-207); w = conj(psi) grad
//      psi/(|psi|+1e-30) (:265-275) -> f1 = 2 alpha Im w_x, f2 = 2 alpha Im w_y,
//      f3 = Re w_x, f4 = Re w_y (:303-317), two real fields per complex F_x
//   4. spectra y pass over kx in [0, K]: F_y, Helmholtz split, shell index
//      mshl = nint(|k|) in integer arithmetic, six shell sums in a
//      shared-memory histogram (:332-402); modes with kx > 0 stand for their
//      Hermitian mirror (weight 2) for the real fields' spectra 1-5
//   5. fixed-order reduction of the per-CTA histograms
//   6. signed plaquette winding count of psi (new, no reference counterpart)
// Shell sums are FP64 in both precisions; scalars are summed on the host
// with Neumaier compensation in a fixed order.
#pragma once
#include <cmath>
#include <vector>
#include "vk_kernels.cuh"
#include "vk_solver.h"

namespace vk {

// Nearest integer to sqrt(k2) (the reference's nint(sqrt(rk2)), |rk| is never
// a half-integer for integer k2) computed in integers.
__device__ __forceinline__ int shell_of(int k2) {
  int m = (int)sqrt((double)k2);
  while ((m + 1) * (m + 1) <= k2) ++m;
  while (m * m > k2) --m;
  return (k2 > m * m + m) ? m + 1 : m;
}

// rows kx of kpsi --(* i kx  or  * i ky)--> F^-1_y --> dst[y][kx]
template <typename T, int L, int AXIS>
__global__ void __launch_bounds__(GeoY<T, L>::NT, GeoY<T, L>::MINB) k_yinv_grad(const cplx<T>* __restrict__ kpsi, cplx<T>* __restrict__ dst,
                                                          const cplx<T>* __restrict__ tw, int nx) {
  typedef GeoY<T, L> G;
  typedef cplx<T> C;
  extern __shared__ __align__(16) unsigned char smraw[];
  C* s = reinterpret_cast<C*>(smraw);
  const int x0 = blockIdx.x * G::R;
  for (int e = threadIdx.x; e < G::R * L; e += G::NT) {
    const int r = e / L, y = e % L;
    const C v = kpsi[(size_t)(x0 + r) * L + y];
    const T k = T(AXIS == 0 ? kwn(x0 + r, nx) : kwn(y, L));
    s[r * G::LP + pidx(y)] = mkc<T>(-k * v.y, k * v.x);  // (zi*k)*kpsi
  }
  __syncthreads();
  fft_rows<T, L, G::R, G::NT, +1>(s, tw);
  for (int e = threadIdx.x; e < G::R * L; e += G::NT) {
    const int r = e % G::R, y = e / G::R;
    dst[(size_t)y * nx + x0 + r] = s[r * G::LP + pidx(y)];
  }
}

// Y1 of the diagnostics: like k_y1 but also stores the masked rho^ rows
// kx in [0,K] (all ky) for the interaction spectrum.
template <typename T, int L>
__global__ void __launch_bounds__(GeoY<T, L>::NT, GeoY<T, L>::MINB) k_y1_store(const cplx<T>* __restrict__ Tb, cplx<T>* __restrict__ Tc,
                                                         cplx<T>* __restrict__ rhohat, const cplx<T>* __restrict__ tw,
                                                         StepConsts c) {
  typedef GeoY<T, L> G;
  typedef cplx<T> C;
  extern __shared__ __align__(16) unsigned char smraw[];
  C* s = reinterpret_cast<C*>(smraw);
  const int l0 = blockIdx.x * G::R;
  const int K = c.K;
  for (int e = threadIdx.x; e < G::R * L; e += G::NT) {
    const int r = e / L, y = e % L;
    C v = mkc<T>(T(0), T(0));
    if (l0 + r <= K) v = Tb[(size_t)(l0 + r) * L + y];
    s[r * G::LP + pidx(y)] = v;
  }
  __syncthreads();
  fft_rows<T, L, G::R, G::NT, -1>(s, tw);
  for (int e = threadIdx.x; e < G::R * L; e += G::NT) {
    const int r = e / L, ky = e % L;
    const int k1 = l0 + r, k2 = kwn(ky, L);
    C v = s[r * G::LP + pidx(ky)];
    if (k1 * k1 + k2 * k2 > c.k2max) {
      v = mkc<T>(T(0), T(0));
      s[r * G::LP + pidx(ky)] = v;
    }
    if (k1 <= K) rhohat[(size_t)k1 * L + ky] = v;
  }
  __syncthreads();
  fft_rows<T, L, G::R, G::NT, +1>(s, tw);
  for (int e = threadIdx.x; e < G::R * L; e += G::NT) {
    const int r = e % G::R, y = e / G::R;
    if (l0 + r <= K) Tc[(size_t)y * c.pk + l0 + r] = s[r * G::LP + pidx(y)];
  }
}

// Per-CTA scalar partial sums written by k_dx (8 per CTA).
enum DiagSum { DS_MOMX = 0, DS_MOMY, DS_GRAD2, DS_RHO, DS_EINT, DS_EPOT, DS_N };

// Fused diagnostic x pass over rows y (see the file comment, step 3).
// Outputs: F12[kx][y], F34[kx][y] (kx in [0,K]) as interleaved half spectra:
// F12 holds f1's x-spectrum in rows [0,K] and f2's in rows [K+1, 2K+1];
// F34 likewise for f3, f4.
template <typename T, int L, bool POT>
__global__ void __launch_bounds__(GeoX<T, L>::NT, GeoX<T, L>::MINB) k_dx(const cplx<T>* __restrict__ Tc, const cplx<T>* __restrict__ psi,
                                                   const cplx<T>* __restrict__ gx, const cplx<T>* __restrict__ gy,
                                                   const T* __restrict__ vpot, cplx<T>* __restrict__ F12,
                                                   cplx<T>* __restrict__ F34, double* __restrict__ part,
                                                   const cplx<T>* __restrict__ tw, StepConsts c) {
  typedef GeoX<T, L> G;
  typedef cplx<T> C;
  extern __shared__ __align__(16) unsigned char smraw[];
  C* s = reinterpret_cast<C*>(smraw);
  static_assert(G::NT <= 512, "reduction buffer");
  __shared__ double red[DS_N][512];
  const int y0 = blockIdx.x * G::R;
  const int K = c.K, ny = c.ny, pk = c.pk;
  constexpr int NPAIR = G::R / 2;
  // P_G rho rows in pairs (as in k_x2)
  for (int e = threadIdx.x; e < NPAIR * L; e += G::NT) {
    const int p = e / L, k = e % L;
    C v = mkc<T>(T(0), T(0));
    const size_t ra = (size_t)(y0 + 2 * p) * pk, rb = ra + pk;
    if (k <= K) {
      const C a = Tc[ra + k], b = Tc[rb + k];
      v = mkc<T>(a.x - b.y, a.y + b.x);
    } else if (k >= L - K) {
      const C a = Tc[ra + (L - k)], b = Tc[rb + (L - k)];
      v = mkc<T>(a.x + b.y, b.x - a.y);
    }
    s[p * G::LP + pidx(k)] = v;
  }
  __syncthreads();
  fft_rows<T, L, NPAIR, G::NT, +1, G::NT>(s, tw);
  constexpr int PER = G::R * L / G::NT;
  C z1[PER], z2[PER];
  double acc[DS_N] = {0, 0, 0, 0, 0, 0};
  const T scale = T(c.scale);
  const T two_alpha = T(2.0 * c.alpha);
  const T sml = T((double)1e-30f);  // smlnum = 1e-30 (default-real literal, diagnostics.f90:43)
#pragma unroll
  for (int q = 0; q < PER; ++q) {
    const int e = threadIdx.x + q * G::NT;
    const int r = e / L, x = e % L;
    const size_t gi = (size_t)(y0 + r) * L + x;
    const C zp = s[(r >> 1) * G::LP + pidx(x)];
    const T pg = ((r & 1) == 0 ? zp.x : zp.y) * scale;
    const C ps = psi[gi], ax = gx[gi], ay = gy[gi];
    acc[DS_MOMX] += (double)(ps.x * ax.y - ps.y * ax.x);
    acc[DS_MOMY] += (double)(ps.x * ay.y - ps.y * ay.x);
    acc[DS_GRAD2] += (double)(ax.x * ax.x + ax.y * ax.y) + (double)(ay.x * ay.x + ay.y * ay.y);
    const T r2 = ps.x * ps.x + ps.y * ps.y;
    acc[DS_RHO] += (double)r2;
    acc[DS_EINT] += (double)(fabs(pg) * r2);
    if (POT) acc[DS_EPOT] += (double)(vpot[gi] * pg);
    const T rl = sqrt(r2) + sml;
    // w = conj(psi) * grad psi / rholoc
    const T wxr = (ps.x * ax.x + ps.y * ax.y) / rl, wxi = (ps.x * ax.y - ps.y * ax.x) / rl;
    const T wyr = (ps.x * ay.x + ps.y * ay.y) / rl, wyi = (ps.x * ay.y - ps.y * ay.x) / rl;
    z1[q] = mkc<T>(two_alpha * wxi, two_alpha * wyi);  // f1 + i f2
    z2[q] = mkc<T>(wxr, wyr);                          // f3 + i f4
  }
#pragma unroll
  for (int j = 0; j < DS_N; ++j) red[j][threadIdx.x] = acc[j];
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int j = 0; j < DS_N; ++j) {
      double a = 0.0;
      for (int t = 0; t < G::NT; ++t) a += red[j][t];
      part[(size_t)blockIdx.x * 8 + j] = a;
    }
  }
  for (int pass = 0; pass < 2; ++pass) {
#pragma unroll
    for (int q = 0; q < PER; ++q) {
      const int e = threadIdx.x + q * G::NT;
      const int r = e / L, x = e % L;
      s[r * G::LP + pidx(x)] = pass == 0 ? z1[q] : z2[q];
    }
    __syncthreads();
    fft_rows<T, L, G::R, G::NT, -1>(s, tw);
    cplx<T>* out = pass == 0 ? F12 : F34;
    // unpack the two real fields of each row: A = (Z(k)+conj Z(-k))/2 -> rows [0,K],
    // B = -i(Z(k)-conj Z(-k))/2 -> rows [K+1, 2K+1]
    for (int e = threadIdx.x; e < G::R * (K + 1); e += G::NT) {
      const int r = e % G::R, k = e / G::R;
      const C zk = s[r * G::LP + pidx(k)];
      const C zm = s[r * G::LP + pidx((L - k) & (L - 1))];
      out[(size_t)k * ny + y0 + r] = mkc<T>(T(0.5) * (zk.x + zm.x), T(0.5) * (zk.y - zm.y));
      out[(size_t)(K + 1 + k) * ny + y0 + r] = mkc<T>(T(0.5) * (zk.y + zm.y), T(0.5) * (zm.x - zk.x));
    }
    __syncthreads();
  }
}

// Spectra y pass: one CTA per kx in [0, K]; smem rows 0/1 hold f1,f2 (then
// f3,f4) x-spectra of that kx.  hist[6][nsh] in shared memory (FP64).
struct SpecConsts {
  int nx, ny, K, k2max, nsh;  // nsh = shells kept in the histogram (>= shell of k2max + 1)
  double alpha, g, enorm;
};

template <typename T, int L, int NTS>
__global__ void __launch_bounds__(NTS) k_dy_spec(const cplx<T>* __restrict__ F12, const cplx<T>* __restrict__ F34,
                                              const cplx<T>* __restrict__ rhohat, const cplx<T>* __restrict__ kpsi,
                                              double* __restrict__ hpart, const cplx<T>* __restrict__ tw,
                                              SpecConsts c) {
  typedef cplx<T> C;
  constexpr int LP = padded(L);
  constexpr int NTA = 2 * L / 16;  // threads doing FFT work
  static_assert(NTA <= NTS, "block too small");
  extern __shared__ __align__(16) unsigned char smraw[];
  C* s = reinterpret_cast<C*>(smraw);
  double* hist = reinterpret_cast<double*>(smraw + sizeof(C) * 2 * LP);
  const int kx = blockIdx.x;  // 0..K
  const int K = c.K, nx = c.nx;
  for (int i = threadIdx.x; i < 6 * c.nsh; i += NTS) hist[i] = 0.0;
  for (int e = threadIdx.x; e < 2 * L; e += NTS) {
    const int r = e / L, y = e % L;
    s[r * LP + pidx(y)] = F12[(size_t)(r * (K + 1) + kx) * L + y];
  }
  __syncthreads();
  fft_rows<T, L, 2, NTA, -1, NTS>(s, tw);
  const double w = kx == 0 ? 1.0 : 2.0;  // this mode + its Hermitian mirror (-kx,-ky)
  const double en = c.enorm, al = c.alpha;
  const double kxd = (double)kx;
  for (int ky = threadIdx.x; ky < L; ky += NTS) {
    const int k2i = kwn(ky, L);
    const int ksq = kx * kx + k2i * k2i;
    if (ksq > c.k2max) continue;
    const int m = shell_of(ksq);
    const C a1 = s[pidx(ky)], a2 = s[LP + pidx(ky)];
    const double aa1r = a1.x, aa1i = a1.y, aa2r = a2.x, aa2i = a2.y;
    const double kyd = (double)k2i, kr2 = (double)ksq;
    // bb = -zi*(kx/k^2)*aa1 - zi*(ky/k^2)*aa2 ; cc = zi*k*bb ; dd = aa - cc
    double bbr = 0.0, bbi = 0.0;
    if (ksq != 0) {
      const double fx = kxd / kr2, fy = kyd / kr2;
      bbr = fx * aa1i + fy * aa2i;
      bbi = -(fx * aa1r + fy * aa2r);
    }
    const double c1r = -kxd * bbi, c1i = kxd * bbr, c2r = -kyd * bbi, c2i = kyd * bbr;
    const double d1r = aa1r - c1r, d1i = aa1i - c1i, d2r = aa2r - c2r, d2i = aa2i - c2i;
    const double ekint = en * (aa1r * aa1r + aa1i * aa1i + aa2r * aa2r + aa2i * aa2i);
    const double ekinc = en * (c1r * c1r + c1i * c1i + c2r * c2r + c2i * c2i);
    const double ekini = en * (d1r * d1r + d1i * d1i + d2r * d2r + d2i * d2i);
    const C rh = rhohat[(size_t)kx * L + ky];
    const double eint = en * ((double)rh.x * rh.x + (double)rh.y * rh.y);
    const C p0 = kpsi[(size_t)kx * L + ky];
    double eocc = en * ((double)p0.x * p0.x + (double)p0.y * p0.y);
    if (kx > 0) {
      const C p1 = kpsi[(size_t)(nx - kx) * L + ky];
      eocc += en * ((double)p1.x * p1.x + (double)p1.y * p1.y);
    }
    atomicAdd(&hist[0 * c.nsh + m], w * ekint * 0.5);
    atomicAdd(&hist[1 * c.nsh + m], w * ekini * 0.5);
    atomicAdd(&hist[2 * c.nsh + m], w * ekinc * 0.5);
    atomicAdd(&hist[4 * c.nsh + m], w * eint * 0.5 * c.g * 2.0 * al);
    atomicAdd(&hist[5 * c.nsh + m], eocc);
  }
  __syncthreads();
  for (int e = threadIdx.x; e < 2 * L; e += NTS) {
    const int r = e / L, y = e % L;
    s[r * LP + pidx(y)] = F34[(size_t)(r * (K + 1) + kx) * L + y];
  }
  __syncthreads();
  fft_rows<T, L, 2, NTA, -1, NTS>(s, tw);
  for (int ky = threadIdx.x; ky < L; ky += NTS) {
    const int k2i = kwn(ky, L);
    const int ksq = kx * kx + k2i * k2i;
    if (ksq > c.k2max) continue;
    const int m = shell_of(ksq);
    const C e1 = s[pidx(ky)], e2 = s[LP + pidx(ky)];
    const double equnt = en * ((double)e1.x * e1.x + (double)e1.y * e1.y + (double)e2.x * e2.x + (double)e2.y * e2.y);
    atomicAdd(&hist[3 * c.nsh + m], w * equnt * 2.0 * (al * al));
  }
  __syncthreads();
  for (int i = threadIdx.x; i < 6 * c.nsh; i += NTS) hpart[(size_t)blockIdx.x * 6 * c.nsh + i] = hist[i];
}

// spec[j][m] = sum over CTAs of hpart[b][j][m] (fixed order), m < nsh.
__global__ void k_spec_reduce(const double* __restrict__ hpart, int nblk, int nsh, double* __restrict__ spec);

// Signed plaquette windings of psi: counts[0] += #(+1), counts[1] += #(-1).
template <typename T>
__global__ void k_vortex_count(const cplx<T>* __restrict__ psi, int nx, int ny, int* __restrict__ counts) {
  __shared__ int sp, sm;
  if (threadIdx.x == 0) { sp = 0; sm = 0; }
  __syncthreads();
  int lp = 0, lm = 0;
  const size_t n = (size_t)nx * ny;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int y = (int)(i / nx), x = (int)(i % nx);
    const int x1 = (x + 1) % nx, y1 = (y + 1) % ny;
    const cplx<T> a = psi[(size_t)y * nx + x], b = psi[(size_t)y * nx + x1];
    const cplx<T> cc = psi[(size_t)y1 * nx + x1], d = psi[(size_t)y1 * nx + x];
    auto dph = [](cplx<T> u, cplx<T> v) {  // arg(conj(u) v)
      const double re = (double)u.x * v.x + (double)u.y * v.y, im = (double)u.x * v.y - (double)u.y * v.x;
      return atan2(im, re);
    };
    const double wsum = dph(a, b) + dph(b, cc) + dph(cc, d) + dph(d, a);
    const long q = lround(wsum / 6.283185307179586476925286766559);
    if (q > 0) lp += (int)q;
    if (q < 0) lm += (int)(-q);
  }
  atomicAdd(&sp, lp);
  atomicAdd(&sm, lm);
  __syncthreads();
  if (threadIdx.x == 0) {
    atomicAdd(&counts[0], sp);
    atomicAdd(&counts[1], sm);
  }
}

static inline double neumaier_sum(const double* a, size_t n, size_t stride) {
  double s = 0.0, c = 0.0;
  for (size_t i = 0; i < n; ++i) {
    const double v = a[i * stride];
    const double t = s + v;
    if (std::fabs(s) >= std::fabs(v)) c += (s - t) + v;
    else c += (v - t) + s;
    s = t;
  }
  return s + c;
}

template <typename T>
struct Diagnostics {
  typedef cplx<T> C;
  C *dt_ = nullptr, *gx_ = nullptr, *gy_ = nullptr, *f12_ = nullptr, *f34_ = nullptr, *rhohat_ = nullptr;
  double *part_ = nullptr, *hpart_ = nullptr, *spec_ = nullptr;
  int* cnt_ = nullptr;
  int nsh_ = 0;
  bool ready_ = false;

  template <typename S>
  int alloc(S& S_) {
    if (ready_) return VK_OK;
    const size_t n2 = S_.n2_;
    const int K = S_.K_, nx = S_.nx_, ny = S_.ny_;
    nsh_ = K + 3;
    if (cudaMalloc(&dt_, sizeof(C) * n2) || cudaMalloc(&gx_, sizeof(C) * n2) || cudaMalloc(&gy_, sizeof(C) * n2) ||
        cudaMalloc(&f12_, sizeof(C) * 2 * (size_t)(K + 1) * ny) ||
        cudaMalloc(&f34_, sizeof(C) * 2 * (size_t)(K + 1) * ny) ||
        cudaMalloc(&rhohat_, sizeof(C) * (size_t)(K + 1) * ny) || cudaMalloc(&part_, sizeof(double) * 8 * ny) ||
        cudaMalloc(&hpart_, sizeof(double) * 6 * (size_t)nsh_ * (K + 1)) ||
        cudaMalloc(&spec_, sizeof(double) * 6 * (size_t)nsh_) || cudaMalloc(&cnt_, sizeof(int) * 2)) {
      set_error("vk_diagnostics: device allocation failed");
      release();
      return VK_E_NOMEM;
    }
    (void)nx;
    ready_ = true;
    return VK_OK;
  }

  void release() {
    void* bufs[] = {dt_, gx_, gy_, f12_, f34_, rhohat_, part_, hpart_, spec_, cnt_};
    for (void* b : bufs)
      if (b) cudaFree(b);
    dt_ = gx_ = gy_ = f12_ = f34_ = rhohat_ = nullptr;
    part_ = hpart_ = spec_ = nullptr;
    cnt_ = nullptr;
    ready_ = false;
  }

  template <typename S>
  int run(S& S_, double* scalars, double* spec_out, int32_t* nvort) {
    int rc = alloc(S_);
    if (rc) return rc;
    const int nx = S_.nx_, ny = S_.ny_, K = S_.K_;
    StepConsts c = S_.c_;
    c.rho_bg = 0.0;  // the diagnostics need P_G rho itself
    // 1. gradients
    for (int axis = 0; axis < 2; ++axis) {
      with_len(ny, [&](auto lc) {
        constexpr int L = decltype(lc)::value;
        typedef GeoY<T, L> G;
        const size_t sm = sizeof(C) * G::R * G::LP;
        if (axis == 0) S_.launch_raw("k_yinv_grad", k_yinv_grad<T, L, 0>, nx / G::R, G::NT, sm, (const C*)S_.kpsi_, dt_, (const C*)S_.twy_, nx);
        else S_.launch_raw("k_yinv_grad", k_yinv_grad<T, L, 1>, nx / G::R, G::NT, sm, (const C*)S_.kpsi_, dt_, (const C*)S_.twy_, nx);
      });
      with_len(nx, [&](auto lc) {
        constexpr int L = decltype(lc)::value;
        typedef GeoX<T, L> G;
        S_.launch_raw("k_xinv", k_xinv<T, L, false>, ny / G::R, G::NT, sizeof(C) * G::R * G::LP, (const C*)dt_,
                      axis == 0 ? gx_ : gy_, (const C*)S_.twx_, T(c.scale), K);
      });
    }
    // 2. rho round trip, storing the masked rho^
    with_len(nx, [&](auto lc) {
      constexpr int L = decltype(lc)::value;
      typedef GeoX<T, L> G;
      S_.launch_raw("k_x1", k_x1<T, L, false, false>, S_.x_grid(G::R), G::NT, sizeof(C) * G::R * G::LP, (const C*)S_.Ta_,
                    S_.psi_, S_.Tb_, (const C*)S_.twx_, c);
    });
    if (S_.np_ > 0) {
      // translate_particle_potential(0) for eppot (diagnostics.f90:73-77) and the
      // Parseval force partials for the gp_frc_obj loop (:528-533)
      S_.part_tables();
      S_.y1_pot(true, rhohat_);
      S_.vtot_phys();
    } else {
      with_len(ny, [&](auto lc) {
        constexpr int L = decltype(lc)::value;
        typedef GeoY<T, L> G;
        S_.launch_raw("k_y1_store", k_y1_store<T, L>, (K + 1 + G::R - 1) / G::R, G::NT, sizeof(C) * G::R * G::LP,
                      (const C*)S_.Tb_, S_.Tc_, rhohat_, (const C*)S_.twy_, c);
      });
    }
    // 3. fused x pass
    const int nblk_x = ny / S_.geo_rows_x(nx);
    with_len(nx, [&](auto lc) {
      constexpr int L = decltype(lc)::value;
      typedef GeoX<T, L> G;
      const size_t sm = sizeof(C) * G::R * G::LP;
      if (S_.np_ > 0)
        S_.launch_raw("k_dx", k_dx<T, L, true>, ny / G::R, G::NT, sm, (const C*)S_.Tc_, (const C*)S_.psi_,
                      (const C*)gx_, (const C*)gy_, (const T*)S_.vpot_, f12_, f34_, part_, (const C*)S_.twx_, c);
      else
        S_.launch_raw("k_dx", k_dx<T, L, false>, ny / G::R, G::NT, sm, (const C*)S_.Tc_, (const C*)S_.psi_,
                      (const C*)gx_, (const C*)gy_, (const T*)nullptr, f12_, f34_, part_, (const C*)S_.twx_, c);
    });
    // 4. spectra
    SpecConsts sc;
    sc.nx = nx;
    sc.ny = ny;
    sc.K = K;
    sc.k2max = S_.k2max_;
    sc.nsh = nsh_;
    sc.alpha = S_.p_.alpha;
    sc.g = S_.p_.gstrength;
    const double inv = 1.0 / ((double)nx * (double)ny);
    sc.enorm = inv * inv;
    with_len(ny, [&](auto lc) {
      constexpr int L = decltype(lc)::value;
      constexpr int NTS = (2 * L / 16) < 32 ? 32 : (2 * L / 16);
      const size_t sm = sizeof(C) * 2 * padded(L) + sizeof(double) * 6 * (size_t)nsh_;
      S_.launch_raw("k_dy_spec", k_dy_spec<T, L, NTS>, K + 1, NTS, sm, (const C*)f12_, (const C*)f34_,
                    (const C*)rhohat_, (const C*)S_.kpsi_, hpart_, (const C*)S_.twy_, sc);
    });
    S_.launch_raw("k_spec_reduce", k_spec_reduce, (6 * nsh_ + 255) / 256, 256, 0, (const double*)hpart_, K + 1,
                  nsh_, spec_);
    if (S_.np_ > 0) S_.launch_raw("k_part_update", k_part_update, 1, kPartThreads, part_update_smem(S_.np_), S_.ps_, S_.pc_, 0);
    // 6. vortex count
    if (cudaMemsetAsync(cnt_, 0, 2 * sizeof(int), S_.st_) != cudaSuccess) {
      set_error("vk_diagnostics: memset failed");
      return VK_E_CUDA;
    }
    S_.launch_raw("k_vortex_count", k_vortex_count<T>, (int)std::min<size_t>((S_.n2_ + 255) / 256, 152 * 8), 256,
                  0, (const C*)S_.psi_, nx, ny, cnt_);
    rc = S_.check_launch();
    if (rc) return rc;
    std::vector<double> part((size_t)8 * nblk_x), sp((size_t)6 * nsh_);
    int cnt[2];
    if (cudaMemcpyAsync(part.data(), part_, sizeof(double) * part.size(), cudaMemcpyDeviceToHost, S_.st_) ||
        cudaMemcpyAsync(sp.data(), spec_, sizeof(double) * sp.size(), cudaMemcpyDeviceToHost, S_.st_) ||
        cudaMemcpyAsync(cnt, cnt_, sizeof(cnt), cudaMemcpyDeviceToHost, S_.st_) ||
        cudaStreamSynchronize(S_.st_)) {
      set_error(std::string("vk_diagnostics: ") + cudaGetErrorString(cudaGetLastError()));
      return VK_E_CUDA;
    }
    const double two_pi = 6.283185307179586476925286766559;
    const double dvol = (two_pi / nx) * (two_pi / ny), area = two_pi * two_pi;
    const double al = S_.p_.alpha, g = S_.p_.gstrength, om = S_.c_.omega;  // omega_chem (evolves under SGLE)
    double sums[DS_N];
    for (int j = 0; j < DS_N; ++j) sums[j] = neumaier_sum(part.data() + j, nblk_x, 8);
    const double momx = 2.0 * al * sums[DS_MOMX] * dvol / area;
    const double momy = 2.0 * al * sums[DS_MOMY] * dvol / area;
    const double egrad = 2.0 * al * (al * sums[DS_GRAD2]) * dvol / area;
    const double echem = 2.0 * al * (om * sums[DS_RHO]) * dvol / area;
    const double eintr = 2.0 * al * (0.5 * g * sums[DS_EINT]) * dvol / area;
    const double eppot = 2.0 * al * sums[DS_EPOT] * dvol / area;
    const double norm = sums[DS_RHO] * dvol;
    scalars[0] = momx;
    scalars[1] = momy;
    scalars[2] = egrad;
    scalars[3] = echem;
    scalars[4] = eintr;
    scalars[5] = egrad + eintr;
    scalars[6] = norm;
    scalars[7] = eppot;
    scalars[8] = 0.0;
    scalars[9] = 0.0;
    if (S_.np_ > 0) {
      // particle energies (diagnostics.f90:209-239); gpdeltaE is only set once
      // a force evaluation ran (shortrange_repulsion), so the very first call
      // reports esrep = 0 like the reference.
      const int np = S_.np_;
      std::vector<double> pos(2 * (size_t)np), vel(2 * (size_t)np);
      if (cudaMemcpy(pos.data(), S_.ps_.pos, sizeof(double) * pos.size(), cudaMemcpyDeviceToHost) ||
          cudaMemcpy(vel.data(), S_.ps_.vel, sizeof(double) * vel.size(), cudaMemcpyDeviceToHost)) {
        set_error("vk_diagnostics: particle readback failed");
        return VK_E_CUDA;
      }
      const double fac = S_.rep_init_ ? S_.erep_factor_ : 0.0;
      double ek = 0.0, es = 0.0;
      for (int i = 0; i < np; ++i) {
        ek += vel[2 * i] * vel[2 * i] + vel[2 * i + 1] * vel[2 * i + 1];
        for (int j = 0; j < np; ++j) {
          if (i == j) continue;
          const double x = pos[2 * i] - pos[2 * j], y = pos[2 * i + 1] - pos[2 * j + 1];
          double den = 1.0;
          for (int k = 0; k < 6; ++k) den *= (-3.0 + std::cos(x) + std::cos(y));
          es += fac / den;
        }
      }
      scalars[8] = 0.5 * S_.p_.gp_mass_part * ek;
      scalars[9] = np == 1 ? 0.0 : 0.5 * es;
      S_.rep_init_ = true;
    }
    const int ns = S_.nshell_;
    for (int j = 0; j < 6; ++j)
      for (int m = 0; m <= ns; ++m) spec_out[(size_t)j * (ns + 1) + m] = (m < nsh_) ? sp[(size_t)j * nsh_ + m] : 0.0;
    if (nvort) {
      nvort[0] = cnt[0];
      nvort[1] = cnt[1];
    }
    return VK_OK;
  }
};

}  // namespace vk
