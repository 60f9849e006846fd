// vk_kernels.cuh -- fused row-pass kernels of the 2D GPE stepper (sm_103a).
//
// Every 2D transform is two row passes.  The "x pass" holds rows y of a
// physical-space field (x contiguous) and writes its x-spectrum TRANSPOSED,
// [kx][y]; the "y pass" holds rows kx of that (y contiguous) and finishes the
// 2D transform along y, so the Fourier state sits in the reference's
// transposed layout kpsi[kx][ky] (src/mod_fft.f90:143-146) and every pass
// reads contiguous rows.  The pointwise work of gpe_rhs / gpe_rk4 / ARGLE is
// fused into the passes:
//
//   X1  Ta[y][kx] --F^-1_x--> psi (stored)   rho=|psi|^2 --F_x (two real rows
//       per complex FFT)--> Tb[kx][y], kx in [0,K]
//   Y1  Tb --F_y--> 2/3 mask --F^-1_y--> Tc[y][kx], kx in [0,K]
//   X2  Tc --F^-1_x (two real rows per FFT)--> P_G rho;  N = g P_G rho psi
//       (+ V psi) --F_x--> Td[kx][y]
//   Y2  Td --F_y--> N^; RK4 stage / ARGLE update of kpsi, str1, str2;
//       kpsi_new --F^-1_y--> Ta[y][kx]
//
// K is the largest |k| kept by the 2/3 rule (k1^2+k2^2 < (Nx/3)^2); with the
// RK4 mask every column |kx| > K of kpsi, of the RHS and of Ta is zero, so
// the RK4 passes skip those rows (identical arithmetic on every kept mode).
#pragma once
#include <mutex>
#include <unordered_set>
#include "vk_fft.cuh"
#ifdef __CUDACC__
#include "vk_bulk.cuh"
#define VK_HAVE_BULK 1
#else
#define VK_HAVE_BULK 0  // host builds of the pass bodies: element-wise loads only
#endif

namespace vk {

// Opt in to more than 48 KB of shared memory per CTA when static + dynamic
// shared memory of `fn` needs it (once per kernel).
inline void ensure_smem_attr(const void* fn, size_t dyn_bytes) {
  static std::mutex mu;
  static std::unordered_set<const void*> done;
  std::lock_guard<std::mutex> g(mu);
  if (done.count(fn)) return;
  cudaFuncAttributes a;
  size_t stat = 0;
  if (cudaFuncGetAttributes(&a, fn) == cudaSuccess) stat = a.sharedSizeBytes;
  if (stat + dyn_bytes > 48 * 1024)
    cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(227 * 1024 - stat));
  done.insert(fn);
}


// Launch geometry.  x passes (rows y, GeoX) hold R >= 2 rows per CTA so two
// real rows can share one complex FFT; y passes (rows kx, GeoY) hold R rows.
// NT = R*L/16 threads: full-height transforms run radix-16 stages, the
// half-height paired transforms radix-8 stages on the same threads.  The
// FP32 x passes at L = 1024 use one warp per row (NT = 32 R) and the
// warp-per-row transform of vk_fft.cuh; the FP64 y passes at L = 1024 run
// four warps per row (8 points per thread); at L = 4096 the FP32 passes cap
// their registers for two (x) and three (y) CTAs per SM; the choice of
// geometry and of the transform per pass follows timings on GB300.
// MINB is the CTAs per SM the register budget is sized for.
template <typename T, int L> struct GeoX;
template <typename T, int L> struct GeoY;
#define VK_GEOE(KIND, TT, LL, RR, MB, EE)                                    \
  template <> struct KIND<TT, LL> {                                          \
    static constexpr int L = LL, R = RR, LP = padded(LL), MINB = MB;         \
    static constexpr int NT = RR * LL / EE;                                  \
  };
#define VK_GEO(KIND, TT, LL, RR, MB) VK_GEOE(KIND, TT, LL, RR, MB, 16)
VK_GEO(GeoX, double, 16, 16, 4) VK_GEO(GeoX, double, 32, 16, 4) VK_GEO(GeoX, double, 64, 16, 4)
VK_GEO(GeoX, double, 128, 8, 4) VK_GEO(GeoX, double, 256, 4, 4) VK_GEO(GeoX, double, 512, 2, 4)
VK_GEO(GeoX, double, 1024, 2, 4) VK_GEO(GeoX, double, 2048, 2, 2) VK_GEO(GeoX, double, 4096, 2, 1)
VK_GEO(GeoY, double, 16, 16, 4) VK_GEO(GeoY, double, 32, 8, 8) VK_GEO(GeoY, double, 64, 4, 8)
VK_GEO(GeoY, double, 128, 2, 8) VK_GEO(GeoY, double, 256, 1, 8) VK_GEO(GeoY, double, 512, 1, 8)
VK_GEOE(GeoY, double, 1024, 1, 5, 8) VK_GEO(GeoY, double, 2048, 1, 4) VK_GEO(GeoY, double, 4096, 1, 2)
VK_GEO(GeoX, float, 16, 16, 4) VK_GEO(GeoX, float, 32, 16, 4) VK_GEO(GeoX, float, 64, 16, 4)
VK_GEO(GeoX, float, 128, 8, 4) VK_GEO(GeoX, float, 256, 4, 4) VK_GEO(GeoX, float, 512, 2, 8)
VK_GEOE(GeoX, float, 1024, 4, 2, 32) VK_GEO(GeoX, float, 2048, 2, 2) VK_GEO(GeoX, float, 4096, 2, 2)
VK_GEO(GeoY, float, 16, 16, 4) VK_GEO(GeoY, float, 32, 8, 8) VK_GEO(GeoY, float, 64, 4, 8)
VK_GEO(GeoY, float, 128, 2, 8) VK_GEO(GeoY, float, 256, 1, 8) VK_GEO(GeoY, float, 512, 1, 8)
VK_GEO(GeoY, float, 1024, 1, 8) VK_GEO(GeoY, float, 2048, 1, 4) VK_GEO(GeoY, float, 4096, 1, 3)
#undef VK_GEO
#undef VK_GEOE

__device__ __forceinline__ int kwn(int i, int n) { return i < n / 2 ? i : i - n; }

// Row index of logical row l when only |kx| <= K rows are processed.
__device__ __forceinline__ int pruned_row(int l, int K, int n) { return l <= K ? l : n - (2 * K + 1 - l); }

// Stage NR rows of L values into shared memory (pitch LP, padded index):
// s[r][k] = fetch(r, k).  Every thread holds PER = NR*L/NT elements; the
// global loads of a batch are issued before any of them is stored, so a
// thread has up to 16 loads in flight instead of one load per round trip.
template <typename T, int L, int NR, int NT, int LP, class F>
__device__ __forceinline__ void stage_rows(cplx<T>* __restrict__ s, F fetch) {
  constexpr int PER = NR * L / NT;
  static_assert(NR * L % NT == 0, "threads tile the rows");
  // FP64 passes are DFMA-bound and short of registers: one element at a time
  constexpr int BMAX = sizeof(T) == 4 ? 16 : 1;
  constexpr int B = PER < BMAX ? PER : BMAX;
  constexpr int UNR = sizeof(T) == 4 ? PER / B : 1;
#pragma unroll UNR
  for (int q0 = 0; q0 < PER; q0 += B) {
    cplx<T> v[B];
#pragma unroll
    for (int j = 0; j < B; ++j) {
      const int e = threadIdx.x + (q0 + j) * NT;
      v[j] = fetch(e / L, e % L);
    }
#pragma unroll
    for (int j = 0; j < B; ++j) {
      const int e = threadIdx.x + (q0 + j) * NT;
      s[(e / L) * LP + pidx(e % L)] = v[j];
    }
  }
}

#if VK_HAVE_BULK
// FP64 row tiles by bulk copies (vk_bulk.cuh): rows r < nr of the tile come
// from row_of(r) (L contiguous values), rows nr <= r < NR are zeroed.  Every
// thread must call it; false: a wait ran out, the caller must return.
template <int L, int NR, int NT, int LP, class RowOf>
__device__ __forceinline__ bool bulk_rows(double2* __restrict__ s, RowOf row_of, int nr, int* err,
                                          unsigned long long limit) {
  __shared__ uint64_t bar;
  bulk_begin(&bar, (uint32_t)(nr * L * sizeof(double2)));
#pragma unroll 1
  for (int r = 0; r < NR; ++r) {
    if (r < nr) bulk_row_range<NT>(s + r * LP, row_of(r), 0, L, &bar);
    else
      for (int k = threadIdx.x; k < L; k += NT) s[r * LP + pidx(k)] = make_double2(0.0, 0.0);
  }
  return bulk_wait(&bar, err, limit);
}
#endif

// Scalars shared by the passes (by value in the launch).
struct StepConsts {
  int nx, ny;        // grid
  int K;             // max |k| kept by the 2/3 rule
  int k2max;         // largest kept k1^2+k2^2
  int pk;            // row pitch of Tc (>= K+1)
  // x passes: the last xsingle CTAs of k_x1/k_x2 take one row each (the
  // half-length real transforms) instead of R rows; 0 = row groups only.
  int xsingle;
  double alpha, g, omega, dt;
  double prefac_re, prefac_im;   // (1 - i*disp_factor)/i
  double scale;      // 1/(nx*ny)
  // Background density moved out of the FFTs: the passes transform
  // rho - rho_bg and add g*rho_bg back analytically in Fourier space
  // (g P_G rho psi = g P_G(rho - rho_bg) psi + g rho_bg psi, F[psi] = kpsi).
  // 0 on the plain FP64 path (the reference's arithmetic); Omega/g on the
  // FP32 path, where it removes the large cancelling g psi / Omega kpsi pair.
  double rho_bg;
  // -DGPE_FRCDISP (frc != 0): hypo/hyperviscosity and random-phase forcing
  // in the RK4 right-hand side; the phase counter lives on the device.
  int frc;
  double vishypo, vishype, famp, kf1sq, kf2sq;
  unsigned long long seed;
  const unsigned long long* rng_ctr;
  // -DGPE_SGLE: the chemical potential evolves on the device; noise
  // amplitude noisesigma/sqrt(dvol); -DGPE_SELFTRUNC cut k^2 > ktrunc^2.
  const double* omega_dev;
  double sgle_amp, sqrt_dt, ktrunc2;
  int selftrunc;
  // Bulk row loads (FP64): the error word a CTA sets when its bounded wait
  // for the row's copies runs out, and the poll limit.
  int* async_err;
  unsigned long long async_limit;
};

// Counter-based uniform [0,1) of the forcing phases (SplitMix64 finaliser of
// seed, RHS-evaluation counter and mode index); the oracle defines the same.
__host__ __device__ __forceinline__ unsigned long long vk_mix64(unsigned long long z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
__host__ __device__ __forceinline__ double vk_frc_uniform(unsigned long long seed, unsigned long long ctr,
                                                          unsigned long long mode) {
  return (double)(vk_mix64(vk_mix64(seed ^ (ctr * 0xD1B54A32D192ED03ull)) + mode) >> 11) *
         (1.0 / 9007199254740992.0);
}
// Standard normal pair of the SGLE noise at point idx: Box-Muller on two
// counter-based uniforms (the oracle defines the same).
__device__ __forceinline__ void vk_sgle_normals(unsigned long long seed, unsigned long long ctr,
                                                unsigned long long idx, double* v1, double* v2) {
  const double u1 = 1.0 - vk_frc_uniform(seed, ctr, 2 * idx), u2 = vk_frc_uniform(seed, ctr, 2 * idx + 1);
  const double r = sqrt(-2.0 * log(u1));
  double sn, cs;
  sincos(2.0 * 3.14159265358979323846 * u2, &sn, &cs);
  *v1 = r * cs;
  *v2 = r * sn;
}

// Device view of one field's buffers and constants (ensemble work items
// index an array of these).
template <typename T> struct Field {
  cplx<T>*psi, *kpsi, *str1, *str2, *Ta, *Tb, *Tc, *Td;
  const cplx<T>*twx, *twy;
  StepConsts c;
};

// ------------------------------------------------------------------------
// Generic passes (set_psi, readback, diagnostics helpers).
// ------------------------------------------------------------------------

// rows y of src[y][x] -> F_x -> dst[kx][y] (all kx).
template <typename T, int L>
__global__ void __launch_bounds__(GeoX<T, L>::NT, GeoX<T, L>::MINB) k_xfwd(const cplx<T>* __restrict__ src, cplx<T>* __restrict__ dst,
                                                     const cplx<T>* __restrict__ tw, int ny) {
  typedef GeoX<T, L> G;
  typedef cplx<T> C;
  extern __shared__ __align__(16) unsigned char smraw[];
  C* s = reinterpret_cast<C*>(smraw);
  const int y0 = blockIdx.x * G::R;
  stage_rows<T, L, G::R, G::NT, G::LP>(s, [&](int r, int x) { return src[(size_t)(y0 + r) * L + x]; });
  __syncthreads();
  fft_rows<T, L, G::R, G::NT, -1>(s, tw);
  for (int e = threadIdx.x; e < G::R * L; e += G::NT) {
    const int r = e % G::R, k = e / G::R;
    dst[(size_t)k * ny + y0 + r] = s[r * G::LP + pidx(k)];
  }
}

// rows kx of src[kx][y] -> F_y -> dst[kx][ky].  With MASKOUT the 2/3 mask
// (and an optional shell amplification, ic_OTOC_gpe) is applied on the way out.
template <typename T, int L, bool OTOC>
__global__ void __launch_bounds__(GeoY<T, L>::NT, GeoY<T, L>::MINB) k_yfwd(const cplx<T>* __restrict__ src, cplx<T>* __restrict__ dst,
                                                     const cplx<T>* __restrict__ tw, int nx, int k2max,
                                                     double k_otoc, double eps_otoc) {
  typedef GeoY<T, L> G;
  typedef cplx<T> C;
  extern __shared__ __align__(16) unsigned char smraw[];
  C* s = reinterpret_cast<C*>(smraw);
  const int x0 = blockIdx.x * G::R;
  stage_rows<T, L, G::R, G::NT, G::LP>(s, [&](int r, int y) { return src[(size_t)(x0 + r) * L + y]; });
  __syncthreads();
  fft_rows<T, L, G::R, G::NT, -1>(s, tw);
  for (int e = threadIdx.x; e < G::R * L; e += G::NT) {
    const int r = e / L, ky = e % L;
    C v = s[r * G::LP + pidx(ky)];
    if (OTOC) {
      const int k1 = kwn(x0 + r, nx), k2 = kwn(ky, L);
      const int ksq = k1 * k1 + k2 * k2;
      const double rk = sqrt((double)ksq);
      const int mshl = (int)llrint(rk);  // nint(rk): |rk| is never a half-integer
      if ((double)mshl == k_otoc) v = cscale(v, T(1.0 + eps_otoc));
      if (ksq > k2max) v = mkc<T>(T(0), T(0));
    }
    dst[(size_t)(x0 + r) * L + ky] = v;
  }
}

// rows kx of src[kx][ky] -> F^-1_y -> dst[y][kx] (pitch nx).  DERIV: of
// i*ky*src instead (the y-derivative, ARGLE flow terms).
template <typename T, int L, bool DERIV = false>
__global__ void __launch_bounds__(GeoY<T, L>::NT, GeoY<T, L>::MINB) k_yinv(const cplx<T>* __restrict__ src, cplx<T>* __restrict__ dst,
                                                     const cplx<T>* __restrict__ tw, int nx) {
  typedef GeoY<T, L> G;
  typedef cplx<T> C;
  extern __shared__ __align__(16) unsigned char smraw[];
  C* s = reinterpret_cast<C*>(smraw);
  const int x0 = blockIdx.x * G::R;
  stage_rows<T, L, G::R, G::NT, G::LP>(s, [&](int r, int y) {
    const C v = src[(size_t)(x0 + r) * L + y];
    if (!DERIV) return v;
    const T k = T(kwn(y, L));
    return mkc<T>(-k * v.y, k * v.x);
  });
  __syncthreads();
  fft_rows<T, L, G::R, G::NT, +1>(s, tw);
  for (int e = threadIdx.x; e < G::R * L; e += G::NT) {
    const int r = e % G::R, y = e / G::R;
    dst[(size_t)y * nx + x0 + r] = s[r * G::LP + pidx(y)];
  }
}

// rows y of src[y][kx] -> F^-1_x -> * scale -> dst[y][x].  With PRUNE only
// columns |kx| <= K are read (the rest are known zero).
template <typename T, int L, class G, bool PRUNE>
__device__ __forceinline__ void xinv_body(const cplx<T>* __restrict__ src, cplx<T>* __restrict__ dst,
                                                     const cplx<T>* __restrict__ tw, T scale, int K, const int tile, cplx<T>* __restrict__ s) {
  typedef cplx<T> C;
  const int y0 = tile * G::R;
  stage_rows<T, L, G::R, G::NT, G::LP>(s, [&](int r, int k) {
    C v = mkc<T>(T(0), T(0));
    if (!PRUNE || k <= K || k >= L - K) v = src[(size_t)(y0 + r) * L + k];
    return v;
  });
  __syncthreads();
  fft_rows<T, L, G::R, G::NT, +1>(s, tw);
  for (int e = threadIdx.x; e < G::R * L; e += G::NT) {
    const int r = e / L, x = e % L;
    dst[(size_t)(y0 + r) * L + x] = cscale(s[r * G::LP + pidx(x)], scale);
  }
}

template <typename T, int L, bool PRUNE>
__global__ void __launch_bounds__(GeoX<T, L>::NT, GeoX<T, L>::MINB) k_xinv(const cplx<T>* __restrict__ src, cplx<T>* __restrict__ dst,
                                                     const cplx<T>* __restrict__ tw, T scale, int K) {
  extern __shared__ __align__(16) unsigned char smraw[];
  xinv_body<T, L, GeoX<T, L>, PRUNE>(src, dst, tw, scale, K, blockIdx.x, reinterpret_cast<cplx<T>*>(smraw));
}

// Zero kpsi rows |kx| > K and in-row modes outside the 2/3 disk (the mask at
// the start of gpe_rk4, src/gpe.f90:338-355).
template <typename T>
__global__ void k_mask_four(cplx<T>* __restrict__ f, int nx, int ny, int k2max) {
  const size_t n = (size_t)nx * ny;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int kx = (int)(i / ny), ky = (int)(i % ny);
    const int k1 = kwn(kx, nx), k2 = kwn(ky, ny);
    if (k1 * k1 + k2 * k2 > k2max) f[i] = mkc<T>(T(0), T(0));
  }
}

// ------------------------------------------------------------------------
// X1: psi and the x-spectrum of rho = |psi|^2.
//   FROM_T: Ta[y][kx] --F^-1_x, *scale--> psi (written); else psi is read.
//   PRUNE : Ta columns |kx| > K are zero (RK4).
// Output Tb[kx][y] for kx in [0, K] (Hermitian half of the real rows).
// ------------------------------------------------------------------------
template <typename T, int L, class G, bool FROM_T, bool PRUNE>
__device__ __forceinline__ void x1_body(const cplx<T>* __restrict__ Ta, cplx<T>* __restrict__ psi,
                                                   cplx<T>* __restrict__ Tb, const cplx<T>* __restrict__ tw,
                                                   StepConsts c, const int tile, cplx<T>* __restrict__ s) {
  typedef cplx<T> C;
  const int y0 = tile * G::R;
  const int ny = c.ny, K = c.K;
  if (FROM_T) {
    stage_rows<T, L, G::R, G::NT, G::LP>(s, [&](int r, int k) {
      C v = mkc<T>(T(0), T(0));
      if (!PRUNE || k <= K || k >= L - K) v = Ta[(size_t)(y0 + r) * L + k];
      return v;
    });
    __syncthreads();
    fft_rows<T, L, G::R, G::NT, +1>(s, tw);
    const T scale = T(c.scale);
    for (int e = threadIdx.x; e < G::R * L; e += G::NT) {
      const int r = e / L, x = e % L;
      C v = cscale(s[r * G::LP + pidx(x)], scale);
      s[r * G::LP + pidx(x)] = v;
      psi[(size_t)(y0 + r) * L + x] = v;
    }
  } else {
    stage_rows<T, L, G::R, G::NT, G::LP>(s, [&](int r, int x) { return psi[(size_t)(y0 + r) * L + x]; });
  }
  __syncthreads();
  // rho for row pairs: z_p(x) = rho(x, y0+2p) + i rho(x, y0+2p+1), into row p.
  constexpr int NPAIR = G::R / 2;
  constexpr int PER = NPAIR * L / G::NT;
  static_assert(NPAIR * L % G::NT == 0, "pairing tile");
  C z[PER];
#pragma unroll
  for (int q = 0; q < PER; ++q) {
    const int e = threadIdx.x + q * G::NT;
    const int p = e / L, x = e % L;
    const C a = s[(2 * p) * G::LP + pidx(x)], b = s[(2 * p + 1) * G::LP + pidx(x)];
    const T bg = T(c.rho_bg);
    z[q] = mkc<T>(a.x * a.x + a.y * a.y - bg, b.x * b.x + b.y * b.y - bg);
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < PER; ++q) {
    const int e = threadIdx.x + q * G::NT;
    const int p = e / L, x = e % L;
    s[p * G::LP + pidx(x)] = z[q];
  }
  __syncthreads();
  fft_rows<T, L, NPAIR, G::NT, -1, G::NT>(s, tw);
  // unpack: A(k) = (Z(k) + conj Z(-k))/2, B(k) = -i (Z(k) - conj Z(-k))/2
  for (int e = threadIdx.x; e < G::R * (K + 1); e += G::NT) {
    const int r = e % G::R, k = e / G::R;
    const int p = r >> 1;
    const C zk = s[p * G::LP + pidx(k)];
    const C zm = s[p * G::LP + pidx((L - k) & (L - 1))];
    C v;
    if ((r & 1) == 0) v = mkc<T>(T(0.5) * (zk.x + zm.x), T(0.5) * (zk.y - zm.y));
    else v = mkc<T>(T(0.5) * (zk.y + zm.y), T(0.5) * (zm.x - zk.x));
    Tb[(size_t)k * ny + y0 + r] = v;
  }
}

// X1 on one row y (the tail CTAs of k_x1).  The real row rho runs as the
// L/2-point complex transform of z[n] = rho(2n) + i rho(2n+1) on the L-point
// twiddle table, and is unpacked with
//   E(k) = (Z(k) + conj Z(L/2-k))/2,  O(k) = -i (Z(k) - conj Z(L/2-k))/2,
//   rho^(k) = E(k) + W_L^k O(k),  k in [0, K] (K < L/2).
//   BULK (FP64): the row arrives by bulk copies (vk_bulk.cuh) instead of
//   element-wise loads; the pruned band K < k < L-K is zeroed in shared memory.
template <typename T, int L, class G, bool FROM_T, bool PRUNE, bool SPREAD = false, bool BULK = false>
__device__ __forceinline__ void x1_single_body(const cplx<T>* __restrict__ Ta, cplx<T>* __restrict__ psi,
                                               cplx<T>* __restrict__ Tb, const cplx<T>* __restrict__ tw,
                                               StepConsts c, const int y, cplx<T>* __restrict__ s) {
  typedef cplx<T> C;
  constexpr int H = L / 2;
  constexpr bool SP = SPREAD && H / G::NT >= 4;  // all threads in both transforms
  constexpr int NA = SP || G::NT < L / 16 ? G::NT : L / 16;  // threads of the L-point transform
  constexpr int NH = SP || G::NT < H / 8 ? G::NT : H / 8;    // threads of the L/2-point transform
  static_assert(!BULK || (VK_HAVE_BULK && sizeof(T) == 8), "bulk row loads: FP64 device code");
  const int ny = c.ny, K = c.K;
  if constexpr (BULK) {
#if VK_HAVE_BULK
    __shared__ uint64_t bar;
    const int kin = FROM_T && PRUNE ? K + 1 : L;  // copied: [0, kin) and, pruned, [L-K, L)
    bulk_begin(&bar, (uint32_t)((FROM_T && PRUNE ? 2 * K + 1 : L) * sizeof(C)));
    const C* row = (FROM_T ? Ta : psi) + (size_t)y * L;
    bulk_row_range<G::NT>(s, row, 0, kin, &bar);
    if (FROM_T && PRUNE) {
      bulk_row_range<G::NT>(s, row, L - K, L, &bar);
      for (int k = kin + threadIdx.x; k < L - K; k += G::NT) s[pidx(k)] = mkc<T>(T(0), T(0));
    }
    if (!bulk_wait(&bar, c.async_err, c.async_limit)) return;
#endif
  }
  if (FROM_T) {
    if constexpr (!BULK)
      stage_rows<T, L, 1, G::NT, G::LP>(s, [&](int, int k) {
        C v = mkc<T>(T(0), T(0));
        if (!PRUNE || k <= K || k >= L - K) v = Ta[(size_t)y * L + k];
        return v;
      });
    __syncthreads();
    fft_rows<T, L, 1, NA, +1, G::NT>(s, tw);
    const T scale = T(c.scale);
    for (int x = threadIdx.x; x < L; x += G::NT) {
      const C v = cscale(s[pidx(x)], scale);
      s[pidx(x)] = v;
      psi[(size_t)y * L + x] = v;
    }
  } else if constexpr (!BULK) {
    stage_rows<T, L, 1, G::NT, G::LP>(s, [&](int, int x) { return psi[(size_t)y * L + x]; });
  }
  __syncthreads();
  constexpr int PER = H / G::NT;
  static_assert(H % G::NT == 0, "half-row tile");
  C z[PER];
  const T bg = T(c.rho_bg);
#pragma unroll
  for (int q = 0; q < PER; ++q) {
    const int n = threadIdx.x + q * G::NT;
    const C a = s[pidx(2 * n)], b = s[pidx(2 * n + 1)];
    z[q] = mkc<T>(a.x * a.x + a.y * a.y - bg, b.x * b.x + b.y * b.y - bg);
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < PER; ++q) s[pidx(threadIdx.x + q * G::NT)] = z[q];
  __syncthreads();
  fft_rows<T, H, 1, NH, -1, G::NT, 2>(s, tw);
  for (int k = threadIdx.x; k <= K; k += G::NT) {
    const C zk = s[pidx(k)], zm = s[pidx((H - k) & (H - 1))];
    const T er = T(0.5) * (zk.x + zm.x), ei = T(0.5) * (zk.y - zm.y);
    const T o_r = T(0.5) * (zk.y + zm.y), o_i = T(0.5) * (zm.x - zk.x);
    const C w = __ldg(tw + k);
    Tb[(size_t)k * ny + y] = mkc<T>(er + (w.x * o_r - w.y * o_i), ei + (w.x * o_i + w.y * o_r));
  }
}

// BULK (FP64): the single-row CTAs load their row by bulk copies.
template <typename T, int L, bool FROM_T, bool PRUNE, bool BULK = false>
__global__ void __launch_bounds__(GeoX<T, L>::NT, GeoX<T, L>::MINB) k_x1(const cplx<T>* __restrict__ Ta, cplx<T>* __restrict__ psi,
                                                   cplx<T>* __restrict__ Tb, const cplx<T>* __restrict__ tw,
                                                   StepConsts c) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int npair = (int)gridDim.x - c.xsingle;
  if (L < 128 || (int)blockIdx.x < npair)
    x1_body<T, L, GeoX<T, L>, FROM_T, PRUNE>(Ta, psi, Tb, tw, c, blockIdx.x, reinterpret_cast<cplx<T>*>(smraw));
  else if constexpr (L >= 128)
    x1_single_body<T, L, GeoX<T, L>, FROM_T, PRUNE, false, BULK>(
        Ta, psi, Tb, tw, c, GeoX<T, L>::R * npair + ((int)blockIdx.x - npair), reinterpret_cast<cplx<T>*>(smraw));
}

// ------------------------------------------------------------------------
// Y1: rows kx in [0,K] of Tb: F_y, 2/3 mask, F^-1_y -> Tc[y][kx] (pitch pk).
// ------------------------------------------------------------------------
// BULK (FP64): the rows arrive by bulk copies (bulk_rows).
template <typename T, int L, class G, bool BULK = false>
__device__ __forceinline__ void y1_body(const cplx<T>* __restrict__ Tb, cplx<T>* __restrict__ Tc,
                                                   const cplx<T>* __restrict__ tw, StepConsts c, const int tile, cplx<T>* __restrict__ s) {
  typedef cplx<T> C;
  static_assert(!BULK || (VK_HAVE_BULK && sizeof(T) == 8), "bulk row loads: FP64 device code");
  const int l0 = tile * G::R;
  const int K = c.K;
  if constexpr (BULK) {
#if VK_HAVE_BULK
    const int nr = min(G::R, K + 1 - l0);
    if (!bulk_rows<L, G::R, G::NT, G::LP>(s, [&](int r) { return Tb + (size_t)(l0 + r) * L; }, nr, c.async_err,
                                         c.async_limit))
      return;
#endif
  } else {
    stage_rows<T, L, G::R, G::NT, G::LP>(s, [&](int r, int y) {
      C v = mkc<T>(T(0), T(0));
      if (l0 + r <= K) v = Tb[(size_t)(l0 + r) * L + y];
      return v;
    });
  }
  __syncthreads();
  fft_rows<T, L, G::R, G::NT, -1>(s, tw);
  for (int e = threadIdx.x; e < G::R * L; e += G::NT) {
    const int r = e / L, ky = e % L;
    const int k1 = l0 + r, k2 = kwn(ky, L);
    if (k1 * k1 + k2 * k2 > c.k2max) s[r * G::LP + pidx(ky)] = mkc<T>(T(0), T(0));
  }
  __syncthreads();
  fft_rows<T, L, G::R, G::NT, +1>(s, tw);
  for (int e = threadIdx.x; e < G::R * L; e += G::NT) {
    const int r = e % G::R, y = e / G::R;
    if (l0 + r <= K) Tc[(size_t)y * c.pk + l0 + r] = s[r * G::LP + pidx(y)];
  }
}

template <typename T, int L, bool BULK = false>
__global__ void __launch_bounds__(GeoY<T, L>::NT, GeoY<T, L>::MINB) k_y1(const cplx<T>* __restrict__ Tb, cplx<T>* __restrict__ Tc,
                                                   const cplx<T>* __restrict__ tw, StepConsts c) {
  extern __shared__ __align__(16) unsigned char smraw[];
  y1_body<T, L, GeoY<T, L>, BULK>(Tb, Tc, tw, c, blockIdx.x, reinterpret_cast<cplx<T>*>(smraw));
}

// ------------------------------------------------------------------------
// X2: rows y of Tc (kx in [0,K]) -> P_G rho (real, two rows per complex
// F^-1_x) -> N = SIGN*g*P_G rho*psi [+ SIGN*V*psi] -> F_x -> Td[kx][y].
// SIGN = +1 for gpe_rhs (src/gpe.f90:583-594), -1 for ARGLE (:101-112).
// PRUNE_OUT: only |kx| <= K columns of Td are written (RK4).
// ------------------------------------------------------------------------
template <typename T, int L, class G, int SIGN, bool PRUNE_OUT, bool POT>
__device__ __forceinline__ void x2_body(const cplx<T>* __restrict__ Tc, const cplx<T>* __restrict__ psi,
                                                   const T* __restrict__ vpot, cplx<T>* __restrict__ Td,
                                                   const cplx<T>* __restrict__ tw, StepConsts c, const int tile, cplx<T>* __restrict__ s) {
  typedef cplx<T> C;
  const int y0 = tile * G::R;
  const int K = c.K, ny = c.ny, pk = c.pk;
  constexpr int NPAIR = G::R / 2;
  // Z_p(k) = A(k) + i B(k) with the Hermitian extension to negative k.
  stage_rows<T, L, NPAIR, G::NT, G::LP>(s, [&](int p, int k) {
    C v = mkc<T>(T(0), T(0));
    const size_t ra = (size_t)(y0 + 2 * p) * pk, rb = ra + pk;
    if (k <= K) {
      const C a = Tc[ra + k], b = Tc[rb + k];
      v = mkc<T>(a.x - b.y, a.y + b.x);
    } else if (k >= L - K) {
      const C a = Tc[ra + (L - k)], b = Tc[rb + (L - k)];
      // conj(a) + i conj(b)
      v = mkc<T>(a.x + b.y, b.x - a.y);
    }
    return v;
  });
  __syncthreads();
  fft_rows<T, L, NPAIR, G::NT, +1, G::NT>(s, tw);
  constexpr int PER = G::R * L / G::NT;
  C nv[PER];
  const T gsc = T(SIGN * c.g * c.scale);  // g and the 1/(nx ny) of the inverse transform
#pragma unroll
  for (int q = 0; q < PER; ++q) {
    const int e = threadIdx.x + q * G::NT;
    const int r = e / L, x = e % L;
    const C z = s[(r >> 1) * G::LP + pidx(x)];
    const C ps = psi[(size_t)(y0 + r) * L + x];
    const T gp = gsc * ((r & 1) == 0 ? z.x : z.y);  // SIGN g P_G[|psi|^2](x, y0+r)
    C n = mkc<T>(gp * ps.x, gp * ps.y);
    if (POT) {
      const T v = T(SIGN) * vpot[(size_t)(y0 + r) * L + x];
      n.x += v * ps.x;
      n.y += v * ps.y;
    }
    nv[q] = n;
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < PER; ++q) {
    const int e = threadIdx.x + q * G::NT;
    const int r = e / L, x = e % L;
    s[r * G::LP + pidx(x)] = nv[q];
  }
  __syncthreads();
  fft_rows<T, L, G::R, G::NT, -1>(s, tw);
  if (PRUNE_OUT) {
    const int ncol = 2 * K + 1;
    for (int e = threadIdx.x; e < G::R * ncol; e += G::NT) {
      const int r = e % G::R, l = e / G::R;
      const int k = pruned_row(l, K, L);
      Td[(size_t)k * ny + y0 + r] = s[r * G::LP + pidx(k)];
    }
  } else {
    for (int e = threadIdx.x; e < G::R * L; e += G::NT) {
      const int r = e % G::R, k = e / G::R;
      Td[(size_t)k * ny + y0 + r] = s[r * G::LP + pidx(k)];
    }
  }
}

// X2 on one row y (the tail CTAs of k_x2).  The Hermitian row A(k) of Tc
// (A(k) = conj A(L-k), zero for K < k < L-K) is inverted as one L/2-point
// complex transform: with
//   Z(k) = A(k) + conj A(L/2-k) + i (A(k) - conj A(L/2-k)) W_L^-k,
// k in [0, L/2), F^-1 Z (n) = P_G rho(2n) + i P_G rho(2n+1).
template <typename T, int L, class G, int SIGN, bool PRUNE_OUT, bool POT, bool SPREAD = false>
__device__ __forceinline__ void x2_single_body(const cplx<T>* __restrict__ Tc, const cplx<T>* __restrict__ psi,
                                               const T* __restrict__ vpot, cplx<T>* __restrict__ Td,
                                               const cplx<T>* __restrict__ tw, StepConsts c, const int y,
                                               cplx<T>* __restrict__ s) {
  typedef cplx<T> C;
  constexpr int H = L / 2;
  constexpr bool SP = SPREAD && H / G::NT >= 4;
  constexpr int NA = SP || G::NT < L / 16 ? G::NT : L / 16;
  constexpr int NH = SP || G::NT < H / 8 ? G::NT : H / 8;
  const int K = c.K, ny = c.ny;
  const C* row = Tc + (size_t)y * c.pk;
  stage_rows<T, H, 1, G::NT, padded(H)>(s, [&](int, int k) {
    const int m = H - k;
    const C a = k <= K ? row[k] : mkc<T>(T(0), T(0));
    const C b = m <= K ? row[m] : mkc<T>(T(0), T(0));
    const T er = a.x + b.x, ei = a.y - b.y;  // a + conj b
    const T dr = a.x - b.x, di = a.y + b.y;  // a - conj b
    const C w = __ldg(tw + k);               // W_L^k; W_L^-k = conj
    const T o_r = dr * w.x + di * w.y, o_i = di * w.x - dr * w.y;
    return mkc<T>(er - o_i, ei + o_r);
  });
  __syncthreads();
  fft_rows<T, H, 1, NH, +1, G::NT, 2>(s, tw);
  constexpr int PER = L / G::NT;
  C nv[PER];
  const T gsc = T(SIGN * c.g * c.scale);  // g and the 1/(nx ny) of the inverse transform
#pragma unroll
  for (int q = 0; q < PER; ++q) {
    const int x = threadIdx.x + q * G::NT;
    const C z = s[pidx(x >> 1)];
    const C ps = psi[(size_t)y * L + x];
    const T gp = gsc * ((x & 1) == 0 ? z.x : z.y);  // SIGN g P_G[|psi|^2](x, y)
    C n = mkc<T>(gp * ps.x, gp * ps.y);
    if (POT) {
      const T v = T(SIGN) * vpot[(size_t)y * L + x];
      n.x += v * ps.x;
      n.y += v * ps.y;
    }
    nv[q] = n;
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < PER; ++q) s[pidx(threadIdx.x + q * G::NT)] = nv[q];
  __syncthreads();
  fft_rows<T, L, 1, NA, -1, G::NT>(s, tw);
  if (PRUNE_OUT) {
    for (int l = threadIdx.x; l < 2 * K + 1; l += G::NT) {
      const int k = pruned_row(l, K, L);
      Td[(size_t)k * ny + y] = s[pidx(k)];
    }
  } else {
    for (int k = threadIdx.x; k < L; k += G::NT) Td[(size_t)k * ny + y] = s[pidx(k)];
  }
}

template <typename T, int L, int SIGN, bool PRUNE_OUT, bool POT>
__global__ void __launch_bounds__(GeoX<T, L>::NT, GeoX<T, L>::MINB) k_x2(const cplx<T>* __restrict__ Tc, const cplx<T>* __restrict__ psi,
                                                   const T* __restrict__ vpot, cplx<T>* __restrict__ Td,
                                                   const cplx<T>* __restrict__ tw, StepConsts c) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int npair = (int)gridDim.x - c.xsingle;
  if (L < 128 || (int)blockIdx.x < npair)
    x2_body<T, L, GeoX<T, L>, SIGN, PRUNE_OUT, POT>(Tc, psi, vpot, Td, tw, c, blockIdx.x, reinterpret_cast<cplx<T>*>(smraw));
  else if constexpr (L >= 128)  // all threads in both transforms: measured faster for x2, not for x1
    x2_single_body<T, L, GeoX<T, L>, SIGN, PRUNE_OUT, POT, true>(Tc, psi, vpot, Td, tw, c,
                                                           GeoX<T, L>::R * npair + ((int)blockIdx.x - npair),
                                                           reinterpret_cast<cplx<T>*>(smraw));
}

// Stage coefficients with the reference's evaluation order
// (dt*oney6, dt*oney6*two, dt*half, dt) and the RHS constants.
template <typename T> struct Rk4Coef { T c1, c2, pr, pi, al, omb; };
template <typename T, int STAGE>
__device__ __forceinline__ Rk4Coef<T> rk4_coef(const StepConsts& c) {
  const double oney6 = 1.0 / 6.0;
  Rk4Coef<T> q;
  q.c2 = T((STAGE == 1 || STAGE == 4) ? c.dt * oney6 : c.dt * oney6 * 2.0);
  q.c1 = T(STAGE == 3 ? c.dt : c.dt * 0.5);
  q.pr = T(c.prefac_re);
  q.pi = T(c.prefac_im);
  q.al = T(c.alpha);
  q.omb = T(c.omega) - T(c.g * c.rho_bg);
  return q;
}

// One Fourier mode of an RK4 stage: rhs = prefac*((alpha k^2 - Omega) kpsi
// + N^) on the 2/3 disk (src/gpe.f90:609-669; FRC adds :623-658), the stage
// update of src/gpe.f90:366-489 (str1 / str2 written at gi); returns the new
// kpsi, 0 off the disk.
template <typename T, int STAGE, bool FRC>
__device__ __forceinline__ cplx<T> rk4_mode(const StepConsts& c, const Rk4Coef<T>& q, int ksq, size_t gi, cplx<T> nh,
                                            cplx<T> ps, cplx<T> s1v, cplx<T> s2v, cplx<T>* __restrict__ str1,
                                            cplx<T>* __restrict__ str2, unsigned long long rctr) {
  typedef cplx<T> C;
  C nw = mkc<T>(T(0), T(0));
  if (ksq <= c.k2max) {
    const T kin = q.al * T(ksq) - q.omb;
    const C t = mkc<T>(kin * ps.x + nh.x, kin * ps.y + nh.y);
    C rhs = mkc<T>(q.pr * t.x - q.pi * t.y, q.pr * t.y + q.pi * t.x);
    if (FRC) {  // src/gpe.f90:623-658, in the reference's order
      const double kr2 = (double)ksq;
      const double x2 = kr2 * kr2, x4 = x2 * x2, x8 = x4 * x4;  // kradius2**8
      if (ksq != 0) {
        const T a = T(c.vishypo * (1.0 / x8));
        rhs = mkc<T>(rhs.x - a * ps.x, rhs.y - a * ps.y);
      }
      const T b = T(c.vishype * x8);
      rhs = mkc<T>(rhs.x - b * ps.x, rhs.y - b * ps.y);
      if (kr2 >= c.kf1sq && kr2 <= c.kf2sq) {
        double sn, cs;
        sincos(2.0 * 3.14159265358979323846 * vk_frc_uniform(c.seed, rctr, gi), &sn, &cs);
        rhs = mkc<T>(rhs.x + T(c.famp * cs), rhs.y + T(c.famp * sn));
      }
    }
    if (STAGE == 1) {
      str1[gi] = ps;
      str2[gi] = mkc<T>(q.c2 * rhs.x, q.c2 * rhs.y);
      nw = mkc<T>(ps.x + q.c1 * rhs.x, ps.y + q.c1 * rhs.y);
    } else {
      const C s2 = mkc<T>(s2v.x + q.c2 * rhs.x, s2v.y + q.c2 * rhs.y);
      if (STAGE < 4) {
        str2[gi] = s2;
        nw = mkc<T>(s1v.x + q.c1 * rhs.x, s1v.y + q.c1 * rhs.y);
      } else {
        nw = mkc<T>(s1v.x + s2.x, s1v.y + s2.y);
      }
    }
  }
  return nw;
}

// ------------------------------------------------------------------------
// Y2 (RK4 stage STAGE = 1..4): rows |kx| <= K of Td: F_y -> N^ ->
// rhs = prefac*((alpha k^2 - Omega) kpsi + N^), masked (src/gpe.f90:609-669)
// then the stage update of src/gpe.f90:366-489; kpsi_new --F^-1_y--> Ta.
// FRC: the -DGPE_FRCDISP terms (a separate instantiation, so the plain
// kernel carries none of their registers).
// ------------------------------------------------------------------------
template <typename T, int L, class G, int STAGE, bool FRC = false, bool BULK = false>
__device__ __forceinline__ void y2_rk4_body(const cplx<T>* __restrict__ Td, cplx<T>* __restrict__ kpsi,
                                                       cplx<T>* __restrict__ str1, cplx<T>* __restrict__ str2,
                                                       cplx<T>* __restrict__ Ta, const cplx<T>* __restrict__ tw,
                                                       StepConsts c, const int tile, cplx<T>* __restrict__ s) {
  typedef cplx<T> C;
  static_assert(!BULK || (VK_HAVE_BULK && sizeof(T) == 8), "bulk row loads: FP64 device code");
  const int l0 = tile * G::R;
  const int K = c.K, nx = c.nx;
  const int nrow = 2 * K + 1;
  if constexpr (BULK) {
#if VK_HAVE_BULK
    const int nr = min(G::R, nrow - l0);
    if (!bulk_rows<L, G::R, G::NT, G::LP>(
            s, [&](int r) { return Td + (size_t)pruned_row(l0 + r, K, nx) * L; }, nr, c.async_err, c.async_limit))
      return;
#endif
  } else {
    stage_rows<T, L, G::R, G::NT, G::LP>(s, [&](int r, int y) {
      C v = mkc<T>(T(0), T(0));
      if (l0 + r < nrow) v = Td[(size_t)pruned_row(l0 + r, K, nx) * L + y];
      return v;
    });
  }
  __syncthreads();
  fft_rows<T, L, G::R, G::NT, -1>(s, tw);
  const Rk4Coef<T> q = rk4_coef<T, STAGE>(c);
  const unsigned long long rctr = FRC ? *c.rng_ctr : 0ull;
  // batches of B elements per thread: all loads of a batch before any use
  constexpr int PER = G::R * L / G::NT;
  constexpr int B = sizeof(T) == 4 ? (PER < 8 ? PER : 8) : 1;
  constexpr int UNR = sizeof(T) == 4 ? PER / B : 1;
#pragma unroll UNR
  for (int q0 = 0; q0 < PER; q0 += B) {
    C ps[B], s1v[B], s2v[B];
#pragma unroll
    for (int j = 0; j < B; ++j) {
      const int e = threadIdx.x + (q0 + j) * G::NT;
      const int r = e / L, ky = e % L;
      const bool act = l0 + r < nrow;
      const size_t gi = act ? (size_t)pruned_row(l0 + r, K, nx) * L + ky : 0;
      ps[j] = act ? kpsi[gi] : mkc<T>(T(0), T(0));
      if (STAGE > 1) {
        s1v[j] = act ? str1[gi] : mkc<T>(T(0), T(0));
        s2v[j] = act ? str2[gi] : mkc<T>(T(0), T(0));
      }
    }
#pragma unroll
    for (int j = 0; j < B; ++j) {
      const int e = threadIdx.x + (q0 + j) * G::NT;
      const int r = e / L, ky = e % L;
      if (l0 + r >= nrow) continue;
      const int kxi = pruned_row(l0 + r, K, nx);
      const int k1 = kwn(kxi, nx), k2 = kwn(ky, L);
      const size_t gi = (size_t)kxi * L + ky;
      const C nw = rk4_mode<T, STAGE, FRC>(c, q, k1 * k1 + k2 * k2, gi, s[r * G::LP + pidx(ky)], ps[j], s1v[j], s2v[j],
                                           str1, str2, rctr);
      kpsi[gi] = nw;
      s[r * G::LP + pidx(ky)] = nw;
    }
  }
  __syncthreads();
  fft_rows<T, L, G::R, G::NT, +1>(s, tw);
  for (int e = threadIdx.x; e < G::R * L; e += G::NT) {
    const int r = e % G::R, y = e / G::R;
    if (l0 + r < nrow) Ta[(size_t)y * nx + pruned_row(l0 + r, K, nx)] = s[r * G::LP + pidx(y)];
  }
}

template <typename T, int L, int STAGE, bool FRC = false, bool BULK = false>
__global__ void __launch_bounds__(GeoY<T, L>::NT, GeoY<T, L>::MINB) k_y2_rk4(const cplx<T>* __restrict__ Td, cplx<T>* __restrict__ kpsi,
                                                       cplx<T>* __restrict__ str1, cplx<T>* __restrict__ str2,
                                                       cplx<T>* __restrict__ Ta, const cplx<T>* __restrict__ tw,
                                                       StepConsts c) {
  extern __shared__ __align__(16) unsigned char smraw[];
  y2_rk4_body<T, L, GeoY<T, L>, STAGE, FRC, BULK>(Td, kpsi, str1, str2, Ta, tw, c, blockIdx.x,
                                                  reinterpret_cast<cplx<T>*>(smraw));
}

// ------------------------------------------------------------------------
// Y2 (ARGLE, src/gpe.f90:181-222, no mask): all rows kx of Td: F_y -> N^,
// kpsi <- (kpsi + dt (N^ + Omega kpsi)) / (1 + alpha k^2 dt);
// kpsi_new --F^-1_y--> Ta.  RESID: per-CTA FP64 partial sums of
// |new-old|^2, |old|^2, |new|^2 into part[blockIdx][3].
// ------------------------------------------------------------------------
template <typename T, int L, class G, bool RESID, bool DERIV = false, bool SGLE = false>
__device__ __forceinline__ void y2_argle_body(const cplx<T>* __restrict__ Td, cplx<T>* __restrict__ kpsi,
                                                         cplx<T>* __restrict__ Ta, const cplx<T>* __restrict__ tw,
                                                         double* __restrict__ part, StepConsts c, const int tile, cplx<T>* __restrict__ s,
                                                         cplx<T>* __restrict__ Tg = nullptr,
                                                         const cplx<T>* __restrict__ Tn = nullptr) {
  typedef cplx<T> C;
  static_assert(G::NT <= 512, "reduction buffer");
  __shared__ double red[3][512];
  const int x0 = tile * G::R;
  const int nx = c.nx;
  stage_rows<T, L, G::R, G::NT, G::LP>(s, [&](int r, int y) { return Td[(size_t)(x0 + r) * L + y]; });
  // SGLE: the x-spectrum of the noise, rows kx, in the second R rows (the
  // derivative rows of DERIV reuse them: each slot is read, then written, by
  // the same thread)
  cplx<T>* sn = s + G::R * G::LP;
  if (SGLE) stage_rows<T, L, G::R, G::NT, G::LP>(sn, [&](int r, int y) { return Tn[(size_t)(x0 + r) * L + y]; });
  __syncthreads();
  fft_rows<T, L, G::R, G::NT, -1>(s, tw);
  if (SGLE) fft_rows<T, L, G::R, G::NT, -1>(sn, tw);
  const T al = T(c.alpha), om = T(SGLE ? *c.omega_dev : c.omega), dt = T(c.dt);
  double dsum = 0.0, osum = 0.0, nsum = 0.0;
  constexpr int PER = G::R * L / G::NT;
  constexpr int B = sizeof(T) == 4 ? (PER < 8 ? PER : 8) : 1;
#pragma unroll 1
  for (int q0 = 0; q0 < PER; q0 += B) {
  C oldv[B];
#pragma unroll
  for (int j = 0; j < B; ++j) {
    const int e = threadIdx.x + (q0 + j) * G::NT;
    oldv[j] = kpsi[(size_t)(x0 + e / L) * L + e % L];
  }
#pragma unroll
  for (int j = 0; j < B; ++j) {
    const int e = threadIdx.x + (q0 + j) * G::NT;
    const int r = e / L, ky = e % L;
    const int k1 = kwn(x0 + r, nx), k2 = kwn(ky, L);
    const size_t gi = (size_t)(x0 + r) * L + ky;
    const C old = oldv[j];
    const C nh = s[r * G::LP + pidx(ky)];
    const T omb = om - T(c.g * c.rho_bg);
    const C t1 = mkc<T>(nh.x + omb * old.x, nh.y + omb * old.y);
    const T t2 = T(1) + al * T(k1 * k1 + k2 * k2) * dt;
    C nw = mkc<T>(old.x + dt * t1.x, old.y + dt * t1.y);
    if (SGLE && k1 * k1 + k2 * k2 <= c.k2max) {  // noise_term = F[noise] sqrt(dt), masked (:199-209)
      const C z = sn[r * G::LP + pidx(ky)];
      const T sd = T(c.sqrt_dt);
      nw = mkc<T>(nw.x + sd * z.x, nw.y + sd * z.y);
    }
    nw.x = nw.x / t2;
    nw.y = nw.y / t2;
    if (SGLE && c.selftrunc && (double)(k1 * k1 + k2 * k2) > c.ktrunc2) nw = mkc<T>(T(0), T(0));  // :213-217
    kpsi[gi] = nw;
    s[r * G::LP + pidx(ky)] = nw;
    if (DERIV) s[(G::R + r) * G::LP + pidx(ky)] = mkc<T>(-T(k2) * nw.y, T(k2) * nw.x);  // i ky kpsi
    if (RESID) {
      const double dx = (double)nw.x - (double)old.x, dy = (double)nw.y - (double)old.y;
      dsum += dx * dx + dy * dy;
      osum += (double)old.x * old.x + (double)old.y * old.y;
      nsum += (double)nw.x * nw.x + (double)nw.y * nw.y;
    }
  }
  }
  if (RESID) {
    red[0][threadIdx.x] = dsum;
    red[1][threadIdx.x] = osum;
    red[2][threadIdx.x] = nsum;
  }
  __syncthreads();
  if (RESID && threadIdx.x == 0) {  // fixed order: deterministic
    double a = 0, b = 0, d = 0;
    for (int t = 0; t < G::NT; ++t) { a += red[0][t]; b += red[1][t]; d += red[2][t]; }
    part[tile * 3 + 0] = a;
    part[tile * 3 + 1] = b;
    part[tile * 3 + 2] = d;
  }
  fft_rows<T, L, G::R, G::NT, +1>(s, tw);
  if (DERIV) fft_rows<T, L, G::R, G::NT, +1>(s + G::R * G::LP, tw);
  for (int e = threadIdx.x; e < G::R * L; e += G::NT) {
    const int r = e % G::R, y = e / G::R;
    Ta[(size_t)y * nx + x0 + r] = s[r * G::LP + pidx(y)];
    if (DERIV) Tg[(size_t)y * nx + x0 + r] = s[(G::R + r) * G::LP + pidx(y)];
  }
}

// The flow and noise variants hold two rows per CTA: at most four CTAs per
// SM, so that they keep 128 registers a thread.
template <typename T, int L, bool RESID, bool DERIV = false, bool SGLE = false>
__global__ void __launch_bounds__(GeoY<T, L>::NT, (DERIV || SGLE) && GeoY<T, L>::MINB > 4 ? 4 : GeoY<T, L>::MINB) k_y2_argle(const cplx<T>* __restrict__ Td, cplx<T>* __restrict__ kpsi,
                                                         cplx<T>* __restrict__ Ta, const cplx<T>* __restrict__ tw,
                                                         double* __restrict__ part, StepConsts c,
                                                         cplx<T>* __restrict__ Tg = nullptr,
                                                         const cplx<T>* __restrict__ Tn = nullptr) {
  extern __shared__ __align__(16) unsigned char smraw[];
  y2_argle_body<T, L, GeoY<T, L>, RESID, DERIV, SGLE>(Td, kpsi, Ta, tw, part, c, blockIdx.x,
                                                      reinterpret_cast<cplx<T>*>(smraw), Tg, Tn);
}

// SGLE noise (src/gpe.f90:149-165): rows y, noise(x, y) = (v1 + i v2)
// noisesigma/sqrt(dvol) from the counter-based normals of point y*nx + x,
// F_x -> Tn[kx][y] (all kx).
template <typename T, int L>
__global__ void __launch_bounds__(GeoX<T, L>::NT, GeoX<T, L>::MINB) k_noise_x(cplx<T>* __restrict__ Tn,
                                                             const cplx<T>* __restrict__ tw, StepConsts c) {
  typedef GeoX<T, L> G;
  typedef cplx<T> C;
  extern __shared__ __align__(16) unsigned char smraw[];
  C* s = reinterpret_cast<C*>(smraw);
  const int y0 = blockIdx.x * G::R;
  const unsigned long long ctr = *c.rng_ctr;
  for (int e = threadIdx.x; e < G::R * L; e += G::NT) {
    const int r = e / L, x = e % L;
    double v1, v2;
    vk_sgle_normals(c.seed, ctr, (unsigned long long)(y0 + r) * L + x, &v1, &v2);
    s[r * G::LP + pidx(x)] = mkc<T>(T(v1 * c.sgle_amp), T(v2 * c.sgle_amp));
  }
  __syncthreads();
  fft_rows<T, L, G::R, G::NT, -1>(s, tw);
  for (int e = threadIdx.x; e < G::R * L; e += G::NT) {
    const int r = e % G::R, k = e / G::R;
    Tn[(size_t)k * c.ny + y0 + r] = s[r * G::LP + pidx(k)];
  }
}

// Per-block sums of |psi|^2 (Fortran ABS squared), fixed order.
template <typename T>
__global__ void k_sum_abs2(const cplx<T>* __restrict__ psi, size_t n, double* __restrict__ part) {
  __shared__ double sh[256];
  double a = 0.0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const double h = hypot((double)psi[i].x, (double)psi[i].y);
    a += h * h;
  }
  sh[threadIdx.x] = a;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

// finiteT_adhoc_chempot (src/gpe.f90:226-264): omega -= dt nuN/(Lx Ly)
// (norm - Nparticle), norm = dvol sum |psi|^2.  One thread.
__global__ void k_chempot(const double* __restrict__ part, int nblk, double* __restrict__ omega, double dt,
                          double nun_area, double dvol, double nparticle);

// ------------------------------------------------------------------------
// X2 for ARGLE with the flow terms of src/gpe.f90:78-146: rows y of
// Tc -> P_G rho (two real rows per F^-1_x); rows of i*kx*Ta and of Tg
// (= F^-1_y[i ky kpsi]) -> F^-1_x -> grad psi; N = -g P_G rho psi plus
//   FLOW 1 (-DGPE_ADVECTION): -i(u.grad psi) - (1/4)(1/alpha)|u|^2 psi,
//          u = (sin x cos y, -cos x sin y) at x = i1 dx, y = i2 dy;
//   FLOW 2 (-DGPE_COUNTERFLOW): -i(v.grad psi), v = (vnx, vny);
// then F_x -> Td[kx][y] (all kx).  Shared memory: 3 R rows.
// ------------------------------------------------------------------------
template <typename T, int L, int FLOW>
__global__ void __launch_bounds__(GeoX<T, L>::NT, 1) k_x2_flow(const cplx<T>* __restrict__ Tc, const cplx<T>* __restrict__ psi,
                                                             const cplx<T>* __restrict__ Ta, const cplx<T>* __restrict__ Tg,
                                                             cplx<T>* __restrict__ Td, const cplx<T>* __restrict__ tw,
                                                             StepConsts c, double vnx, double vny) {
  typedef GeoX<T, L> G;
  typedef cplx<T> C;
  extern __shared__ __align__(16) unsigned char smraw[];
  C* s = reinterpret_cast<C*>(smraw);
  C* sg = s + G::R * G::LP;  // rows [0,R): d/dx psi, [R,2R): d/dy psi
  const int y0 = blockIdx.x * G::R;
  const int K = c.K, ny = c.ny, pk = c.pk;
  constexpr int NPAIR = G::R / 2;
  stage_rows<T, L, NPAIR, G::NT, G::LP>(s, [&](int p, int k) {
    C v = mkc<T>(T(0), T(0));
    const size_t ra = (size_t)(y0 + 2 * p) * pk, rb = ra + pk;
    if (k <= K) {
      const C a = Tc[ra + k], b = Tc[rb + k];
      v = mkc<T>(a.x - b.y, a.y + b.x);
    } else if (k >= L - K) {
      const C a = Tc[ra + (L - k)], b = Tc[rb + (L - k)];
      v = mkc<T>(a.x + b.y, b.x - a.y);
    }
    return v;
  });
  stage_rows<T, L, 2 * G::R, G::NT, G::LP>(sg, [&](int r, int k) {
    if (r < G::R) {
      const C v = Ta[(size_t)(y0 + r) * L + k];
      const T kx = T(kwn(k, L));
      return mkc<T>(-kx * v.y, kx * v.x);
    }
    return Tg[(size_t)(y0 + r - G::R) * L + k];
  });
  __syncthreads();
  fft_rows<T, L, NPAIR, G::NT, +1, G::NT>(s, tw);
  fft_rows<T, L, 2 * G::R, G::NT, +1>(sg, tw);
  constexpr int PER = G::R * L / G::NT;
  C nv[PER];
  const T gs = T(-c.g);
  const T scale = T(c.scale);
  const double two_pi = 6.283185307179586476925286766559;
  const double dx = two_pi / L, dy = two_pi / ny;
#pragma unroll
  for (int q = 0; q < PER; ++q) {
    const int e = threadIdx.x + q * G::NT;
    const int r = e / L, x = e % L;
    const C z = s[(r >> 1) * G::LP + pidx(x)];
    const T pg = ((r & 1) == 0 ? z.x : z.y) * scale;
    const C ps = psi[(size_t)(y0 + r) * L + x];
    const T gp = gs * pg;
    C n = mkc<T>(gp * ps.x, gp * ps.y);
    const C a1 = cscale(sg[r * G::LP + pidx(x)], scale), a2 = cscale(sg[(G::R + r) * G::LP + pidx(x)], scale);
    T ux, uy;
    if (FLOW == 1) {
      double sx, cx, sy, cy;
      sincos(x * dx, &sx, &cx);
      sincos((y0 + r) * dy, &sy, &cy);
      ux = T(sx * cy);
      uy = T(-cx * sy);
    } else {
      ux = T(vnx);
      uy = T(vny);
    }
    const C v = mkc<T>(ux * a1.x + uy * a2.x, ux * a1.y + uy * a2.y);
    n = mkc<T>(n.x + v.y, n.y - v.x);  // -i v
    if (FLOW == 1) {
      const T w = T(0.25 * (1.0 / c.alpha)) * (ux * ux + uy * uy);
      n = mkc<T>(n.x - w * ps.x, n.y - w * ps.y);
    }
    nv[q] = n;
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < PER; ++q) {
    const int e = threadIdx.x + q * G::NT;
    s[(e / L) * G::LP + pidx(e % L)] = nv[q];
  }
  __syncthreads();
  fft_rows<T, L, G::R, G::NT, -1>(s, tw);
  for (int e = threadIdx.x; e < G::R * L; e += G::NT) {
    const int r = e % G::R, k = e / G::R;
    Td[(size_t)k * ny + y0 + r] = s[r * G::LP + pidx(k)];
  }
}

// Seeded vortex state (vk_common.cu).
__global__ void k_ic_vortices(double2* __restrict__ out, int nx, int ny, const double* __restrict__ vx,
                              const double* __restrict__ vy, const int* __restrict__ vq, int nv, double xi0,
                              double S);

// Sum per-CTA partials in a fixed order (deterministic) into out[0..2].
__global__ void k_reduce_partials3(const double* __restrict__ part, int nblk, double* __restrict__ out);

}  // namespace vk
