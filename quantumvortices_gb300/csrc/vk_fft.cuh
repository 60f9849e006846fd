// vk_fft.cuh -- row FFT engine for sm_103a.
//
// A CTA holds R rows of L complex points in shared memory (row pitch
// LP = L + L/16: one pad slot per 16 points keeps the strided Stockham stores
// free of bank conflicts for 8- and 16-byte elements).  The transform is a
// mixed-radix Stockham auto-sort FFT: every stage reads RAD points at stride
// L/RAD, multiplies by table twiddles, runs a radix-RAD codelet in registers
// and writes RAD points at stride NS, so the output comes out in natural
// order.  Twiddles come from a per-length table W_L[k] = exp(-2 pi i k/L)
// generated on the host in FP64 (and rounded once for FP32).
//
// FP64 on GB300 issues about two DFMA per clock per SM, so the codelets are
// written for the fewest floating-point instructions: radix-16/8/4 butterflies
// with +-i rotations as register swaps, and every product by a constant
// rotation or a table twiddle fused into the butterfly that consumes it.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace vk {

template <typename T> struct cvec;
template <> struct cvec<double> { using type = double2; };
template <> struct cvec<float> { using type = float2; };
template <typename T> using cplx = typename cvec<T>::type;

template <typename T> __device__ __forceinline__ cplx<T> mkc(T x, T y) { cplx<T> r; r.x = x; r.y = y; return r; }
template <typename C> __device__ __forceinline__ C cadd(C a, C b) { a.x += b.x; a.y += b.y; return a; }
template <typename C> __device__ __forceinline__ C csub(C a, C b) { a.x -= b.x; a.y -= b.y; return a; }
template <typename C> __device__ __forceinline__ C cmul(C a, C b) {
  C r;
  r.x = a.x * b.x - a.y * b.y;
  r.y = a.x * b.y + a.y * b.x;
  return r;
}
template <typename C> __device__ __forceinline__ C cconj(C a) { a.y = -a.y; return a; }
template <typename C, typename S> __device__ __forceinline__ C cscale(C a, S s) { a.x *= s; a.y *= s; return a; }

// Multiply by exp(DIR * i*pi/2): -i for the forward (DIR<0), +i for inverse.
template <int DIR, typename C> __device__ __forceinline__ C rot90(C a) {
  C r;
  if (DIR < 0) { r.x = a.y; r.y = -a.x; } else { r.x = -a.y; r.y = a.x; }
  return r;
}
// Multiply by exp(DIR * i*pi/4) = (1 + DIR*i)/sqrt(2).
template <int DIR, typename C> __device__ __forceinline__ C rot45(C a) {
  typedef decltype(a.x) T;
  const T r = T(0.70710678118654752440084436210484903928);
  C o;
  if (DIR < 0) { o.x = (a.x + a.y) * r; o.y = (a.y - a.x) * r; }
  else { o.x = (a.x - a.y) * r; o.y = (a.x + a.y) * r; }
  return o;
}
// Multiply by exp(DIR * i*3pi/4).
template <int DIR, typename C> __device__ __forceinline__ C rot135(C a) { return rot90<DIR>(rot45<DIR>(a)); }
// Multiply by the constant (c, DIR*s): exp(DIR*i*theta) with c = cos, s = sin.
template <int DIR, typename C, typename T> __device__ __forceinline__ C rotc(C a, T c, T s) {
  C o;
  if (DIR < 0) { o.x = a.x * c + a.y * s; o.y = a.y * c - a.x * s; }
  else { o.x = a.x * c - a.y * s; o.y = a.y * c + a.x * s; }
  return o;
}

// ---- radix codelets: v[k] <- sum_m v[m] exp(DIR*2*pi*i*m*k/RAD) ----------
//
// Each codelet is a first butterfly layer over the pairs (m, m + RAD/2)
// followed by a tail.  Butterflies whose second operand is multiplied by a
// constant rotation or a table twiddle w are written as
//   e' = e + w o   (four FMAs: the products fused into the sum),
//   o' = e - w o = 2e - e'   (two FMAs),
// six FP64 instructions instead of four for the product and four for the
// sum and difference; the FP64 passes are bound by the FP64 pipe.

template <typename C> __device__ __forceinline__ void bfly(C& e, C& o) {
  const C t = e;
  e = cadd(t, o);
  o = csub(t, o);
}

// (e, o) <- (e + w o, e - w o) for w = (c, DIR*s).
template <int DIR, typename C, typename T> __device__ __forceinline__ void bfly_rot(C& e, C& o, T c, T s) {
  C p;
  if (DIR < 0) {  // w o = (o.x c + o.y s, o.y c - o.x s)
    p.x = fma(o.x, c, fma(o.y, s, e.x));
    p.y = fma(o.y, c, fma(-o.x, s, e.y));
  } else {        // w o = (o.x c - o.y s, o.y c + o.x s)
    p.x = fma(o.x, c, fma(-o.y, s, e.x));
    p.y = fma(o.y, c, fma(o.x, s, e.y));
  }
  o.x = fma(T(2), e.x, -p.x);
  o.y = fma(T(2), e.y, -p.y);
  e = p;
}

// (a, b) <- (a + w b, a - w b) for a table twiddle w (already conjugated for
// the inverse).
template <typename C> __device__ __forceinline__ void bfly_tw(C& a, C& b, C w) {
  typedef decltype(a.x) T;
  C p;
  p.x = fma(b.x, w.x, fma(-b.y, w.y, a.x));
  p.y = fma(b.y, w.x, fma(b.x, w.y, a.y));
  b.x = fma(T(2), a.x, -p.x);
  b.y = fma(T(2), a.y, -p.y);
  a = p;
}

// Tails: on entry v[m] = s_m = x_m + x_{m+RAD/2} and v[m+RAD/2] = d_m =
// x_m - x_{m+RAD/2} (m < RAD/2) for the RAD inputs x; on return v holds the
// DFT of x in natural order.

template <int DIR, typename C> __device__ __forceinline__ void dft4_tail(C& a0, C& a1, C& a2, C& a3) {
  // in: a0 = s0, a1 = s1, a2 = d0, a3 = d1
  C s0 = a0, s1 = a1, d0 = a2, d1 = rot90<DIR>(a3);
  bfly(s0, s1);
  bfly(d0, d1);
  a0 = s0; a2 = s1; a1 = d0; a3 = d1;
}

template <int DIR, typename C> __device__ __forceinline__ void dft8_tail(C* v) {
  typedef decltype(v[0].x) T;
  const T r = T(0.70710678118654752440084436210484903928);
  // even outputs: DFT4 of x0, x2, x4, x6 (pairs (x0,x4), (x2,x6));
  // odd: DFT4 of x1, x3, x5, x7 (pairs (x1,x5), (x3,x7))
  C e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6];
  C o0 = v[1], o1 = v[3], o2 = v[5], o3 = v[7];
  dft4_tail<DIR>(e0, e1, e2, e3);
  dft4_tail<DIR>(o0, o1, o2, o3);
  bfly(e0, o0);
  bfly_rot<DIR>(e1, o1, r, r);
  o2 = rot90<DIR>(o2);
  bfly(e2, o2);
  bfly_rot<DIR>(e3, o3, -r, r);
  v[0] = e0; v[1] = e1; v[2] = e2; v[3] = e3;
  v[4] = o0; v[5] = o1; v[6] = o2; v[7] = o3;
}

template <int DIR, typename C> __device__ __forceinline__ void dft16_tail(C* v) {
  typedef decltype(v[0].x) T;
  const T r = T(0.70710678118654752440084436210484903928);
  const T c1 = T(0.92387953251128675612818318939678828682);  // cos(pi/8)
  const T s1 = T(0.38268343236508977172845998403039886676);  // sin(pi/8)
  // even outputs: DFT8 of x_{2i} (its pairs (x_{2i}, x_{2i+8}) are s_{2i}, d_{2i})
  C e[8], o[8];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    e[i] = v[2 * i]; e[i + 4] = v[8 + 2 * i];
    o[i] = v[2 * i + 1]; o[i + 4] = v[9 + 2 * i];
  }
  dft8_tail<DIR>(e);
  dft8_tail<DIR>(o);
  bfly(e[0], o[0]);
  bfly_rot<DIR>(e[1], o[1], c1, s1);
  bfly_rot<DIR>(e[2], o[2], r, r);
  bfly_rot<DIR>(e[3], o[3], s1, c1);
  o[4] = rot90<DIR>(o[4]);
  bfly(e[4], o[4]);
  bfly_rot<DIR>(e[5], o[5], -s1, c1);
  bfly_rot<DIR>(e[6], o[6], -r, r);
  bfly_rot<DIR>(e[7], o[7], -c1, s1);
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    v[k] = e[k];
    v[k + 8] = o[k];
  }
}

template <int RAD, int DIR, typename C> __device__ __forceinline__ void dft_tail(C* v) {
  if (RAD == 4) dft4_tail<DIR>(v[0], v[1], v[2], v[3]);
  else if (RAD == 8) dft8_tail<DIR>(v);
  else if (RAD == 16) dft16_tail<DIR>(v);
}

template <int RAD, int DIR, typename C> __device__ __forceinline__ void dft(C* v) {
#pragma unroll
  for (int m = 0; m < RAD / 2; ++m) bfly(v[m], v[m + RAD / 2]);
  dft_tail<RAD, DIR>(v);
}

template <int DIR, typename C> __device__ __forceinline__ void dft16(C* v) { dft<16, DIR>(v); }

// 32-point DFT in registers: even/odd DFT16 and one radix-2 layer with the
// W32^k rotations, k = 0..15 (cos and sin of k*pi/16).
template <int DIR, typename C> __device__ __forceinline__ void dft32(C* v) {
  typedef decltype(v[0].x) T;
  C e[16], o[16];
#pragma unroll
  for (int i = 0; i < 16; ++i) { e[i] = v[2 * i]; o[i] = v[2 * i + 1]; }
  dft16<DIR>(e);
  dft16<DIR>(o);
  const T c1 = T(0.98078528040323044912618223613424), s1 = T(0.19509032201612826784828486847702);  // pi/16
  const T c2 = T(0.92387953251128675612818318939679), s2 = T(0.38268343236508977172845998403040);  // pi/8
  const T c3 = T(0.83146961230254523707878837761791), s3 = T(0.55557023301960222474283081394853);  // 3pi/16
  o[1] = rotc<DIR>(o[1], c1, s1);
  o[2] = rotc<DIR>(o[2], c2, s2);
  o[3] = rotc<DIR>(o[3], c3, s3);
  o[4] = rot45<DIR>(o[4]);
  o[5] = rotc<DIR>(o[5], s3, c3);
  o[6] = rotc<DIR>(o[6], s2, c2);
  o[7] = rotc<DIR>(o[7], s1, c1);
  o[8] = rot90<DIR>(o[8]);
  o[9] = rot90<DIR>(rotc<DIR>(o[9], c1, s1));
  o[10] = rot90<DIR>(rotc<DIR>(o[10], c2, s2));
  o[11] = rot90<DIR>(rotc<DIR>(o[11], c3, s3));
  o[12] = rot135<DIR>(o[12]);
  o[13] = rot90<DIR>(rotc<DIR>(o[13], s3, c3));
  o[14] = rot90<DIR>(rotc<DIR>(o[14], s2, c2));
  o[15] = rot90<DIR>(rotc<DIR>(o[15], s1, c1));
#pragma unroll
  for (int k = 0; k < 16; ++k) {
    v[k] = cadd(e[k], o[k]);
    v[k + 16] = csub(e[k], o[k]);
  }
}


// ---- plans ----------------------------------------------------------------
// PlanFor<L, MAXRAD>: radices of an L-point transform, none above MAXRAD.
// Every plan costs about 31-32 FP64 instructions per point at L = 1024.

template <int... Rs> struct RadixList {};
template <int L, int MAXRAD> struct PlanFor;
#define VK_PLAN(LL, MR, ...) \
  template <> struct PlanFor<LL, MR> { using type = RadixList<__VA_ARGS__>; };
VK_PLAN(16, 16, 16) VK_PLAN(32, 16, 8, 4) VK_PLAN(64, 16, 8, 8) VK_PLAN(128, 16, 16, 8)
VK_PLAN(256, 16, 16, 16) VK_PLAN(512, 16, 8, 8, 8) VK_PLAN(1024, 16, 16, 16, 4)
VK_PLAN(2048, 16, 16, 16, 8) VK_PLAN(4096, 16, 16, 16, 16)
VK_PLAN(16, 8, 8, 2) VK_PLAN(32, 8, 8, 4) VK_PLAN(64, 8, 8, 8) VK_PLAN(128, 8, 8, 4, 4)
VK_PLAN(256, 8, 8, 8, 4) VK_PLAN(512, 8, 8, 8, 8) VK_PLAN(1024, 8, 8, 8, 4, 4)
VK_PLAN(2048, 8, 8, 8, 8, 4) VK_PLAN(4096, 8, 8, 8, 8, 8)
VK_PLAN(16, 4, 4, 4) VK_PLAN(32, 4, 4, 4, 2) VK_PLAN(64, 4, 4, 4, 4) VK_PLAN(128, 4, 4, 4, 4, 2)
VK_PLAN(256, 4, 4, 4, 4, 4) VK_PLAN(512, 4, 4, 4, 4, 4, 2) VK_PLAN(1024, 4, 4, 4, 4, 4, 4)
VK_PLAN(2048, 4, 4, 4, 4, 4, 4, 2) VK_PLAN(4096, 4, 4, 4, 4, 4, 4, 4)
#undef VK_PLAN

__host__ __device__ constexpr int padded(int L) { return L + L / 16; }
__device__ __forceinline__ int pidx(int i) { return i + (i >> 4); }

// One Stockham stage over NR rows held in s (pitch LP); threads [0, NTA) of
// the block (size NTB) do the work, all threads pass the barriers.  The
// twiddle table holds W_{TWS*L}: TWS = 2 runs an L-point transform on the
// table of a 2L-point one.
template <typename T, int L, int NR, int NTA, int RAD, int NS, int DIR, int NTB, int TWS = 1>
__device__ __forceinline__ void stockham_stage(cplx<T>* s, const cplx<T>* __restrict__ tw) {
  typedef cplx<T> C;
  constexpr int NB = L / RAD;
  constexpr int LP = padded(L);
  static_assert((NR * NB) % NTA == 0, "threads must tile the butterflies");
  constexpr int PER = (NR * NB) / NTA;
  const bool active = (NTA == NTB) || ((int)threadIdx.x < NTA);
  C v[PER][RAD];
  if (active) {
#pragma unroll
    for (int p = 0; p < PER; ++p) {
      const int b = threadIdx.x + p * NTA;
      const int row = b / NB, j = b % NB;
      const C* sr = s + row * LP;
#pragma unroll
      for (int m = 0; m < RAD; ++m) v[p][m] = sr[pidx(j + m * NB)];
      if (NS > 1) {
        // twiddles fused into the first butterfly layer
        const int jj = j % NS;
#pragma unroll
        for (int m = 0; m < RAD / 2; ++m) {
          if (m > 0) {
            C w = __ldg(tw + jj * m * (TWS * L / (NS * RAD)));
            if (DIR > 0) w.y = -w.y;
            v[p][m] = cmul(v[p][m], w);
          }
          C wb = __ldg(tw + jj * (m + RAD / 2) * (TWS * L / (NS * RAD)));
          if (DIR > 0) wb.y = -wb.y;
          bfly_tw(v[p][m], v[p][m + RAD / 2], wb);
        }
        dft_tail<RAD, DIR>(v[p]);
      } else {
        dft<RAD, DIR>(v[p]);
      }
    }
  }
  __syncthreads();
  if (active) {
#pragma unroll
    for (int p = 0; p < PER; ++p) {
      const int b = threadIdx.x + p * NTA;
      const int row = b / NB, j = b % NB;
      C* sr = s + row * LP;
      const int base = (j / NS) * NS * RAD + (j % NS);
#pragma unroll
      for (int m = 0; m < RAD; ++m) sr[pidx(base + m * NS)] = v[p][m];
    }
  }
  __syncthreads();
}

template <typename T, int L, int NR, int NTA, int DIR, int NS, int NTB, int TWS>
__device__ __forceinline__ void run_stages(cplx<T>*, const cplx<T>*, RadixList<>) {}

template <typename T, int L, int NR, int NTA, int DIR, int NS, int NTB, int TWS, int RAD, int... Rest>
__device__ __forceinline__ void run_stages(cplx<T>* s, const cplx<T>* tw, RadixList<RAD, Rest...>) {
  stockham_stage<T, L, NR, NTA, RAD, NS, DIR, NTB, TWS>(s, tw);
  run_stages<T, L, NR, NTA, DIR, NS * RAD, NTB, TWS>(s, tw, RadixList<Rest...>());
}

__host__ __device__ constexpr int plan_maxrad(int e) { return e >= 16 ? 16 : (e >= 8 ? 8 : 4); }

// 1024-point transform of NR rows with one warp per row (FP32): the
// four-step split 1024 = 32 x 32 inside the warp.  Lane l holds x[l + 32 j]
// (j = 0..31), does a DFT32 over j, multiplies by W1024^(l k2), and the warp
// transposes through the row's own shared-memory slots (pitch 33); lane k2
// then does a DFT32 over l and writes X[k2 + 32 k1] in natural order.  Only
// __syncwarp between the phases: no block-wide barriers inside the
// transform.
template <typename T, int L, int NR, int DIR>
__device__ __forceinline__ void fft_rows_warp(cplx<T>* s, const cplx<T>* __restrict__ tw) {
  static_assert(L == 1024, "four-step 32 x 32");
  typedef cplx<T> C;
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (w < NR) {
    C* row = s + w * padded(L);
    C v[32];
#pragma unroll
    for (int j = 0; j < 32; ++j) v[j] = row[pidx(l + 32 * j)];
    dft32<DIR>(v);
#pragma unroll
    for (int k2 = 1; k2 < 32; ++k2) {
      C t = __ldg(tw + l * k2);
      if (DIR > 0) t.y = -t.y;
      v[k2] = cmul(v[k2], t);
    }
    __syncwarp();
#pragma unroll
    for (int k2 = 0; k2 < 32; ++k2) row[k2 * 33 + l] = v[k2];
    __syncwarp();
#pragma unroll
    for (int n1 = 0; n1 < 32; ++n1) v[n1] = row[l * 33 + n1];
    dft32<DIR>(v);
    __syncwarp();
#pragma unroll
    for (int k1 = 0; k1 < 32; ++k1) row[pidx(l + 32 * k1)] = v[k1];
  }
  __syncthreads();
}

// In-place FFT of the first NR rows of s by threads [0, NTA) of a block of
// NTB threads; every thread must call it.  The plan's largest radix is the
// number of points per thread (NR*L/NTA), capped at 16.  The caller must
// __syncthreads() after filling s; on return s holds the natural-order
// transform and the block is synchronised.  DIR = -1 forward, +1 inverse.
// FP32 1024-point rows with exactly one warp per row take the warp-per-row
// transform instead (the x passes; measured on GB300, the y passes and the
// paired half-height transforms are faster in the Stockham stages).
// TWS = 2: tw is the table of a 2L-point transform (the half-length
// transforms of single real rows).
template <typename T, int L, int NR, int NTA, int DIR, int NTB = NTA, int TWS = 1>
__device__ __forceinline__ void fft_rows(cplx<T>* s, const cplx<T>* __restrict__ tw) {
  if constexpr (sizeof(T) == 4 && L == 1024 && NTA == NTB && NTA == 32 * NR && TWS == 1) {
    fft_rows_warp<T, L, NR, DIR>(s, tw);
  } else {
    constexpr int E = NR * L / NTA;
    static_assert(E >= 4, "at least four points per thread");
    run_stages<T, L, NR, NTA, DIR, 1, NTB, TWS>(s, tw, typename PlanFor<L, plan_maxrad(E)>::type());
  }
}

}  // namespace vk
