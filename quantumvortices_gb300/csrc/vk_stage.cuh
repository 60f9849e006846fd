// vk_stage.cuh -- persistent RK4 stage kernel and its grid-wide barrier.
//
// The four passes of one RK4 stage (X1, Y1, X2, Y2 of vk_kernels.cuh) run in
// one cooperative launch: the CTAs stride over each pass's tiles and meet at
// a grid-wide barrier between passes.  Every wait is bounded.
#pragma once
#include "vk_kernels.cuh"

namespace vk {

// count: CTAs arrived at the current barrier; gen: barrier generation; err:
// 0, or 1 + the index of the barrier where some CTA gave up (the host reads
// it and resets the whole struct before the next launch).
struct GridBarrier {
  unsigned int count;
  unsigned int gen;
  int err;
  int pad;
};

__device__ __forceinline__ unsigned int ld_acquire_gpu(const unsigned int* p) {
  unsigned int v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_gpu(unsigned int* p, unsigned int v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ int ld_relaxed_gpu(const int* p) {
  int v;
  asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// All CTAs of the grid (co-resident: cooperative launch) meet here.  Thread 0
// makes the CTA's writes visible (fence), arrives, and the last arrival
// resets the count and releases the next generation; the others poll it with
// acquire loads.  A CTA that polls more than `limit` times, or finds err set,
// records the barrier index (the first one wins) and returns false; the
// caller then returns, so a launch that timed out ends without further waits.
__device__ __forceinline__ bool grid_sync(GridBarrier* b, unsigned long long limit, int where) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = ld_relaxed_gpu(&b->err) == 0;
    if (ok) {
      const unsigned int g = ld_acquire_gpu(&b->gen);
      __threadfence();
      const unsigned int arrived = atomicAdd(&b->count, 1u) + 1u;
      if (arrived == gridDim.x) {
        b->count = 0u;
        st_release_gpu(&b->gen, g + 1u);
      } else {
        unsigned long long polls = 0;
        while (ld_acquire_gpu(&b->gen) == g) {
          if (polls++ >= limit || ld_relaxed_gpu(&b->err) != 0) {
            atomicCAS(&b->err, 0, 1 + where);
            ok = 0;
            break;
          }
          __nanosleep(64);
        }
      }
    }
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// Geometry of the persistent stage kernel: x tiles of R rows and y tiles with
// one block size.  FP32 at L = 1024: x tiles of two rows with one warp per
// row in the row transforms (the x kernels' layout at half the height) and
// the y kernels' one-column tiles; 64 threads, six CTAs per SM (registers
// capped at 168: the x bodies alone would take 255, which left four CTAs and
// measured slower than the separate pass kernels).
template <typename T, int LL> struct GeoFused;
template <> struct GeoFused<float, 1024> {
  struct X {
    static constexpr int L = 1024, R = 2, LP = padded(1024), NT = 64, MINB = 6;
  };
  typedef GeoY<float, 1024> Y;
  static constexpr int NT = 64, MINB = 6;
};

// One RK4 stage of one field in one launch (plain RHS: no particles, no
// forcing).  The tile loops run the pass bodies of the four pass kernels, and
// at half height the x tiles take the same row transforms, so the result
// equals the four-kernel stage bit for bit.  FROM_T = false: the first stage
// of a run, X1 reads psi.
template <typename T, int L, int STAGE, bool FROM_T>
__global__ void __launch_bounds__(GeoFused<T, L>::NT, GeoFused<T, L>::MINB)
    k_stage_rk4(Field<T> f, GridBarrier* bar, unsigned long long limit) {
  typedef typename GeoFused<T, L>::X GX;
  typedef typename GeoFused<T, L>::Y GY;
  static_assert(GX::NT == GY::NT && GY::NT == GeoFused<T, L>::NT, "one block size for the four passes");
  extern __shared__ __align__(16) unsigned char smraw[];
  cplx<T>* s = reinterpret_cast<cplx<T>*>(smraw);
  const StepConsts& c = f.c;
  const int nxt = c.ny / GX::R;
  for (int t = blockIdx.x; t < nxt; t += gridDim.x) {
    x1_body<T, L, GX, FROM_T, FROM_T>(f.Ta, f.psi, f.Tb, f.twx, c, t, s);
    __syncthreads();
  }
  if (!grid_sync(bar, limit, 3 * (STAGE - 1))) return;
  const int ny1 = (c.K + GY::R) / GY::R;
  for (int t = blockIdx.x; t < ny1; t += gridDim.x) {
    y1_body<T, L, GY>(f.Tb, f.Tc, f.twy, c, t, s);
    __syncthreads();
  }
  if (!grid_sync(bar, limit, 3 * (STAGE - 1) + 1)) return;
  for (int t = blockIdx.x; t < nxt; t += gridDim.x) {
    x2_body<T, L, GX, +1, true, false>(f.Tc, f.psi, (const T*)nullptr, f.Td, f.twx, c, t, s);
    __syncthreads();
  }
  if (!grid_sync(bar, limit, 3 * (STAGE - 1) + 2)) return;
  const int ny2 = (2 * c.K + GY::R) / GY::R;
  for (int t = blockIdx.x; t < ny2; t += gridDim.x) {
    y2_rk4_body<T, L, GY, STAGE, false>(f.Td, f.kpsi, f.str1, f.str2, f.Ta, f.twy, c, t, s);
    __syncthreads();
  }
}

}  // namespace vk
