// vk_nn.cu -- the learned ARGLE warm-start network on tcgen05 tensor cores.
//
// A 4-level periodic conv encoder-decoder (3x3 convolutions, channels
// base*2^l, 2x2 average pooling down, nearest upsampling up, additive skips,
// ReLU) maps 3 input channels (Re/Im of the vortex phase ansatz, signed
// vortex-charge density) to a 2-channel Re/Im correction of the ansatz.
// Activations and weights are BF16 (activations NHWC, channels padded to a
// multiple of 16); every convolution -- forward, data gradient and weight
// gradient -- is an implicit GEMM on tcgen05.mma.kind::f16 with FP32
// accumulation in tensor memory; master weights and Adam moments are FP32.
//
//   forward   D[pixel, co]      = sum_{tap,ci} in[pixel+off(tap), ci] W[co,tap,ci]
//   dgrad     dX[pixel, ci]     = sum_{tap,co} dY[pixel+off(tap), co] W[co,8-tap,ci]
//   wgrad     dW[tap*Cin+ci, co] = sum_pixel in[pixel+off(tap), ci] dY[pixel, co]
// (off(tap) = (tap/3-1, tap%3-1), periodic).  No reference counterpart: the
// reference has no machine learning.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <string>
#include <type_traits>
#include <vector>
#include "../../include/vk.h"
#include "vk_solver.h"
#include "vk_tc.cuh"

namespace vk {
namespace nn {

typedef __nv_bfloat16 bf16;

__device__ __forceinline__ int wrapi(int v, int n) { return v < 0 ? v + n : (v >= n ? v - n : v); }
__device__ __forceinline__ bool ld_err_nonzero(const int* err) { return *(volatile const int*)err != 0; }

// ------------------------------------------------------------------ conv --
// Implicit-GEMM convolution, one CTA = 128 output pixels x BN output
// channels (channel block blockIdx.y).  The reduction index kk = tap*Cin + ci
// runs over 9*Cin in chunks of 64 (a chunk may span taps; the tail is
// zero-filled), which is also the row layout of the weights [co][tap][ci], so
// a weight tile is 64 contiguous values per output channel.  Operand tiles
// stream through an S-stage shared-memory ring with cp.async (16-byte
// vectors, 8 channels of one pixel); thread 0 issues the chunk's four
// K = 16 MMAs and commits them to the stage's mbarrier, which frees the stage
// for the copies S - 1 chunks ahead.  Every wait is bounded.
constexpr int kConvStages = 2;

template <int BN>
__global__ void __launch_bounds__(128) k_conv(const bf16* __restrict__ in, int H, int W, int nimg, int Cin,
                                              const bf16* __restrict__ wgt, const float* __restrict__ bias,
                                              int cout, int relu, bf16* __restrict__ out_bf, int ldo,
                                              float* __restrict__ out_f, int nout, int* __restrict__ err) {
  constexpr int S = kConvStages;
  constexpr int ABYTES = 128 * 64 * 2, BBYTES = BN * 64 * 2, STAGE = ABYTES + BBYTES;
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ __align__(8) uint64_t bar[S];
  __shared__ uint32_t tslot;
  const int tid = threadIdx.x, warp = tid >> 5;
  const int npix = nimg * H * W;  // the images are stacked: image b holds rows [b H, (b + 1) H)
  const int p0 = blockIdx.x * 128, n0 = blockIdx.y * BN;
  const int KT = 9 * Cin, nck = (KT + 63) / 64;
  constexpr uint32_t NCOL = BN < 32 ? 32 : BN;
  if (warp == 0) tc::tmem_alloc(&tslot, NCOL);
  if (tid < S) tc::mbar_init(&bar[tid]);
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t taddr = tslot;
  const uint32_t idesc = tc::idesc_bf16(128, BN);
  // this thread's A vectors: column kv = tid & 7 of rows tid/8 + 16 j
  const int kv = tid & 7;
  int py[8], px[8], pyb[8];  // row in the image, column, first row of the image
  bool pin[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const int p = p0 + (tid >> 3) + 16 * j;
    pin[j] = p < npix;
    const int row = pin[j] ? p / W : 0;
    pyb[j] = row - row % H;
    py[j] = row - pyb[j];
    px[j] = pin[j] ? p % W : 0;
  }
  auto load_chunk = [&](int i, int buf) {
    unsigned char* sA = sm + buf * STAGE;
    unsigned char* sB = sA + ABYTES;
    const int kk = i * 64 + 8 * kv;
    const bool kin = kk < KT;
    const int tap = kin ? kk / Cin : 0, ci = kin ? kk - tap * Cin : 0;
    const int dy = tap / 3 - 1, dx = tap % 3 - 1;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int r = (tid >> 3) + 16 * j;
      const bool ok = kin && pin[j];
      const int src = ok ? (pyb[j] + wrapi(py[j] + dy, H)) * W + wrapi(px[j] + dx, W) : 0;
      tc::cp_async16<true>(sA + (r >> 3) * 1024 + kv * 128 + (r & 7) * 16, in + (size_t)src * Cin + ci, ok ? 16u : 0u);
    }
#pragma unroll
    for (int j = 0; j < (BN * 8 + 127) / 128; ++j) {
      const int r = (tid >> 3) + 16 * j;
      if (r < BN) {
        const bf16* src = kin ? wgt + (size_t)(n0 + r) * KT + kk : wgt;
        tc::cp_async16<false>(sB + (r >> 3) * 1024 + kv * 128 + (r & 7) * 16, src, kin ? 16u : 0u);
      }
    }
  };
#pragma unroll
  for (int s0 = 0; s0 < S - 1; ++s0) {
    if (s0 < nck) load_chunk(s0, s0);
    tc::cp_async_commit();
  }
  bool ok = true;
  int issued = 0;  // chunks whose MMAs were issued (same count in every thread)
  for (int i = 0; i < nck; ++i) {
    tc::cp_async_wait<S - 2>();
    tc::fence_async_smem();
    tc::fence_before();
    if (!__syncthreads_and(ok)) { ok = false; break; }
    tc::fence_after();
    ++issued;
    if (tid == 0) {
      const uint32_t a0 = tc::smem_u32(sm + (i % S) * STAGE);
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const uint64_t ad = tc::smem_desc(a0 + j * 256, 128, 1024);
        const uint64_t bd = tc::smem_desc(a0 + ABYTES + j * 256, 128, 1024);
        tc::mma(taddr, ad, bd, idesc, (i > 0 || j > 0) ? 1u : 0u);
      }
      tc::commit(&bar[i % S]);
    }
    const int jn = i + S - 1;
    if (jn < nck) {
      if (i >= 1) ok = tc::mbar_wait(&bar[(i - 1) % S], ((i - 1) / S) & 1, err) && ok;
      if (ok) load_chunk(jn, jn % S);
    }
    tc::cp_async_commit();
  }
  // drain: own copies, then the last issued MMAs (bounded; also after a timeout)
  tc::cp_async_wait<0>();
  if (issued > 0) ok = tc::mbar_wait(&bar[(issued - 1) % S], ((issued - 1) / S) & 1, err) && ok;
  tc::fence_after();
  if (__syncthreads_and(ok)) {
    const int r = 32 * warp + (tid & 31);
    const int p = p0 + r;
    constexpr int NC = BN < 32 ? 16 : 32;
#pragma unroll 1
    for (int c0 = 0; c0 < BN; c0 += NC) {
      float v[32];
      const uint32_t ta = taddr + ((uint32_t)(32 * warp) << 16) + c0;
      if (NC == 16) tc::tmem_ld16(ta, v);
      else tc::tmem_ld32(ta, v);
      if (p < npix) {
#pragma unroll
        for (int j = 0; j < NC; ++j) {
          const int c = n0 + c0 + j;
          float a = v[j] + ((bias && c < cout) ? bias[c] : 0.f);
          if (relu) a = fmaxf(a, 0.f);
          v[j] = a;
        }
        if (out_bf) {
#pragma unroll
          for (int q = 0; q < NC / 8; ++q) {
            uint4 w;
            __nv_bfloat162 h0 = __floats2bfloat162_rn(v[8 * q + 0], v[8 * q + 1]);
            __nv_bfloat162 h1 = __floats2bfloat162_rn(v[8 * q + 2], v[8 * q + 3]);
            __nv_bfloat162 h2 = __floats2bfloat162_rn(v[8 * q + 4], v[8 * q + 5]);
            __nv_bfloat162 h3 = __floats2bfloat162_rn(v[8 * q + 6], v[8 * q + 7]);
            w.x = *reinterpret_cast<uint32_t*>(&h0);
            w.y = *reinterpret_cast<uint32_t*>(&h1);
            w.z = *reinterpret_cast<uint32_t*>(&h2);
            w.w = *reinterpret_cast<uint32_t*>(&h3);
            *reinterpret_cast<uint4*>(out_bf + (size_t)p * ldo + n0 + c0 + 8 * q) = w;
          }
        }
        if (out_f)
          for (int j = 0; j < NC; ++j)
            if (n0 + c0 + j < nout) out_f[(size_t)p * nout + n0 + c0 + j] = v[j];
      }
    }
  }
  tc::fence_before();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(taddr, NCOL);
}

// TMA-fed convolution, Cin a multiple of CK (64, or 16/32 for the narrow
// layers).  The input is first copied into a periodically padded image stack
// [nimg][H+2][W+2][Cin] (k_pad), so that every tap of a 128-pixel tile is one
// rectangular box: TMA loads it (box {CK channels, BW pixels, 128/BW rows},
// BW = min(W, 128)) straight into the swizzle layout of rows of CK channels
// (2 CK bytes: the 128-, 64- or 32-byte swizzle), and the weight tile (box
// {CK, BN} of the [coutp][9 Cin] weight matrix) beside it.  The K loop runs
// over (tap, CK-channel chunk), for CK = 64 in the order of k_conv, through
// an S-stage ring: thread 0
// issues the loads on the stage's "full" mbarrier, thread 32 waits for it,
// issues the chunk's four K = 16 MMAs and commits them to the stage's "empty"
// mbarrier, which frees the stage for the load S chunks ahead.  Every wait is
// bounded; after a timeout the CTA waits (bounded) for its loads and MMAs in
// flight, frees its tensor memory and leaves the error word set.  On GB300
// the 512^2 training step (batches of 8) ran at 88 TFLOP/s with it against
// 81 without.
template <int BN, int S, int CK>
__global__ void __launch_bounds__(128) k_conv_tma(const __grid_constant__ CUtensorMap tmA,
                                                  const __grid_constant__ CUtensorMap tmB, int H, int W, int nimg,
                                                  int Cin, const float* __restrict__ bias, int cout, int relu,
                                                  bf16* __restrict__ out_bf, int ldo, float* __restrict__ out_f,
                                                  int nout, int* __restrict__ err) {
  constexpr int ABYTES = 128 * CK * 2, BBYTES = BN * CK * 2, STAGE = ABYTES + BBYTES;
  static_assert(ABYTES % (16 * CK) == 0 && STAGE % (16 * CK) == 0, "tiles on swizzle-atom boundaries");
  extern __shared__ __align__(1024) unsigned char smraw[];
  __shared__ __align__(8) uint64_t full[S], empty[S], done;
  __shared__ uint32_t tslot;
  __shared__ int s_loaded;
  // the 128-byte swizzle needs 1024-byte aligned tiles
  unsigned char* sm = smraw + ((1024 - (tc::smem_u32(smraw) & 1023)) & 1023);
  const int tid = threadIdx.x, warp = tid >> 5;
  const int npix = nimg * H * W;
  const int p0 = blockIdx.x * 128, n0 = blockIdx.y * BN;
  const int BW = W < 128 ? W : 128, BH = 128 / BW;
  const int row = p0 / W, x0 = p0 - row * W, b = row / H, y0 = row - b * H;
  const int cch = Cin / CK, nck = 9 * cch;
  constexpr uint32_t NCOL = BN < 32 ? 32 : BN;
  if (warp == 0) tc::tmem_alloc(&tslot, NCOL);
  if (tid == 0) {
    for (int i = 0; i < S; ++i) {
      tc::mbar_init(&full[i]);
      tc::mbar_init(&empty[i]);
    }
    tc::mbar_init(&done);
    s_loaded = 0;
  }
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t taddr = tslot;
  const uint32_t idesc = tc::idesc_bf16(128, BN);
  bool ok = true;
  if (tid == 0) {
    // producer: chunk i = (tap, channel chunk) into stage i % S
    int i = 0;
    for (; i < nck && ok; ++i) {
      const int st = i % S;
      if (i >= S) ok = tc::mbar_wait(&empty[st], ((i - S) / S) & 1, err);
      if (!ok) break;
      const int tap = i / cch, c0 = CK * (i - tap * cch);
      const int dy = tap / 3 - 1, dx = tap % 3 - 1;
      unsigned char* sA = sm + st * STAGE;
      tc::mbar_arrive_expect_tx(&full[st], STAGE);
      tc::tma_load_4d(sA, &tmA, &full[st], c0, x0 + 1 + dx, y0 + 1 + dy, b);
      tc::tma_load_2d(sA + ABYTES, &tmB, &full[st], tap * Cin + c0, n0);
    }
    s_loaded = i;
  } else if (tid == 32) {
    // MMA issuer
    for (int i = 0; i < nck && ok; ++i) {
      const int st = i % S;
      ok = tc::mbar_wait(&full[st], (i / S) & 1, err);
      if (!ok) break;
      tc::fence_after();
      const uint32_t a0 = tc::smem_u32(sm + st * STAGE);
#pragma unroll
      for (int j = 0; j < CK / 16; ++j) {
        const uint64_t ad = tc::smem_desc_swk<CK>(a0 + 32 * j);
        const uint64_t bd = tc::smem_desc_swk<CK>(a0 + ABYTES + 32 * j);
        tc::mma(taddr, ad, bd, idesc, (i > 0 || j > 0) ? 1u : 0u);
      }
      tc::commit(&empty[st]);
    }
    tc::commit(&done);  // arrives when every MMA issued above has finished
  }
  __syncthreads();
  // every thread: the MMAs done (bounded), then the epilogue
  ok = tc::mbar_wait(&done, 0, err) && ok;
  if (tid == 0 && ld_err_nonzero(err)) {
    // a wait ran out somewhere: let this CTA's loads land before its shared
    // memory goes away (bounded waits on the stages still in flight)
    const int loaded = s_loaded;
    for (int i = loaded - S < 0 ? 0 : loaded - S; i < loaded; ++i) tc::mbar_wait(&full[i % S], (i / S) & 1, err);
  }
  tc::fence_after();
  if (__syncthreads_and(ok)) {
    const int r = 32 * warp + (tid & 31);
    const int p = p0 + r;
    constexpr int NC = BN < 32 ? 16 : 32;
#pragma unroll 1
    for (int c0 = 0; c0 < BN; c0 += NC) {
      float v[32];
      const uint32_t ta = taddr + ((uint32_t)(32 * warp) << 16) + c0;
      if (NC == 16) tc::tmem_ld16(ta, v);
      else tc::tmem_ld32(ta, v);
      if (p < npix) {
#pragma unroll
        for (int j = 0; j < NC; ++j) {
          const int c = n0 + c0 + j;
          float a = v[j] + ((bias && c < cout) ? bias[c] : 0.f);
          if (relu) a = fmaxf(a, 0.f);
          v[j] = a;
        }
        if (out_bf) {
#pragma unroll
          for (int q = 0; q < NC / 8; ++q) {
            uint4 w;
            __nv_bfloat162 h0 = __floats2bfloat162_rn(v[8 * q + 0], v[8 * q + 1]);
            __nv_bfloat162 h1 = __floats2bfloat162_rn(v[8 * q + 2], v[8 * q + 3]);
            __nv_bfloat162 h2 = __floats2bfloat162_rn(v[8 * q + 4], v[8 * q + 5]);
            __nv_bfloat162 h3 = __floats2bfloat162_rn(v[8 * q + 6], v[8 * q + 7]);
            w.x = *reinterpret_cast<uint32_t*>(&h0);
            w.y = *reinterpret_cast<uint32_t*>(&h1);
            w.z = *reinterpret_cast<uint32_t*>(&h2);
            w.w = *reinterpret_cast<uint32_t*>(&h3);
            *reinterpret_cast<uint4*>(out_bf + (size_t)p * ldo + n0 + c0 + 8 * q) = w;
          }
        }
        if (out_f)
          for (int j = 0; j < NC; ++j)
            if (n0 + c0 + j < nout) out_f[(size_t)p * nout + n0 + c0 + j] = v[j];
      }
    }
  }
  tc::fence_before();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(taddr, NCOL);
}

// Channel-major copies for the TMA-fed weight gradient.  A block moves
// 64-pixel x 64-channel tiles of 8 consecutive image rows through shared
// memory with 16-byte loads (8 channels of a pixel) and 16-byte stores (8
// pixels of a channel).  W must be a multiple of 64 and C of 8.
// SHIFT = false: NHWC [nimg][H][W][C] -> [nimg][C][H][W]; with db, also
// db[c] += sum over the pixels of in[.][c] for c < nbias (the bias gradient).
// SHIFT = true: the three x-shifted, y-padded copies
// out[dx][nimg][C][H+2][W] = in[.][(y - 1) mod H][(x + dx - 1) mod W][.],
// dx = 0, 1, 2, so that every tap of a 64-pixel row chunk starts on a 64-pixel
// boundary (TMA wants the innermost coordinate on a 16-byte boundary).
template <bool SHIFT>
__global__ void __launch_bounds__(256) k_chw(const bf16* __restrict__ in, bf16* __restrict__ out, int H, int W, int C,
                                             int nimg, float* __restrict__ db, int nbias) {
  constexpr int NX = SHIFT ? 66 : 64;   // pixels x0 - 1 .. x0 + 64 when shifted
  // Row pitch (bf16) of the channel-major tile: 66 = 33 words, so channel
  // row r starts at bank r mod 32.  The scattered stores of the load phase
  // (lanes: 4 pixels x 8 channel groups, rows 8 g + k) then fall on 4 bank
  // groups (2-way), and the 8-pixel reads of the store phase (lanes: 4
  // channels x 8 pixel groups) on 32 distinct banks; a pitch of 72 (36
  // words) put all 8 channel groups on one bank.
  constexpr int SP = 66;
  constexpr int ROWS = 8;               // image rows per block (one bias atomic per channel and block)
  __shared__ __align__(16) bf16 t[64][SP];
  const int Hp = SHIFT ? H + 2 : H;
  const int x0 = blockIdx.x * 64, c0 = blockIdx.y * 64;
  const int nc = min(64, C - c0);  // channels of this tile (a multiple of 8)
  const size_t plane = (size_t)nimg * C * Hp * W;
  float sum[2] = {0.f, 0.f};
  const int r1 = min((int)(blockIdx.z + 1) * ROWS, nimg * Hp);
  for (int row = blockIdx.z * ROWS; row < r1; ++row) {
    const int b = row / Hp, yp = row - b * Hp;
    const int ys = SHIFT ? (yp == 0 ? H - 1 : (yp == H + 1 ? 0 : yp - 1)) : yp;
    __syncthreads();  // the previous row's tile has been read
    for (int v = threadIdx.x; v < NX * 8; v += blockDim.x) {
      const int i = v >> 3, g = v & 7;
      if (8 * g >= nc) continue;
      int xs = SHIFT ? x0 - 1 + i : x0 + i;
      xs = xs < 0 ? xs + W : (xs >= W ? xs - W : xs);
      const uint4 q = *reinterpret_cast<const uint4*>(in + (((size_t)b * H + ys) * W + xs) * C + c0 + 8 * g);
      const bf16* e = reinterpret_cast<const bf16*>(&q);
#pragma unroll
      for (int k = 0; k < 8; ++k) t[8 * g + k][i] = e[k];
    }
    __syncthreads();
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int v = threadIdx.x + 256 * h;
      const int c = v >> 3, pg = v & 7;
      if (c >= nc) continue;
#pragma unroll
      for (int dx = 0; dx < (SHIFT ? 3 : 1); ++dx) {
        uint4 q;
        bf16* e = reinterpret_cast<bf16*>(&q);
#pragma unroll
        for (int k = 0; k < 8; ++k) e[k] = t[c][8 * pg + k + dx];
        if (!SHIFT)
#pragma unroll
          for (int k = 0; k < 8; ++k) sum[h] += __bfloat162float(e[k]);
        *reinterpret_cast<uint4*>(out + dx * plane + (((size_t)b * C + c0 + c) * Hp + yp) * W + x0 + 8 * pg) = q;
      }
    }
  }
  if (!SHIFT && db) {
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      // the 8 threads of channel c are consecutive lanes
      float x = sum[h];
      x += __shfl_xor_sync(0xffffffffu, x, 1);
      x += __shfl_xor_sync(0xffffffffu, x, 2);
      x += __shfl_xor_sync(0xffffffffu, x, 4);
      const int v = threadIdx.x + 256 * h, c = v >> 3;
      if ((v & 7) == 0 && c < nc && c0 + c < nbias) atomicAdd(&db[c0 + c], x);
    }
  }
}

// Weight gradient on TMA-fed tiles: dW[m][n] += sum over this CTA's pixels q
// of X[q + off(tap)][ci] dY[q][n], m = tap Cin + ci.  X comes from its three
// x-shifted, y-padded channel-major copies [3][nimg][Cin][H+2][W] and dY from
// its channel-major copy [nimg][N][H][W], so for a chunk of 64 pixels of one
// image row every (tap, channel block) of the A tile and the whole B tile are
// rectangular boxes, starting on 64-pixel boundaries, that TMA loads,
// pixel-contiguous (K-major), in the 128-byte swizzle layout.  A tile of 128 rows takes 128/CB boxes of
// CB = min(Cin, 128) channels (one tap each).  Ring, roles, bounded waits and
// the timeout path as in k_conv_tma; the FP32 result is added to dW with
// atomics (the pixel range of a launch is split over blockIdx.y).
template <int BN, int S>
__global__ void __launch_bounds__(128) k_wgrad_tma(const __grid_constant__ CUtensorMap tmX,
                                                   const __grid_constant__ CUtensorMap tmD, int H, int W, int nimg,
                                                   int Cin, int pix_per_cta, float* __restrict__ dW,
                                                   int* __restrict__ err) {
  constexpr int ABYTES = 128 * 128, BBYTES = BN * 128, STAGE = ABYTES + BBYTES;
  static_assert(STAGE % 1024 == 0, "1024-byte aligned stages");
  extern __shared__ __align__(1024) unsigned char smraw[];
  __shared__ __align__(8) uint64_t full[S], empty[S], done;
  __shared__ uint32_t tslot;
  __shared__ int s_loaded;
  unsigned char* sm = smraw + ((1024 - (tc::smem_u32(smraw) & 1023)) & 1023);
  const int tid = threadIdx.x, warp = tid >> 5;
  const int npix = nimg * H * W, M = 9 * Cin;
  const int m0 = blockIdx.x * 128;
  const int q0 = blockIdx.y * pix_per_cta, q1 = min(npix, q0 + pix_per_cta);
  const int nck = q1 > q0 ? (q1 - q0) / 64 : 0;
  const int CB = Cin < 128 ? Cin : 128;
  constexpr uint32_t NCOL = BN < 32 ? 32 : BN;
  if (warp == 0) tc::tmem_alloc(&tslot, NCOL);
  if (tid == 0) {
    for (int i = 0; i < S; ++i) {
      tc::mbar_init(&full[i]);
      tc::mbar_init(&empty[i]);
    }
    tc::mbar_init(&done);
    s_loaded = 0;
  }
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t taddr = tslot;
  const uint32_t idesc = tc::idesc_bf16(128, BN);
  bool ok = true;
  if (tid == 0) {
    // A boxes of this M tile: rows [r, r + CB) hold tap m / Cin, channels from m % Cin
    int i = 0;
    for (; i < nck && ok; ++i) {
      const int st = i % S;
      if (i >= S) ok = tc::mbar_wait(&empty[st], ((i - S) / S) & 1, err);
      if (!ok) break;
      const int q = q0 + 64 * i;
      const int row = q / W, x0 = q - row * W, b = row / H, y = row - b * H;
      unsigned char* sA = sm + st * STAGE;
      int nbox = 0;
      for (int r = 0; r < 128 && m0 + r < M; r += CB) ++nbox;
      tc::mbar_arrive_expect_tx(&full[st], (uint32_t)(nbox * CB * 128 + BBYTES));
      for (int r = 0; r < 128 && m0 + r < M; r += CB) {
        const int m = m0 + r, tap = m / Cin, ci = m - tap * Cin;
        tc::tma_load_5d(sA + r * 128, &tmX, &full[st], x0, y + tap / 3, ci, b, tap % 3);
      }
      tc::tma_load_4d(sA + ABYTES, &tmD, &full[st], x0, y, 0, b);
    }
    s_loaded = i;
  } else if (tid == 32) {
    for (int i = 0; i < nck && ok; ++i) {
      const int st = i % S;
      ok = tc::mbar_wait(&full[st], (i / S) & 1, err);
      if (!ok) break;
      tc::fence_after();
      const uint32_t a0 = tc::smem_u32(sm + st * STAGE);
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const uint64_t ad = tc::smem_desc_sw128(a0 + 32 * j);
        const uint64_t bd = tc::smem_desc_sw128(a0 + ABYTES + 32 * j);
        tc::mma(taddr, ad, bd, idesc, (i > 0 || j > 0) ? 1u : 0u);
      }
      tc::commit(&empty[st]);
    }
    tc::commit(&done);
  }
  __syncthreads();
  ok = tc::mbar_wait(&done, 0, err) && ok;
  if (tid == 0 && ld_err_nonzero(err)) {
    const int loaded = s_loaded;
    for (int i = loaded - S < 0 ? 0 : loaded - S; i < loaded; ++i) tc::mbar_wait(&full[i % S], (i / S) & 1, err);
  }
  tc::fence_after();
  if (__syncthreads_and(ok) && nck > 0) {
    const int m = m0 + 32 * warp + (tid & 31);
    constexpr int NC = BN < 32 ? 16 : 32;
#pragma unroll 1
    for (int c0 = 0; c0 < BN; c0 += NC) {
      float v[32];
      const uint32_t ta = taddr + ((uint32_t)(32 * warp) << 16) + c0;
      if (NC == 16) tc::tmem_ld16(ta, v);
      else tc::tmem_ld32(ta, v);
      if (m < M)
#pragma unroll
        for (int j = 0; j < NC; j += 4)
          atomicAdd(reinterpret_cast<float4*>(&dW[(size_t)m * BN + c0 + j]), make_float4(v[j], v[j + 1], v[j + 2], v[j + 3]));
    }
  }
  tc::fence_before();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(taddr, NCOL);
}

// Periodic padding: out[b][y][x][c] = in[b][(y-1) mod H][(x-1) mod W][c] on
// the (H+2) x (W+2) stack, 16-byte vectors (C a multiple of 8).
__global__ void k_pad(const bf16* __restrict__ in, bf16* __restrict__ out, int H, int W, int C, int nimg) {
  const int cv = C / 8, Wp = W + 2, Hp = H + 2;
  const size_t n = (size_t)nimg * Hp * Wp * cv;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int v = (int)(i % cv);
    size_t t = i / cv;
    const int x = (int)(t % Wp);
    t /= Wp;
    const int y = (int)(t % Hp), b = (int)(t / Hp);
    const int ys = y == 0 ? H - 1 : (y == H + 1 ? 0 : y - 1), xs = x == 0 ? W - 1 : (x == W + 1 ? 0 : x - 1);
    reinterpret_cast<uint4*>(out)[i] =
        reinterpret_cast<const uint4*>(in)[(((size_t)b * H + ys) * W + xs) * cv + v];
  }
}

// Row-block convolution for the narrow layers (Cin <= 64, W a multiple of
// 128, H a multiple of RB).  A CTA computes RB output rows x 128 columns x BN
// channels in RB tensor-memory accumulators.  Each of the RB + 2 input rows
// it needs (periodic) is gathered once, as three column-shifted K-major tiles
// (dx = -1, 0, +1; [128 pixels][Cin]); each tile feeds the accumulators of up
// to three output rows (dy = -1, 0, +1) with the weights of tap (dy, dx),
// which stay in shared memory for the whole CTA.  Per output pixel that is
// 3 (RB + 2) / RB gathered row tiles instead of the 9 of k_conv.  Two input
// stages: row s + 1 is gathered while the tensor core works on row s.
template <int BN, int CIN, int RB>
__global__ void __launch_bounds__(128) k_conv_rows(const bf16* __restrict__ in, int H, int W,
                                                   const bf16* __restrict__ wgt, const float* __restrict__ bias,
                                                   int cout, int relu, bf16* __restrict__ out_bf, int ldo,
                                                   float* __restrict__ out_f, int nout, int* __restrict__ err) {
  constexpr int TA = 128 * CIN * 2;  // one shifted input tile
  constexpr int STAGE = 3 * TA;
  constexpr int WT = BN * CIN * 2;   // one tap's weight tile
  constexpr int VR = CIN / 8;        // 16-byte vectors per pixel
  constexpr int NS = RB + 2;         // input rows
  constexpr uint32_t SBO = (CIN / 8) * 128;
  constexpr int ACC = RB * BN;
  constexpr uint32_t NCOL = ACC <= 32 ? 32 : (ACC <= 64 ? 64 : (ACC <= 128 ? 128 : (ACC <= 256 ? 256 : 512)));
  extern __shared__ __align__(1024) unsigned char sm[];
  unsigned char* sW = sm;           // 9 * WT
  unsigned char* sI = sm + 9 * WT;  // 2 * STAGE
  __shared__ __align__(8) uint64_t bar[2];
  __shared__ uint32_t tslot;
  const int tid = threadIdx.x, warp = tid >> 5;
  // stacked images: rows [y0, y0 + RB) lie in image y0 / H (RB divides H)
  const int x0 = blockIdx.x * 128, y0 = blockIdx.y * RB, n0 = blockIdx.z * BN;
  const int yb = y0 - y0 % H, yl = y0 - yb;
  if (warp == 0) tc::tmem_alloc(&tslot, NCOL);
  if (tid < 2) tc::mbar_init(&bar[tid]);
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t taddr = tslot;
  const uint32_t idesc = tc::idesc_bf16(128, BN);
  // weights of all nine taps: rows co = n0 + r, K = ci (row stride 9 * CIN)
  for (int i = tid; i < 9 * BN * VR; i += 128) {
    const int tap = i / (BN * VR), rem = i - tap * (BN * VR), r = rem / VR, kv = rem - r * VR;
    tc::cp_async16<false>(sW + tap * WT + tc::tile_off(r, 8 * kv, CIN), wgt + ((size_t)(n0 + r) * 9 + tap) * CIN + 8 * kv,
                          16u);
  }
  tc::cp_async_commit();
  auto load_row = [&](int srow, int buf) {
    const int j = yb + wrapi(yl - 1 + srow, H);
    unsigned char* st = sI + buf * STAGE;
    for (int i = tid; i < 3 * 128 * VR; i += 128) {
      const int dx = i / (128 * VR), rem = i - dx * (128 * VR), m = rem / VR, kv = rem - m * VR;
      const int x = wrapi(x0 + m + dx - 1, W);
      tc::cp_async16<true>(st + dx * TA + tc::tile_off(m, 8 * kv, CIN), in + ((size_t)j * W + x) * CIN + 8 * kv, 16u);
    }
  };
  load_row(0, 0);
  tc::cp_async_commit();
  bool ok = true;
  int issued = 0;
  for (int srow = 0; srow < NS; ++srow) {
    if (srow + 1 < NS) {
      if (srow >= 1) ok = tc::mbar_wait(&bar[(srow - 1) & 1], ((srow - 1) >> 1) & 1, err) && ok;  // frees buffer
      if (ok) load_row(srow + 1, (srow + 1) & 1);
    }
    tc::cp_async_commit();
    tc::cp_async_wait<1>();  // everything but the newest group: row srow (and the weights)
    tc::fence_async_smem();
    tc::fence_before();
    if (!__syncthreads_and(ok)) { ok = false; break; }
    tc::fence_after();
    ++issued;
    if (tid == 0) {
      const uint32_t a0 = tc::smem_u32(sI + (srow & 1) * STAGE), w0 = tc::smem_u32(sW);
#pragma unroll
      for (int dy = -1; dy <= 1; ++dy) {
        const int r = srow - 1 - dy;  // output row fed by input row srow through dy
        if (r < 0 || r >= RB) continue;
#pragma unroll
        for (int dx = 0; dx < 3; ++dx) {
          const int tap = (dy + 1) * 3 + dx;
#pragma unroll
          for (int kk = 0; kk < CIN / 16; ++kk) {
            const uint64_t ad = tc::smem_desc(a0 + dx * TA + kk * 256, 128, SBO);
            const uint64_t bd = tc::smem_desc(w0 + tap * WT + kk * 256, 128, SBO);
            const bool first = (dy == -1 && dx == 0 && kk == 0);  // input row srow = r opens accumulator r
            tc::mma(taddr + (uint32_t)(r * BN), ad, bd, idesc, first ? 0u : 1u);
          }
        }
      }
      tc::commit(&bar[srow & 1]);
    }
  }
  tc::cp_async_wait<0>();
  if (issued > 0) ok = tc::mbar_wait(&bar[(issued - 1) & 1], ((issued - 1) >> 1) & 1, err) && ok;
  tc::fence_after();
  if (__syncthreads_and(ok) && issued == NS) {
    const int xcol = x0 + 32 * warp + (tid & 31);
    constexpr int NC = BN < 32 ? 16 : 32;
#pragma unroll 1
    for (int r = 0; r < RB; ++r) {
      const size_t p = (size_t)(y0 + r) * W + xcol;
#pragma unroll 1
      for (int c0 = 0; c0 < BN; c0 += NC) {
        float v[32];
        const uint32_t ta = taddr + ((uint32_t)(32 * warp) << 16) + (uint32_t)(r * BN + c0);
        if (NC == 16) tc::tmem_ld16(ta, v);
        else tc::tmem_ld32(ta, v);
#pragma unroll
        for (int j = 0; j < NC; ++j) {
          const int c = n0 + c0 + j;
          float a = v[j] + ((bias && c < cout) ? bias[c] : 0.f);
          if (relu) a = fmaxf(a, 0.f);
          v[j] = a;
        }
        if (out_bf) {
#pragma unroll
          for (int q = 0; q < NC / 8; ++q) {
            uint4 w;
            __nv_bfloat162 h0 = __floats2bfloat162_rn(v[8 * q + 0], v[8 * q + 1]);
            __nv_bfloat162 h1 = __floats2bfloat162_rn(v[8 * q + 2], v[8 * q + 3]);
            __nv_bfloat162 h2 = __floats2bfloat162_rn(v[8 * q + 4], v[8 * q + 5]);
            __nv_bfloat162 h3 = __floats2bfloat162_rn(v[8 * q + 6], v[8 * q + 7]);
            w.x = *reinterpret_cast<uint32_t*>(&h0);
            w.y = *reinterpret_cast<uint32_t*>(&h1);
            w.z = *reinterpret_cast<uint32_t*>(&h2);
            w.w = *reinterpret_cast<uint32_t*>(&h3);
            *reinterpret_cast<uint4*>(out_bf + p * ldo + n0 + c0 + 8 * q) = w;
          }
        }
        if (out_f)
          for (int j = 0; j < NC; ++j)
            if (n0 + c0 + j < nout) out_f[p * nout + n0 + c0 + j] = v[j];
      }
    }
  }
  tc::fence_before();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(taddr, NCOL);
}

// 8x8 transpose of 16-bit values: r[i] holds 8 channels of pixel i; on
// return t[c] holds channel c of pixels 0..7 (both as 4 x u32 pairs).
__device__ __forceinline__ void transpose8x8(const uint4 (&r)[8], uint4 (&t)[8]) {
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    uint32_t lo[4], hi[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const uint32_t x = (&r[2 * k].x)[j], y = (&r[2 * k + 1].x)[j];
      lo[k] = __byte_perm(x, y, 0x5410);
      hi[k] = __byte_perm(x, y, 0x7632);
    }
    t[2 * j] = make_uint4(lo[0], lo[1], lo[2], lo[3]);
    t[2 * j + 1] = make_uint4(hi[0], hi[1], hi[2], hi[3]);
  }
}

// Weight gradient dW[m][co] (m = tap*Cin + ci) += sum over this CTA's pixel
// range of in[q + off(tap)][ci] * dy[q][co]: rows m in a tile of 128,
// columns BN = all output channels, reduction over pixels in chunks of 64.
// Both operands are channel-contiguous in memory and pixel-contiguous in
// the K-major tiles, so each thread loads 8x8 blocks (8 pixels x 16 bytes),
// transposes them in registers and stores one 128-byte core matrix.  The
// loads run DEPTH chunks ahead of the tensor core (register sets), and the
// MMA tiles are double-buffered.  With db != nullptr the CTAs of the first
// row tile also reduce the bias gradient db[co] += sum_q dy[q][co] (co < nb)
// from the dy blocks they already hold.
template <int BN, int DEPTH>
__global__ void __launch_bounds__(128) k_wgrad(const bf16* __restrict__ in, const bf16* __restrict__ dy, int H, int W,
                                               int nimg, int Cin, int pix_per_cta, float* __restrict__ dW,
                                               float* __restrict__ db, int nb, int* __restrict__ err) {
  constexpr int ABYTES = 128 * 64 * 2, STAGE = ABYTES + BN * 64 * 2;
  constexpr int NBB = (BN + 127) / 128;  // B blocks per thread
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ __align__(8) uint64_t bar[2];
  __shared__ uint32_t tslot;
  const int tid = threadIdx.x, warp = tid >> 5;
  const int npix = nimg * H * W, M = 9 * Cin;  // stacked images, as in k_conv
  const int m0 = blockIdx.x * 128;
  const int q0 = blockIdx.y * pix_per_cta, q1 = min(npix, q0 + pix_per_cta);
  const int nck = q1 > q0 ? (q1 - q0 + 63) / 64 : 0;
  const bool do_bias = db != nullptr && blockIdx.x == 0;
  constexpr uint32_t NCOL = BN < 32 ? 32 : BN;
  if (warp == 0) tc::tmem_alloc(&tslot, NCOL);
  if (tid < 2) tc::mbar_init(&bar[tid]);
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t taddr = tslot;
  const uint32_t idesc = tc::idesc_bf16(128, BN);
  // A block of this thread: rows m0 + 8*rb .. +7 (one tap), pixels 8*kb .. +7
  const int rb = tid >> 3, kb = tid & 7;
  const int mA = m0 + 8 * rb;
  const bool rowok = mA < M;
  const int tap = rowok ? mA / Cin : 0, ci0 = rowok ? mA - tap * Cin : 0;
  const int ty = tap / 3 - 1, tx = tap % 3 - 1;
  uint4 ra[DEPTH][8], rbv[DEPTH][NBB][8];
  float bsum[NBB][8];
#pragma unroll
  for (int b = 0; b < NBB; ++b)
#pragma unroll
    for (int c = 0; c < 8; ++c) bsum[b][c] = 0.f;
  auto load_regs = [&](int i, auto slot_c) {
    constexpr int SL = decltype(slot_c)::value;
    const int qb = q0 + i * 64 + 8 * kb;
#pragma unroll
    for (int e = 0; e < 8; ++e) {
      const int q = qb + e;
      uint4 v = make_uint4(0, 0, 0, 0);
      if (rowok && q < q1) {
        const int y = q / W, x = q - y * W;
        const int yb = y - y % H;
        const int src = (yb + wrapi(y - yb + ty, H)) * W + wrapi(x + tx, W);
        v = *reinterpret_cast<const uint4*>(in + (size_t)src * Cin + ci0);
      }
      ra[SL][e] = v;
    }
#pragma unroll
    for (int b = 0; b < NBB; ++b) {
      const int cb = (tid + 128 * b) >> 3;
#pragma unroll
      for (int e = 0; e < 8; ++e) {
        const int q = qb + e;
        uint4 v = make_uint4(0, 0, 0, 0);
        if (cb < BN / 8 && q < q1) v = *reinterpret_cast<const uint4*>(dy + (size_t)q * BN + 8 * cb);
        rbv[SL][b][e] = v;
      }
    }
  };
  auto store_regs = [&](int buf, auto slot_c) {
    constexpr int SL = decltype(slot_c)::value;
    unsigned char* sA = sm + buf * STAGE;
    unsigned char* sB = sA + ABYTES;
    uint4 t[8];
    transpose8x8(ra[SL], t);
#pragma unroll
    for (int c = 0; c < 8; ++c) *reinterpret_cast<uint4*>(sA + rb * 1024 + kb * 128 + c * 16) = t[c];
#pragma unroll
    for (int b = 0; b < NBB; ++b) {
      const int cb = (tid + 128 * b) >> 3;
      if (cb < BN / 8) {
        if (do_bias) {
#pragma unroll
          for (int e = 0; e < 8; ++e) {
            const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&rbv[SL][b][e]);
#pragma unroll
            for (int c = 0; c < 4; ++c) {
              const float2 f = __bfloat1622float2(h[c]);
              bsum[b][2 * c] += f.x;
              bsum[b][2 * c + 1] += f.y;
            }
          }
        }
        transpose8x8(rbv[SL][b], t);
#pragma unroll
        for (int c = 0; c < 8; ++c) *reinterpret_cast<uint4*>(sB + cb * 1024 + kb * 128 + c * 16) = t[c];
      }
    }
  };
  bool ok = true;
  int issued = 0;
  // one chunk: free its tile buffer, fill it from the register set, issue its MMAs, prefetch
  auto step = [&](int i, auto slot_c) -> bool {
    const int buf = i & 1;
    if (i >= 2) ok = tc::mbar_wait(&bar[buf], ((i - 2) >> 1) & 1, err) && ok;
    if (ok) store_regs(buf, slot_c);
    tc::fence_async_smem();
    tc::fence_before();
    if (!__syncthreads_and(ok)) { ok = false; return false; }
    tc::fence_after();
    ++issued;
    if (tid == 0) {
      const uint32_t a0 = tc::smem_u32(sm + buf * STAGE);
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const uint64_t ad = tc::smem_desc(a0 + j * 256, 128, 1024);
        const uint64_t bd = tc::smem_desc(a0 + ABYTES + j * 256, 128, 1024);
        tc::mma(taddr, ad, bd, idesc, (i > 0 || j > 0) ? 1u : 0u);
      }
      tc::commit(&bar[buf]);
    }
    if (i + DEPTH < nck) load_regs(i + DEPTH, slot_c);
    return true;
  };
  using S0 = std::integral_constant<int, 0>;
  using S1 = std::integral_constant<int, DEPTH - 1>;
  if (nck > 0) load_regs(0, S0());
  if (DEPTH == 2 && nck > 1) load_regs(1, S1());
  if (DEPTH == 2) {
    for (int i = 0; i < nck; i += 2) {
      if (!step(i, S0())) break;
      if (i + 1 < nck && !step(i + 1, S1())) break;
    }
  } else {
    for (int i = 0; i < nck; ++i)
      if (!step(i, S0())) break;
  }
  if (issued > 0) ok = tc::mbar_wait(&bar[(issued - 1) & 1], ((issued - 1) >> 1) & 1, err) && ok;
  tc::fence_after();
  if (__syncthreads_and(ok) && issued > 0) {  // CTA-uniform: every warp runs the TMEM loads
    const int r = 32 * warp + (tid & 31);
    const int m = m0 + r;
    constexpr int NC = BN < 32 ? 16 : 32;
#pragma unroll 1
    for (int c0 = 0; c0 < BN; c0 += NC) {
      float v[32];
      const uint32_t ta = taddr + ((uint32_t)(32 * warp) << 16) + c0;
      if (NC == 16) tc::tmem_ld16(ta, v);
      else tc::tmem_ld32(ta, v);
      if (m < M)
#pragma unroll
        for (int j = 0; j < NC; j += 4)
          atomicAdd(reinterpret_cast<float4*>(&dW[(size_t)m * BN + c0 + j]), make_float4(v[j], v[j + 1], v[j + 2], v[j + 3]));
    }
    if (do_bias) {
#pragma unroll
      for (int b = 0; b < NBB; ++b) {
        const int cb = (tid + 128 * b) >> 3;
#pragma unroll
        for (int c = 0; c < 8; ++c) {
          float x = bsum[b][c];
          x += __shfl_xor_sync(0xffffffffu, x, 1);
          x += __shfl_xor_sync(0xffffffffu, x, 2);
          x += __shfl_xor_sync(0xffffffffu, x, 4);
          bsum[b][c] = x;
        }
        if (kb == 0 && cb < BN / 8)
          for (int c = 0; c < 8; ++c)
            if (8 * cb + c < nb) atomicAdd(&db[8 * cb + c], bsum[b][c]);
      }
    }
  }
  tc::fence_before();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(taddr, NCOL);
}

// ------------------------------------------------------------ elementwise --

// planar [nimg][cin][npix] FP32 -> NHWC BF16 [nimg * npix][cpad]
__global__ void k_pack_input(const float* __restrict__ in, bf16* __restrict__ out, int npix, int nimg, int cin,
                             int cpad) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nimg * npix * cpad; i += gridDim.x * blockDim.x) {
    const int p = i / cpad, c = i % cpad, b = p / npix, q = p - b * npix;
    out[i] = __float2bfloat16(c < cin ? in[((size_t)b * cin + c) * npix + q] : 0.f);
  }
}
__global__ void k_pool(const bf16* __restrict__ in, bf16* __restrict__ out, int H, int W, int C) {
  const int h = H / 2, w = W / 2;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < h * w * C; i += gridDim.x * blockDim.x) {
    const int c = i % C, p = i / C, y = p / w, x = p % w;
    const size_t b = ((size_t)(2 * y) * W + 2 * x) * C + c;
    const float s = __bfloat162float(in[b]) + __bfloat162float(in[b + C]) + __bfloat162float(in[b + (size_t)W * C]) +
                    __bfloat162float(in[b + (size_t)W * C + C]);
    out[i] = __float2bfloat16(0.25f * s);
  }
}
__global__ void k_pool_bwd(const bf16* __restrict__ dout, bf16* __restrict__ din, int H, int W, int C) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < H * W * C; i += gridDim.x * blockDim.x) {
    const int c = i % C, p = i / C, y = p / W, x = p % W;
    din[i] = __float2bfloat16(0.25f * __bfloat162float(dout[((size_t)(y / 2) * (W / 2) + x / 2) * C + c]));
  }
}
__global__ void k_up(const bf16* __restrict__ in, bf16* __restrict__ out, int H, int W, int C) {
  // out is H x W, in is H/2 x W/2; 8 channels per thread step
  const int cv = C / 8;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < H * W * cv; i += gridDim.x * blockDim.x) {
    const int c = i % cv, p = i / cv, y = p / W, x = p % W;
    reinterpret_cast<uint4*>(out)[i] = reinterpret_cast<const uint4*>(in)[((size_t)(y / 2) * (W / 2) + x / 2) * cv + c];
  }
}
__global__ void k_up_bwd(const bf16* __restrict__ dout, bf16* __restrict__ din, int H, int W, int C) {
  // dout is H x W, din is H/2 x W/2
  const int h = H / 2, w = W / 2;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < h * w * C; i += gridDim.x * blockDim.x) {
    const int c = i % C, p = i / C, y = p / w, x = p % w;
    const size_t b = ((size_t)(2 * y) * W + 2 * x) * C + c;
    const float s = __bfloat162float(dout[b]) + __bfloat162float(dout[b + C]) +
                    __bfloat162float(dout[b + (size_t)W * C]) + __bfloat162float(dout[b + (size_t)W * C + C]);
    din[i] = __float2bfloat16(s);
  }
}
// The elementwise kernels below take 8 BF16 values (16 bytes) per thread
// step; n is a multiple of 8 (channels are padded to 16).
__global__ void k_add(const bf16* __restrict__ a, const bf16* __restrict__ b, bf16* __restrict__ o, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n / 8; i += (size_t)gridDim.x * blockDim.x) {
    uint4 qa = reinterpret_cast<const uint4*>(a)[i], qb = reinterpret_cast<const uint4*>(b)[i], qo;
    const __nv_bfloat162* ea = reinterpret_cast<const __nv_bfloat162*>(&qa);
    const __nv_bfloat162* eb = reinterpret_cast<const __nv_bfloat162*>(&qb);
    __nv_bfloat162* eo = reinterpret_cast<__nv_bfloat162*>(&qo);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const float2 fa = __bfloat1622float2(ea[k]), fb = __bfloat1622float2(eb[k]);
      eo[k] = __floats2bfloat162_rn(fa.x + fb.x, fa.y + fb.y);
    }
    reinterpret_cast<uint4*>(o)[i] = qo;
  }
}
// d_pre = d_post * (y > 0)
__global__ void k_relu_bwd(const bf16* __restrict__ y, const bf16* __restrict__ d, bf16* __restrict__ o, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n / 8; i += (size_t)gridDim.x * blockDim.x) {
    uint4 qy = reinterpret_cast<const uint4*>(y)[i], qd = reinterpret_cast<const uint4*>(d)[i], qo;
    const bf16* ey = reinterpret_cast<const bf16*>(&qy);
    const bf16* ed = reinterpret_cast<const bf16*>(&qd);
    bf16* eo = reinterpret_cast<bf16*>(&qo);
#pragma unroll
    for (int k = 0; k < 8; ++k) eo[k] = __bfloat162float(ey[k]) > 0.f ? ed[k] : __float2bfloat16(0.f);
    reinterpret_cast<uint4*>(o)[i] = qo;
  }
}
// MSE loss (mean over the images, pixels and outputs) on the head output
// (FP32 [p][nout], p over the stacked images) against planar targets
// [nimg][nout][npix]; writes the BF16 gradient [p][cpad] and accumulates the
// loss.
__global__ void k_loss(const float* __restrict__ out, const float* __restrict__ tgt, int npix, int nimg, int nout,
                       int cpad, bf16* __restrict__ dout, double* __restrict__ loss) {
  const float inv = 1.f / (float)(nimg * npix * nout);
  double acc = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nimg * npix * cpad; i += gridDim.x * blockDim.x) {
    const int p = i / cpad, c = i % cpad, b = p / npix, q = p - b * npix;
    float g = 0.f;
    if (c < nout) {
      const float e = out[(size_t)p * nout + c] - tgt[((size_t)b * nout + c) * npix + q];
      acc += (double)e * e;
      g = 2.f * e * inv;
    }
    dout[i] = __float2bfloat16(g);
  }
  __shared__ double red[256];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) atomicAdd(loss, red[0] * (double)inv);
}
// master FP32 W[cout][9][cin] -> BF16 Wb[coutp][9][cinp] and flipped
// transpose Wt[cinp][9][coutp] (Wt[ci][t][co] = W[co][8-t][ci]).
__global__ void k_weights(const float* __restrict__ w, int cout, int cin, int coutp, int cinp, bf16* __restrict__ wb,
                          bf16* __restrict__ wt) {
  const int n = coutp * 9 * cinp;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int ci = i % cinp, t = (i / cinp) % 9, co = i / (9 * cinp);
    const float v = (co < cout && ci < cin) ? w[((size_t)co * 9 + t) * cin + ci] : 0.f;
    wb[i] = __float2bfloat16(v);
    wt[((size_t)ci * 9 + (8 - t)) * coutp + co] = __float2bfloat16(v);
  }
}
// dW_gemm[tap*cinp+ci][coutp] -> master-layout grad[co][tap][ci] (+=)
__global__ void k_wgrad_scatter(const float* __restrict__ g, int cout, int cin, int coutp, int cinp,
                                float* __restrict__ grad) {
  const int n = cout * 9 * cin;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int ci = i % cin, t = (i / cin) % 9, co = i / (9 * cin);
    grad[i] += g[((size_t)t * cinp + ci) * coutp + co];
  }
}
// [p][2] over the stacked images -> planar [nimg][2][npix]
__global__ void k_planar2(const float* __restrict__ in, float* __restrict__ out, int npix, int nimg) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < nimg * npix; p += gridDim.x * blockDim.x) {
    const int b = p / npix, q = p - b * npix;
    out[(size_t)b * 2 * npix + q] = in[2 * p];
    out[(size_t)b * 2 * npix + npix + q] = in[2 * p + 1];
  }
}
// hyper = {lr, 1 - b1^t, 1 - b2^t} in device memory, so that a captured
// training step replays with the current step's values.
__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                       size_t n, const float* __restrict__ hyper, float b1, float b2, float eps) {
  const float lr = hyper[0], c1 = hyper[1], c2 = hyper[2];
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi, vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

// --------------------------------------------------------- input features --
// Per-vortex Gaussian factors of the signed charge density:
// gx[j][x] = exp(-dx^2/(2 w^2)), gy[j][y] likewise, dx the periodic distance
// of grid column x (at 2 pi x / W) from vortex j, folded into [-pi, pi).
__global__ void k_feat_tables(const double* __restrict__ pos, int nv, int H, int W, double inv2w2,
                              float* __restrict__ gx, float* __restrict__ gy) {
  const double two_pi = 6.283185307179586476925286766559, pi = 0.5 * two_pi;
  const int n = nv * (W + H);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const bool isx = i < nv * W;
    const int k = isx ? i : i - nv * W;
    const int len = isx ? W : H, j = k / len, t = k - j * len;
    const double c = isx ? pos[2 * j] : pos[2 * j + 1];
    double d = t * (two_pi / len) - c + pi;
    d = d - two_pi * floor(d / two_pi) - pi;
    (isx ? gx : gy)[k] = (float)exp(-d * d * inv2w2);
  }
}
// out [3][H][W] planar FP32: Re psi, Im psi, sum_j q_j gx[j][x] gy[j][y] with
// q_j = +1 for the first half of the vortices and -1 for the rest.
__global__ void k_features(const double2* __restrict__ psi, const float* __restrict__ gx,
                           const float* __restrict__ gy, int nv, int H, int W, float* __restrict__ out) {
  const int npix = H * W;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < npix; p += gridDim.x * blockDim.x) {
    const int y = p / W, x = p - y * W;
    float q = 0.f;
    for (int j = 0; j < nv; ++j) q = fmaf(j < nv / 2 ? gx[j * W + x] : -gx[j * W + x], gy[j * H + y], q);
    const double2 v = psi[p];
    out[p] = (float)v.x;
    out[npix + p] = (float)v.y;
    out[2 * npix + p] = q;
  }
}

// ------------------------------------------------------------- network --

// One image's h x w x c; the buffer holds the network's batch capacity of
// images stacked along h (image b in rows [b h, (b + 1) h)).
struct Tensor {
  bf16* d = nullptr;
  int h = 0, w = 0, c = 0;
  size_t n() const { return (size_t)h * w * c; }
};

struct Conv {
  int cin, cout, cinp, coutp;
  size_t woff, boff;  // offsets into the parameter vector
  bool relu;
  bf16 *wb = nullptr, *wt = nullptr;
};

static int pad16(int c) { return (c + 15) / 16 * 16; }

// cuTensorMapEncodeTiled from the driver, looked up through the runtime (no
// link-time dependency on libcuda).
typedef CUresult (*EncodeTiled)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
static EncodeTiled encode_tiled_fn() {
  void* f = nullptr;
  cudaDriverEntryPointQueryResult q;
  if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
      q != cudaDriverEntryPointSuccess)
    return nullptr;
  return reinterpret_cast<EncodeTiled>(f);
}

class Net {
 public:
  int H, W, base, levels;
  std::vector<Conv> convs;
  size_t nparam = 0;
  float *param = nullptr, *grad = nullptr, *adam_m = nullptr, *adam_v = nullptr;
  float* wscratch = nullptr;  // dW GEMM output
  size_t wscratch_n = 0;
  int* err = nullptr;
  double* loss = nullptr;
  float* out_f = nullptr;     // head output [p][2]
  int64_t steps = 0;
  int nb = 1, bcap = 1;       // images in the current batch, batch capacity
  // One CUDA graph per training step (forward, backward, Adam), captured at
  // the second step of a batch size and replayed after it: the step's inputs
  // are copied into fixed buffers first, and Adam reads lr and its bias
  // corrections from device memory.  VK_NN_GRAPH=0: plain launches.
  float *in_stage = nullptr, *tgt_stage = nullptr, *hyper = nullptr;
  float hyper_h[3] = {0.f, 0.f, 0.f};
  cudaGraphExec_t tgraph = nullptr;
  int tgraph_nb = 0;
  bool graph_ok_ = [] {
    const char* e = std::getenv("VK_NN_GRAPH");
    return !(e && e[0] == '0');
  }();
  static constexpr int kMaxVortices = 4096;  // vk_nn_features
  double2* feat_psi = nullptr;
  double* feat_pos = nullptr;
  float *feat_gx = nullptr, *feat_gy = nullptr;
  cudaStream_t st = nullptr;
  // row-block kernel for the narrow layers (VK_CONV_ROWS=0 turns it off)
  bool rows_ok_ = [] {
    const char* e = std::getenv("VK_CONV_ROWS");
    return !(e && e[0] == '0');
  }();
  // TMA-fed convolution for inputs of 64k channels (VK_CONV_TMA=0 turns it off)
  bool tma_ok_ = [] {
    const char* e = std::getenv("VK_CONV_TMA");
    return !(e && e[0] == '0');
  }();
  // ... and for the narrow layers (16 or 32 input channels) too with VK_CONV_TMA_NARROW=1
  bool tma_narrow_ = [] {
    const char* e = std::getenv("VK_CONV_TMA_NARROW");
    return e && e[0] == '1';
  }();
  bf16* padbuf = nullptr;  // periodically padded input of k_conv_tma
  size_t padbuf_n = 0;
  bf16* xsbuf = nullptr;   // three shifted channel-major input copies (k_wgrad_tma)
  bf16* dchw = nullptr;    // channel-major output gradient (k_wgrad_tma)
  std::vector<void*> allocs;
  // activations (forward) per level and gradient scratch
  Tensor x0;
  std::vector<Tensor> a, s, p, u, c, e, d;   // see forward()
  Tensor b4;
  std::vector<Tensor> g1, g2, g3;             // gradient scratch per level (3 buffers)
  Tensor dhead;

  ~Net() {
    if (tgraph) cudaGraphExecDestroy(tgraph);
    for (auto* q : allocs) cudaFree(q);
    if (st) cudaStreamDestroy(st);
  }

  template <typename X> X* dalloc(size_t n) {
    X* q = nullptr;
    if (cudaMalloc(&q, sizeof(X) * std::max<size_t>(n, 1)) != cudaSuccess) return nullptr;
    cudaMemset(q, 0, sizeof(X) * std::max<size_t>(n, 1));
    allocs.push_back(q);
    return q;
  }
  Tensor tens(int h, int w, int c) {
    Tensor t;
    t.h = h;
    t.w = w;
    t.c = c;
    t.d = dalloc<bf16>(t.n() * bcap);
    return t;
  }
  size_t N(const Tensor& t) const { return t.n() * nb; }  // elements of the current batch
  int add_conv(int cin, int cout, bool relu) {
    Conv cv;
    cv.cin = cin;
    cv.cout = cout;
    cv.cinp = pad16(cin);
    cv.coutp = pad16(cout);
    cv.relu = relu;
    cv.woff = nparam;
    nparam += (size_t)cout * 9 * cin;
    cv.boff = nparam;
    nparam += cout;
    convs.push_back(cv);
    return (int)convs.size() - 1;
  }

  int init(int h, int w, int base_ch, int nlev, uint64_t seed, int batch_cap) {
    bcap = nb = batch_cap;
    H = h;
    W = w;
    base = base_ch;
    levels = nlev;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return VK_E_CUDA;
    // layer list: encoder (2 convs per level), decoder (2 per level), head
    add_conv(3, base, true);
    add_conv(base, base, true);
    for (int l = 1; l < levels; ++l) {
      add_conv(base << (l - 1), base << l, true);
      add_conv(base << l, base << l, true);
    }
    for (int l = levels - 2; l >= 0; --l) {
      add_conv(base << (l + 1), base << l, true);
      add_conv(base << l, base << l, true);
    }
    add_conv(base, 2, false);
    param = dalloc<float>(nparam);
    grad = dalloc<float>(nparam);
    adam_m = dalloc<float>(nparam);
    adam_v = dalloc<float>(nparam);
    err = dalloc<int>(1);
    loss = dalloc<double>(1);
    if (!param || !grad || !adam_m || !adam_v || !err || !loss) return VK_E_NOMEM;
    // He-normal initialisation (host, SplitMix64 + Box-Muller), zero biases
    std::vector<float> hp(nparam, 0.f);
    uint64_t s0 = seed;
    auto next = [&]() {
      uint64_t z = (s0 += 0x9E3779B97F4A7C15ull);
      z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
      z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
      z ^= z >> 31;
      return ((double)(z >> 11) + 0.5) * (1.0 / 9007199254740992.0);
    };
    for (const Conv& cv : convs) {
      const double sd = std::sqrt(2.0 / (9.0 * cv.cin)) * (cv.relu ? 1.0 : 0.1);
      for (size_t i = 0; i < (size_t)cv.cout * 9 * cv.cin; ++i) {
        const double u1 = next(), u2 = next();
        hp[cv.woff + i] = (float)(sd * std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2));
      }
    }
    cudaMemcpy(param, hp.data(), sizeof(float) * nparam, cudaMemcpyHostToDevice);
    size_t mx = 0;
    for (Conv& cv : convs) {
      cv.wb = dalloc<bf16>((size_t)cv.coutp * 9 * cv.cinp);
      cv.wt = dalloc<bf16>((size_t)cv.cinp * 9 * cv.coutp);
      mx = std::max(mx, (size_t)9 * cv.cinp * cv.coutp);
    }
    wscratch = dalloc<float>(mx);
    wscratch_n = mx;
    // activations
    x0 = tens(H, W, 16);
    for (int l = 0; l < levels; ++l) {
      const int hh = H >> l, ww = W >> l, ch = base << l;
      a.push_back(tens(hh, ww, ch));
      s.push_back(tens(hh, ww, ch));
      p.push_back(l + 1 < levels ? tens(hh / 2, ww / 2, ch) : Tensor());
      g1.push_back(tens(hh, ww, std::max(ch, 2 * ch)));
      g2.push_back(tens(hh, ww, std::max(ch, 2 * ch)));
      g3.push_back(tens(hh, ww, std::max(ch, 2 * ch)));
      if (l + 1 < levels) {
        u.push_back(tens(hh, ww, base << (l + 1)));
        c.push_back(tens(hh, ww, ch));
        e.push_back(tens(hh, ww, ch));
        d.push_back(tens(hh, ww, ch));
      } else {
        u.push_back(Tensor());
        c.push_back(Tensor());
        e.push_back(Tensor());
        d.push_back(Tensor());
      }
    }
    dhead = tens(H, W, 16);
    // largest padded input of a TMA convolution: level l holds at most
    // base << (l + 1) channels (the upsampled decoder input)
    for (int l = 0; l < levels; ++l)
      padbuf_n = std::max(padbuf_n, (size_t)bcap * ((H >> l) + 2) * ((W >> l) + 2) * (size_t)(base << (l + 1)));
    padbuf = dalloc<bf16>(padbuf_n);
    xsbuf = dalloc<bf16>(3 * padbuf_n);
    dchw = dalloc<bf16>(padbuf_n);
    out_f = dalloc<float>((size_t)H * W * 2 * bcap);
    in_stage = dalloc<float>((size_t)H * W * 3 * bcap);
    tgt_stage = dalloc<float>((size_t)H * W * 2 * bcap);
    hyper = dalloc<float>(3);
    feat_psi = dalloc<double2>((size_t)H * W);
    feat_pos = dalloc<double>(2 * kMaxVortices);
    feat_gx = dalloc<float>((size_t)kMaxVortices * W);
    feat_gy = dalloc<float>((size_t)kMaxVortices * H);
    for (auto* q : allocs)
      if (!q) return VK_E_NOMEM;
    return refresh_weights();
  }

  int refresh_weights() {
    for (Conv& cv : convs)
      k_weights<<<256, 256, 0, st>>>(param + cv.woff, cv.cout, cv.cin, cv.coutp, cv.cinp, cv.wb, cv.wt);
    return cudaGetLastError() == cudaSuccess ? VK_OK : VK_E_CUDA;
  }

  // ---- launches
  // Convolution of `in` with weights w (rows [cout_p][9*in.c]); output
  // channels split into blocks of BN so that small levels still fill the GPU.
  void conv(const Tensor& in, const bf16* w, int cout_p, int cout, const float* bias, int relu, bf16* out_bf,
            float* out_f32, int nout) {
    if (conv_tma(in, w, cout_p, cout, bias, relu, out_bf, out_f32, nout)) return;
    if (conv_rows(in, w, cout_p, cout, bias, relu, out_bf, out_f32, nout)) return;
    const int npix = nb * in.h * in.w;
    const int tiles = (npix + 127) / 128;
    int bn = std::min(cout_p, 128);
    while (bn > 32 && tiles * (cout_p / bn) < 2 * 152) bn /= 2;
    const dim3 grid(tiles, cout_p / bn);
    switch (bn) {
      case 16: launch_conv<16>(grid, in, w, bias, cout, relu, out_bf, cout_p, out_f32, nout); break;
      case 32: launch_conv<32>(grid, in, w, bias, cout, relu, out_bf, cout_p, out_f32, nout); break;
      case 64: launch_conv<64>(grid, in, w, bias, cout, relu, out_bf, cout_p, out_f32, nout); break;
      default: launch_conv<128>(grid, in, w, bias, cout, relu, out_bf, cout_p, out_f32, nout); break;
    }
  }
  // The TMA-fed kernel when enabled and the shape allows it: Cin a multiple
  // of 64, and 128-pixel tiles that are whole rows or whole row groups of one
  // image.
  bool conv_tma(const Tensor& in, const bf16* w, int cout_p, int cout, const float* bias, int relu, bf16* ob,
                float* of, int nout) {
    const int Hh = in.h, Ww = in.w, C = in.c;
    const int ck = C % 64 == 0 ? 64 : (C % 32 == 0 ? 32 : 16);
    if (!tma_ok_ || (ck < 64 && !tma_narrow_) || C % 16 != 0 || Hh * Ww < 128) return false;
    if (!(Ww % 128 == 0 || (128 % Ww == 0 && Hh % (128 / Ww) == 0))) return false;
    if ((size_t)nb * (Hh + 2) * (Ww + 2) * C > padbuf_n) return false;
    static EncodeTiled enc = encode_tiled_fn();
    if (!enc) return false;
    k_pad<<<blocks((size_t)nb * (Hh + 2) * (Ww + 2) * C / 8), 256, 0, st>>>(in.d, padbuf, Hh, Ww, C, nb);
    const int tiles = nb * Hh * Ww / 128;
    int bn = std::min(cout_p, 128);
    while (bn > 32 && tiles * (cout_p / bn) < 2 * 152) bn /= 2;
    if (cout_p % bn != 0 || bn < 16) return false;
    CUtensorMap ta, tb;
    const int bw = Ww < 128 ? Ww : 128;
    const cuuint64_t gA[4] = {(cuuint64_t)C, (cuuint64_t)Ww + 2, (cuuint64_t)Hh + 2, (cuuint64_t)nb};
    const cuuint64_t sA[3] = {(cuuint64_t)C * 2, (cuuint64_t)(Ww + 2) * C * 2, (cuuint64_t)(Hh + 2) * (Ww + 2) * C * 2};
    const cuuint32_t bA[4] = {(cuuint32_t)ck, (cuuint32_t)bw, (cuuint32_t)(128 / bw), 1};
    const cuuint32_t e4[4] = {1, 1, 1, 1};
    const cuuint64_t gB[2] = {(cuuint64_t)9 * C, (cuuint64_t)cout_p};
    const cuuint64_t sB[1] = {(cuuint64_t)9 * C * 2};
    const cuuint32_t bB[2] = {(cuuint32_t)ck, (cuuint32_t)bn};
    const CUtensorMapSwizzle sw = ck == 64 ? CU_TENSOR_MAP_SWIZZLE_128B
                                           : (ck == 32 ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_32B);
    if (enc(&ta, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, padbuf, gA, sA, bA, e4, CU_TENSOR_MAP_INTERLEAVE_NONE, sw,
            CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS ||
        enc(&tb, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<bf16*>(w), gB, sB, bB, e4,
            CU_TENSOR_MAP_INTERLEAVE_NONE, sw, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return false;
    const dim3 grid(tiles, cout_p / bn);
    auto go = [&](auto ckc) {
      constexpr int CK = decltype(ckc)::value;
      switch (bn) {
        case 16: launch_tma<16, CK>(grid, ta, tb, in, bias, cout, relu, ob, cout_p, of, nout); break;
        case 32: launch_tma<32, CK>(grid, ta, tb, in, bias, cout, relu, ob, cout_p, of, nout); break;
        case 64: launch_tma<64, CK>(grid, ta, tb, in, bias, cout, relu, ob, cout_p, of, nout); break;
        default: launch_tma<128, CK>(grid, ta, tb, in, bias, cout, relu, ob, cout_p, of, nout); break;
      }
    };
    if (ck == 64) go(std::integral_constant<int, 64>());
    else if (ck == 32) go(std::integral_constant<int, 32>());
    else go(std::integral_constant<int, 16>());
    return true;
  }
  // Ring depth: 3 stages for tiles of 64 or more channels (two or three CTAs
  // per SM, so one CTA's epilogue overlaps another's MMAs), 4 for narrower.
  template <int BN> static constexpr int tma_stages() { return BN >= 64 ? 3 : 4; }
  template <int BN, int CK>
  void launch_tma(dim3 grid, const CUtensorMap& ta, const CUtensorMap& tb, const Tensor& in, const float* bias,
                  int cout, int relu, bf16* ob, int ldo, float* of, int nout) {
    constexpr int S = tma_stages<BN>();
    const size_t smem = (size_t)S * (128 * CK * 2 + BN * CK * 2) + 1024;
    static bool attr = false;
    if (!attr) {
      cudaFuncSetAttribute(k_conv_tma<BN, S, CK>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      attr = true;
    }
    k_conv_tma<BN, S, CK><<<grid, 128, smem, st>>>(ta, tb, in.h, in.w, nb, in.c, bias, cout, relu, ob, ldo,
                                                             of, nout, err);
  }
  // The row-block kernel for narrow layers when the shape allows it.
  bool conv_rows(const Tensor& in, const bf16* w, int cout_p, int cout, const float* bias, int relu, bf16* ob,
                 float* of, int nout) {
    const int cin = in.c;
    if (!rows_ok_ || (cin != 16 && cin != 32 && cin != 64) || in.w % 128 != 0 || cout_p > 64) return false;
    int rb = 4;
    int bn = cout_p;
    auto ctas = [&]() { return (in.w / 128) * (nb * in.h / rb) * (cout_p / bn); };
    if (ctas() < 2 * 152 && bn > 32) bn /= 2;
    if (ctas() < 2 * 152) rb = 2;
    if (in.h % rb != 0) return false;
    const dim3 grid(in.w / 128, nb * in.h / rb, cout_p / bn);
#define VK_ROWS(B, CI, R)                                                                     \
  if (bn == B && cin == CI && rb == R) {                                                      \
    launch_rows<B, CI, R>(grid, in, w, bias, cout, relu, ob, cout_p, of, nout);               \
    return true;                                                                              \
  }
    VK_ROWS(16, 16, 4) VK_ROWS(16, 32, 4) VK_ROWS(16, 64, 4) VK_ROWS(32, 16, 4) VK_ROWS(32, 32, 4)
    VK_ROWS(32, 64, 4) VK_ROWS(64, 16, 4) VK_ROWS(64, 32, 4) VK_ROWS(64, 64, 4)
    VK_ROWS(16, 16, 2) VK_ROWS(16, 32, 2) VK_ROWS(16, 64, 2) VK_ROWS(32, 16, 2) VK_ROWS(32, 32, 2)
    VK_ROWS(32, 64, 2) VK_ROWS(64, 16, 2) VK_ROWS(64, 32, 2) VK_ROWS(64, 64, 2)
#undef VK_ROWS
    return false;
  }
  template <int BN, int CIN, int RB>
  void launch_rows(dim3 grid, const Tensor& in, const bf16* w, const float* bias, int cout, int relu, bf16* ob, int ldo,
                   float* of, int nout) {
    const size_t smem = (size_t)9 * BN * CIN * 2 + 2 * 3 * 128 * CIN * 2;
    static bool attr = false;
    if (!attr) {
      cudaFuncSetAttribute(k_conv_rows<BN, CIN, RB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      attr = true;
    }
    k_conv_rows<BN, CIN, RB><<<grid, 128, smem, st>>>(in.d, in.h, in.w, w, bias, cout, relu, ob, ldo, of, nout, err);
  }
  template <int BN>
  void launch_conv(dim3 grid, const Tensor& in, const bf16* w, const float* bias, int cout, int relu, bf16* ob,
                   int ldo, float* of, int nout) {
    const size_t smem = (size_t)kConvStages * (128 * 64 * 2 + BN * 64 * 2);
    static bool attr = false;
    if (!attr) {
      cudaFuncSetAttribute(k_conv<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      attr = true;
    }
    k_conv<BN><<<grid, 128, smem, st>>>(in.d, in.h, in.w, nb, in.c, w, bias, cout, relu, ob, ldo, of, nout, err);
  }
  // dW GEMM (and, with db, the bias gradient of the nb real channels).
  // The TMA-fed weight gradient when enabled and the shape allows it: rows of
  // 64k pixels, Cin dividing 128 or a multiple of it, at most 256 output
  // channels.  On GB300 the k_wgrad launches took 56% of a 512^2 training
  // step (batches of 8) at 30-60 TFLOP/s.
  bool wgrad_tma(const Tensor& in, const bf16* dy, int coutp, float* out, float* db, int nbias) {
    const int Hh = in.h, Ww = in.w, C = in.c;
    if (!tma_ok_ || Ww % 64 != 0 || C % 16 != 0 || (128 % C != 0 && C % 128 != 0) || coutp % 16 != 0 ||
        coutp > 256)
      return false;
    if ((size_t)nb * C * (Hh + 2) * Ww > padbuf_n || (size_t)nb * coutp * Hh * Ww > padbuf_n) return false;
    static EncodeTiled enc = encode_tiled_fn();
    if (!enc) return false;
    const int CB = C < 128 ? C : 128;
    CUtensorMap tx, td;
    const cuuint64_t gX[5] = {(cuuint64_t)Ww, (cuuint64_t)Hh + 2, (cuuint64_t)C, (cuuint64_t)nb, 3};
    const cuuint64_t sX[4] = {(cuuint64_t)Ww * 2, (cuuint64_t)(Hh + 2) * Ww * 2, (cuuint64_t)C * (Hh + 2) * Ww * 2,
                              (cuuint64_t)nb * C * (Hh + 2) * Ww * 2};
    const cuuint32_t bX[5] = {64, 1, (cuuint32_t)CB, 1, 1};
    const cuuint64_t gD[4] = {(cuuint64_t)Ww, (cuuint64_t)Hh, (cuuint64_t)coutp, (cuuint64_t)nb};
    const cuuint64_t sD[3] = {(cuuint64_t)Ww * 2, (cuuint64_t)Hh * Ww * 2, (cuuint64_t)coutp * Hh * Ww * 2};
    const cuuint32_t bD[4] = {64, 1, (cuuint32_t)coutp, 1};
    const cuuint32_t e5[5] = {1, 1, 1, 1, 1};
    if (enc(&tx, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, xsbuf, gX, sX, bX, e5, CU_TENSOR_MAP_INTERLEAVE_NONE,
            CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS ||
        enc(&td, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, dchw, gD, sD, bD, e5, CU_TENSOR_MAP_INTERLEAVE_NONE,
            CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return false;
    k_chw<true><<<dim3(Ww / 64, (C + 63) / 64, (nb * (Hh + 2) + 7) / 8), 256, 0, st>>>(in.d, xsbuf, Hh, Ww, C, nb,
                                                                                      nullptr, 0);
    k_chw<false><<<dim3(Ww / 64, (coutp + 63) / 64, (nb * Hh + 7) / 8), 256, 0, st>>>(dy, dchw, Hh, Ww, coutp, nb, db,
                                                                                     nbias);
    const int npix = nb * Hh * Ww, M = 9 * C;
    const int mt = (M + 127) / 128;
    int ppc = 8192;
    while ((npix + ppc - 1) / ppc * mt < 8 * 152 && ppc > 256) ppc /= 2;
    cudaMemsetAsync(out, 0, sizeof(float) * (size_t)M * coutp, st);
    const dim3 grid(mt, (npix + ppc - 1) / ppc);
    switch (coutp) {
      case 16: launch_wgrad_tma<16, 4>(grid, tx, td, in, ppc, out); break;
      case 32: launch_wgrad_tma<32, 4>(grid, tx, td, in, ppc, out); break;
      case 64: launch_wgrad_tma<64, 4>(grid, tx, td, in, ppc, out); break;
      case 128: launch_wgrad_tma<128, 3>(grid, tx, td, in, ppc, out); break;  // two CTAs per SM
      case 256: launch_wgrad_tma<256, 3>(grid, tx, td, in, ppc, out); break;
      default: return false;
    }
    return true;
  }
  template <int BN, int S>
  void launch_wgrad_tma(dim3 grid, const CUtensorMap& tx, const CUtensorMap& td, const Tensor& in, int ppc,
                        float* out) {
    const size_t smem = (size_t)S * (128 * 128 + BN * 128) + 1024;
    static bool attr = false;
    if (!attr) {
      cudaFuncSetAttribute(k_wgrad_tma<BN, S>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      attr = true;
    }
    k_wgrad_tma<BN, S><<<grid, 128, smem, st>>>(tx, td, in.h, in.w, nb, in.c, ppc, out, err);
  }
  void wgrad(const Tensor& in, const bf16* dy, int coutp, float* out, float* db, int nbias) {
    if (wgrad_tma(in, dy, coutp, out, db, nbias)) return;
    const int npix = nb * in.h * in.w, M = 9 * in.c;
    const int mt = (M + 127) / 128;
    int ppc = 8192;
    while ((npix + ppc - 1) / ppc * mt < 8 * 152 && ppc > 256) ppc /= 2;
    dim3 grid(mt, (npix + ppc - 1) / ppc);
    const size_t smem = 2 * (128 * 64 * 2 + (size_t)coutp * 64 * 2);
    cudaMemsetAsync(out, 0, sizeof(float) * (size_t)M * coutp, st);
    switch (coutp) {
      case 16: launch_wgrad<16, 2>(grid, smem, in, dy, ppc, out, db, nbias); break;
      case 32: launch_wgrad<32, 2>(grid, smem, in, dy, ppc, out, db, nbias); break;
      case 64: launch_wgrad<64, 2>(grid, smem, in, dy, ppc, out, db, nbias); break;
      case 128: launch_wgrad<128, 2>(grid, smem, in, dy, ppc, out, db, nbias); break;
      default: launch_wgrad<256, 1>(grid, smem, in, dy, ppc, out, db, nbias); break;
    }
  }
  template <int BN, int DEPTH>
  void launch_wgrad(dim3 grid, size_t smem, const Tensor& in, const bf16* dy, int ppc, float* out, float* db, int nbias) {
    static bool attr = false;
    if (!attr) {
      cudaFuncSetAttribute(k_wgrad<BN, DEPTH>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      attr = true;
    }
    k_wgrad<BN, DEPTH><<<grid, 128, smem, st>>>(in.d, dy, in.h, in.w, nb, in.c, ppc, out, db, nbias, err);
  }
  static int blocks(size_t n) { return (int)std::min<size_t>((n + 255) / 256, 152 * 16); }

  // Forward pass; returns the head output in out_f [p][2].
  void forward(const float* input) {
    const int npix = H * W;
    k_pack_input<<<blocks((size_t)nb * npix * 16), 256, 0, st>>>(input, x0.d, npix, nb, 3, 16);
    int ci = 0;
    const Tensor* cur = &x0;
    for (int l = 0; l < levels; ++l) {
      const Conv& c1 = convs[ci++];
      conv(*cur, c1.wb, c1.coutp, c1.cout, param + c1.boff, 1, a[l].d, nullptr, 0);
      const Conv& c2 = convs[ci++];
      conv(a[l], c2.wb, c2.coutp, c2.cout, param + c2.boff, 1, s[l].d, nullptr, 0);
      if (l + 1 < levels) {
        k_pool<<<blocks(N(p[l])), 256, 0, st>>>(s[l].d, p[l].d, nb * s[l].h, s[l].w, s[l].c);
        cur = &p[l];
      }
    }
    const Tensor* dec = &s[levels - 1];
    for (int l = levels - 2; l >= 0; --l) {
      k_up<<<blocks(N(u[l]) / 8), 256, 0, st>>>(dec->d, u[l].d, nb * u[l].h, u[l].w, u[l].c);
      const Conv& c1 = convs[ci++];
      conv(u[l], c1.wb, c1.coutp, c1.cout, param + c1.boff, 1, c[l].d, nullptr, 0);
      k_add<<<blocks(N(e[l]) / 8), 256, 0, st>>>(c[l].d, s[l].d, e[l].d, N(e[l]));
      const Conv& c2 = convs[ci++];
      conv(e[l], c2.wb, c2.coutp, c2.cout, param + c2.boff, 1, d[l].d, nullptr, 0);
      dec = &d[l];
    }
    const Conv& hd = convs[ci++];
    conv(*dec, hd.wb, hd.coutp, hd.cout, param + hd.boff, 0, nullptr, out_f, 2);
  }

  // Backward of conv `cv` whose input is `in` and (post-activation) output
  // `out`: dpost -> (ReLU mask) -> wgrad (+bias grad) -> dgrad into din.
  void conv_bwd(const Conv& cv, const Tensor& in, const bf16* out, const bf16* dpost, bf16* dpre_scratch, bf16* din) {
    const size_t nout = (size_t)nb * in.h * in.w * cv.coutp;
    const bf16* dpre = dpost;
    if (cv.relu) {
      k_relu_bwd<<<blocks(nout / 8), 256, 0, st>>>(out, dpost, dpre_scratch, nout);
      dpre = dpre_scratch;
    }
    wgrad(in, dpre, cv.coutp, wscratch, grad + cv.boff, cv.cout);
    k_wgrad_scatter<<<blocks((size_t)cv.cout * 9 * cv.cin), 256, 0, st>>>(wscratch, cv.cout, cv.cin, cv.coutp,
                                                                          cv.cinp, grad + cv.woff);
    if (din) {
      Tensor dp;
      dp.d = const_cast<bf16*>(dpre);
      dp.h = in.h;
      dp.w = in.w;
      dp.c = cv.coutp;
      conv(dp, cv.wt, cv.cinp, cv.cinp, nullptr, 0, din, nullptr, 0);
    }
  }

  // Loss + gradients (accumulated into grad, which is zeroed first).
  void backward(const float* target) {
    const int npix = H * W;
    cudaMemsetAsync(grad, 0, sizeof(float) * nparam, st);
    cudaMemsetAsync(loss, 0, sizeof(double), st);
    k_loss<<<blocks((size_t)nb * npix * 16), 256, 0, st>>>(out_f, target, npix, nb, 2, 16, dhead.d, loss);
    int ci = (int)convs.size() - 1;
    // head
    const Tensor* dec = levels > 1 ? &d[0] : &s[0];
    conv_bwd(convs[ci--], *dec, nullptr, dhead.d, nullptr, g1[0].d);  // g1[0] = d(dec)
    bf16* gcur = g1[0].d;  // gradient w.r.t. the current decoder output
    for (int l = 0; l <= levels - 2; ++l) {
      // d[l] = relu(conv(e[l])) ; e[l] = c[l] + s[l] ; c[l] = relu(conv(u[l])) ; u[l] = up(dec_{l+1})
      conv_bwd(convs[ci--], e[l], d[l].d, gcur, g2[l].d, g3[l].d);  // g3 = d e[l]
      // skip: d s[l] gets d e[l] (added below); c[l] branch:
      conv_bwd(convs[ci--], u[l], c[l].d, g3[l].d, g2[l].d, g1[l].d);  // g1[l] = d u[l] (channels base<<(l+1))
      // up backward -> gradient of the coarser decoder output (or s[levels-1])
      bf16* gnext = g1[l + 1].d;
      k_up_bwd<<<blocks((size_t)nb * (H >> (l + 1)) * (W >> (l + 1)) * (base << (l + 1))), 256, 0, st>>>(
          g1[l].d, gnext, nb * (H >> l), W >> l, base << (l + 1));
      // stash d e[l] for the encoder skip in g3[l] (kept), continue with gnext
      gcur = gnext;
    }
    // encoder, deepest level first; gcur = d s[levels-1]
    for (int l = levels - 1; l >= 0; --l) {
      // s[l] = relu(conv(a[l])), a[l] = relu(conv(in_l)), in_l = p[l-1] or x0
      bf16* ds = gcur;
      if (l < levels - 1) {
        // d s[l] = pool_bwd(d p[l]) + d e[l] (the skip, stashed in g3[l]);
        // d p[l] sits in g2[l], so the result goes to g1[l]
        k_pool_bwd<<<blocks(N(s[l])), 256, 0, st>>>(gcur, g1[l].d, nb * s[l].h, s[l].w, s[l].c);
        k_add<<<blocks(N(s[l]) / 8), 256, 0, st>>>(g1[l].d, g3[l].d, g1[l].d, N(s[l]));
        ds = g1[l].d;
      }
      const int cs = 2 * l + 1, ca = 2 * l;
      conv_bwd(convs[cs], a[l], s[l].d, ds, g2[l].d, g3[l].d);  // g3 = d a[l]
      const Tensor& inl = l > 0 ? p[l - 1] : x0;
      bf16* dprev = l > 0 ? g2[l - 1].d : nullptr;  // d p[l-1] (dimensions of level l)
      // level-l sized scratch for the relu mask of conv ca: reuse g1[l]
      conv_bwd(convs[ca], inl, a[l].d, g3[l].d, g1[l].d, dprev);
      gcur = dprev;
      (void)ci;
    }
  }

  static constexpr float kB1 = 0.9f, kB2 = 0.999f;
  // Adam's step number, lr and bias corrections into device memory (before
  // the step's kernels, outside any graph).
  void adam_hyper(float lr) {
    ++steps;
    hyper_h[0] = lr;
    hyper_h[1] = 1.f - std::pow(kB1, (float)steps);
    hyper_h[2] = 1.f - std::pow(kB2, (float)steps);
    cudaMemcpyAsync(hyper, hyper_h, sizeof(hyper_h), cudaMemcpyHostToDevice, st);
  }
  void adam() {
    k_adam<<<blocks(nparam), 256, 0, st>>>(param, grad, adam_m, adam_v, nparam, hyper, kB1, kB2, 1e-8f);
    refresh_weights();
  }
  void step_kernels() {
    forward(in_stage);
    backward(tgt_stage);
    adam();
  }
  // One training step on device inputs [nb][3][H][W] and targets
  // [nb][2][H][W] (FP32, planar).  The first step of a batch size runs
  // plain launches (it also sets the kernels' attributes); the second is
  // captured into a graph, which the later steps replay.  A capture that
  // fails falls back to plain launches for good.
  void train_step(const float* in_dev, const float* tgt_dev, float lr) {
    const size_t npix = (size_t)H * W;
    cudaMemcpyAsync(in_stage, in_dev, sizeof(float) * 3 * npix * nb, cudaMemcpyDeviceToDevice, st);
    cudaMemcpyAsync(tgt_stage, tgt_dev, sizeof(float) * 2 * npix * nb, cudaMemcpyDeviceToDevice, st);
    adam_hyper(lr);
    if (graph_ok_ && tgraph && tgraph_nb == nb) {
      cudaGraphLaunch(tgraph, st);
      return;
    }
    if (graph_ok_ && tgraph_nb == -nb) {  // second step of this batch size: capture
      if (tgraph) cudaGraphExecDestroy(tgraph);
      tgraph = nullptr;
      cudaGraph_t g = nullptr;
      if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
        step_kernels();
        if (cudaStreamEndCapture(st, &g) == cudaSuccess && g && cudaGraphInstantiate(&tgraph, g, 0) == cudaSuccess) {
          tgraph_nb = nb;
        } else {
          tgraph = nullptr;
          graph_ok_ = false;
        }
        if (g) cudaGraphDestroy(g);
      } else {
        graph_ok_ = false;
      }
      cudaGetLastError();
      if (tgraph) {
        cudaGraphLaunch(tgraph, st);
        return;
      }
    }
    step_kernels();
    if (graph_ok_ && tgraph_nb != nb) tgraph_nb = -nb;
  }

  int check() {
    int h = 0;
    cudaError_t e = cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
      set_error(std::string("vk_nn: ") + cudaGetErrorString(e));
      return VK_E_CUDA;
    }
    if (h) {
      set_error("vk_nn: a tensor-core wait timed out");
      return VK_E_CUDA;
    }
    return VK_OK;
  }
};

}  // namespace nn
}  // namespace vk

// ------------------------------------------------------------------ C ABI --
using vk::set_error;
using vk::nn::Net;

namespace {
constexpr uint32_t kNetMagic = 0x4e4e4554u;
struct NetCtx {
  uint32_t magic;
  Net* n;
};
Net* as_net(void* h) {
  NetCtx* c = static_cast<NetCtx*>(h);
  if (!c || c->magic != kNetMagic || !c->n) {
    set_error("invalid network handle");
    return nullptr;
  }
  return c->n;
}
}  // namespace

extern "C" int vk_nn_create(int32_t h, int32_t w, int32_t base, int32_t levels, uint64_t seed, void** net) {
  return vk_nn_create_batched(h, w, base, levels, 1, seed, net);
}

extern "C" int vk_nn_create_batched(int32_t h, int32_t w, int32_t base, int32_t levels, int32_t batch_cap,
                                    uint64_t seed, void** net) {
  if (!net || batch_cap < 1 || batch_cap > 64 || h <= 0 || w <= 0 || base < 16 || base % 16 || levels < 1 || levels > 5 || (h >> (levels - 1)) < 2 ||
      (w >> (levels - 1)) < 2 || (h % (1 << (levels - 1))) || (w % (1 << (levels - 1))) || (base << (levels - 1)) > 256) {
    set_error("vk_nn_create: need h, w divisible by 2^(levels-1), base a multiple of 16, base*2^(levels-1) <= 256, "
              "batch capacity 1..64");
    return VK_E_INVALID;
  }
  *net = nullptr;
  Net* n = new Net();
  const int rc = n->init(h, w, base, levels, seed, batch_cap);
  if (rc != VK_OK) {
    delete n;
    set_error("vk_nn_create: allocation failed");
    return rc;
  }
  *net = new NetCtx{kNetMagic, n};
  return n->check();
}

extern "C" int vk_nn_set_batch(void* net, int32_t batch) {
  Net* x = as_net(net);
  if (!x) return VK_E_INVALID;
  if (batch < 1 || batch > x->bcap) { set_error("vk_nn_set_batch: batch outside 1..capacity"); return VK_E_INVALID; }
  x->nb = batch;
  return VK_OK;
}

extern "C" int vk_nn_features(void* net, const double* psi_host, const double* pos_host, int32_t n_vort,
                              double width, float* out_dev) {
  Net* x = as_net(net);
  if (!x || !psi_host || !out_dev || (n_vort > 0 && !pos_host) || n_vort < 0 || n_vort > Net::kMaxVortices ||
      !(width > 0)) {
    set_error("vk_nn_features: bad argument (null pointer, vortex count outside 0..4096 or width <= 0)");
    return VK_E_INVALID;
  }
  const int npix = x->H * x->W;
  cudaMemcpyAsync(x->feat_psi, psi_host, sizeof(double2) * npix, cudaMemcpyHostToDevice, x->st);
  if (n_vort > 0) {
    cudaMemcpyAsync(x->feat_pos, pos_host, sizeof(double) * 2 * n_vort, cudaMemcpyHostToDevice, x->st);
    vk::nn::k_feat_tables<<<Net::blocks((size_t)n_vort * (x->W + x->H)), 256, 0, x->st>>>(
        x->feat_pos, n_vort, x->H, x->W, 1.0 / (2.0 * width * width), x->feat_gx, x->feat_gy);
  }
  vk::nn::k_features<<<Net::blocks((size_t)npix), 256, 0, x->st>>>(x->feat_psi, x->feat_gx, x->feat_gy, n_vort,
                                                                    x->H, x->W, out_dev);
  return x->check();
}

extern "C" int vk_nn_destroy(void* net) {
  NetCtx* c = static_cast<NetCtx*>(net);
  if (!as_net(net)) return VK_E_INVALID;
  delete c->n;
  c->magic = 0;
  delete c;
  return VK_OK;
}

extern "C" int vk_nn_num_params(void* net, int64_t* n) {
  Net* x = as_net(net);
  if (!x || !n) return VK_E_INVALID;
  *n = (int64_t)x->nparam;
  return VK_OK;
}

extern "C" int vk_nn_get_params(void* net, float* host, int64_t n) {
  Net* x = as_net(net);
  if (!x || !host || n != (int64_t)x->nparam) { set_error("vk_nn_get_params: bad buffer"); return VK_E_INVALID; }
  cudaMemcpyAsync(host, x->param, sizeof(float) * n, cudaMemcpyDeviceToHost, x->st);
  return x->check();
}

extern "C" int vk_nn_set_params(void* net, const float* host, int64_t n) {
  Net* x = as_net(net);
  if (!x || !host || n != (int64_t)x->nparam) { set_error("vk_nn_set_params: bad buffer"); return VK_E_INVALID; }
  cudaMemcpyAsync(x->param, host, sizeof(float) * n, cudaMemcpyHostToDevice, x->st);
  x->refresh_weights();
  return x->check();
}

// in_dev: device FP32 [3][h][w]; out_dev: device FP32 [2][h][w] (planar).
extern "C" int vk_nn_forward(void* net, const float* in_dev, float* out_dev, void* stream) {
  Net* x = as_net(net);
  if (!x || !in_dev || !out_dev) { set_error("vk_nn_forward: null argument"); return VK_E_INVALID; }
  (void)stream;
  x->forward(in_dev);
  const int npix = x->H * x->W;
  vk::nn::k_planar2<<<Net::blocks((size_t)x->nb * npix), 256, 0, x->st>>>(x->out_f, out_dev, npix, x->nb);
  return x->check();
}

// Loss and the full parameter gradient (grad_host may be NULL).
extern "C" int vk_nn_loss_grad(void* net, const float* in_dev, const float* target_dev, double* loss_out,
                               float* grad_host) {
  Net* x = as_net(net);
  if (!x || !in_dev || !target_dev) { set_error("vk_nn_loss_grad: null argument"); return VK_E_INVALID; }
  x->forward(in_dev);
  x->backward(target_dev);
  if (grad_host) cudaMemcpyAsync(grad_host, x->grad, sizeof(float) * x->nparam, cudaMemcpyDeviceToHost, x->st);
  if (loss_out) cudaMemcpyAsync(loss_out, x->loss, sizeof(double), cudaMemcpyDeviceToHost, x->st);
  return x->check();
}

// One Adam step on the MSE loss of the current batch.  Returns with the
// network's stream synchronised, so the caller may reuse the input buffers.
extern "C" int vk_nn_train_step(void* net, const float* in_dev, const float* target_dev, float lr, double* loss_out) {
  Net* x = as_net(net);
  if (!x || !in_dev || !target_dev) { set_error("vk_nn_train_step: null argument"); return VK_E_INVALID; }
  x->train_step(in_dev, target_dev, lr);
  if (loss_out) cudaMemcpyAsync(loss_out, x->loss, sizeof(double), cudaMemcpyDeviceToHost, x->st);
  return x->check();
}
