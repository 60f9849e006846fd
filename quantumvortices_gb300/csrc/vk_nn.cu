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
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>
#include "../../include/vk.h"
#include "vk_solver.h"
#include "vk_tc.cuh"

namespace vk {
namespace nn {

typedef __nv_bfloat16 bf16;

__device__ __forceinline__ int wrapi(int v, int n) { return v < 0 ? v + n : (v >= n ? v - n : v); }

// ------------------------------------------------------------------ conv --
// One CTA = 128 output pixels x BN channels.  CK = K columns per chunk.
template <int BN>
__global__ void __launch_bounds__(128) k_conv(const bf16* __restrict__ in, int H, int W, int Cin,
                                              const bf16* __restrict__ wgt, const float* __restrict__ bias, int relu,
                                              bf16* __restrict__ out_bf, float* __restrict__ out_f, int nout,
                                              int* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char sm[];
  const int CK = Cin < 64 ? Cin : 64;
  unsigned char* sA = sm;                        // 128 x CK
  unsigned char* sB = sm + 128 * 64 * 2;         // BN x CK
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tslot;
  const int tid = threadIdx.x, warp = tid >> 5;
  const int npix = H * W;
  const int p0 = blockIdx.x * 128;
  constexpr uint32_t NCOL = BN < 32 ? 32 : BN;
  if (warp == 0) tc::tmem_alloc(&tslot, NCOL);
  if (tid == 0) tc::mbar_init(&bar);
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t taddr = tslot;
  const uint32_t idesc = tc::idesc_bf16(128, BN);
  uint32_t phase = 0;
  bool first = true;
  const int vpr = CK / 8;  // 16-byte vectors per tile row
  for (int tap = 0; tap < 9; ++tap) {
    const int dy = tap / 3 - 1, dx = tap % 3 - 1;
    for (int c0 = 0; c0 < Cin; c0 += CK) {
      for (int i = tid; i < 128 * vpr; i += 128) {
        const int r = i / vpr, kv = i % vpr;
        const int p = p0 + r;
        uint4 v = make_uint4(0, 0, 0, 0);
        if (p < npix) {
          const int y = p / W, x = p % W;
          const int src = wrapi(y + dy, H) * W + wrapi(x + dx, W);
          v = *reinterpret_cast<const uint4*>(in + (size_t)src * Cin + c0 + 8 * kv);
        }
        *reinterpret_cast<uint4*>(sA + tc::tile_off(r, 8 * kv, CK)) = v;
      }
      for (int i = tid; i < BN * vpr; i += 128) {
        const int r = i / vpr, kv = i % vpr;
        const uint4 v = *reinterpret_cast<const uint4*>(wgt + ((size_t)r * 9 + tap) * Cin + c0 + 8 * kv);
        *reinterpret_cast<uint4*>(sB + tc::tile_off(r, 8 * kv, CK)) = v;
      }
      tc::fence_async_smem();
      tc::fence_before();
      __syncthreads();
      tc::fence_after();
      if (tid == 0) {
        for (int j = 0; j < CK / 16; ++j) {
          const uint64_t ad = tc::smem_desc(tc::smem_u32(sA) + j * 256, 128, (CK / 8) * 128);
          const uint64_t bd = tc::smem_desc(tc::smem_u32(sB) + j * 256, 128, (CK / 8) * 128);
          tc::mma(taddr, ad, bd, idesc, first ? 0u : 1u);
          first = false;
        }
        tc::commit(&bar);
      }
      tc::mbar_wait(&bar, phase, err);
      phase ^= 1;
      tc::fence_after();
    }
  }
  // epilogue
  const int r = 32 * warp + (tid & 31);
  const int p = p0 + r;
  for (int c0 = 0; c0 < BN; c0 += (BN < 32 ? 16 : 32)) {
    float v[32];
    const uint32_t ta = taddr + ((uint32_t)(32 * warp) << 16) + c0;
    if (BN < 32) tc::tmem_ld16(ta, v);
    else tc::tmem_ld32(ta, v);
    const int nc = BN < 32 ? 16 : 32;
    if (p < npix) {
      for (int j = 0; j < nc; ++j) {
        const int c = c0 + j;
        float a = v[j] + (bias ? bias[c] : 0.f);
        if (relu) a = fmaxf(a, 0.f);
        if (out_bf) out_bf[(size_t)p * BN + c] = __float2bfloat16(a);
        if (out_f && c < nout) out_f[(size_t)p * nout + c] = a;
      }
    }
  }
  tc::fence_before();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(taddr, NCOL);
}

// Weight gradient: rows m = tap*Cin + ci (tile of 128), columns = BN output
// channels, reduction over this CTA's pixel range (chunks of 64 pixels).
template <int BN>
__global__ void __launch_bounds__(128) k_wgrad(const bf16* __restrict__ in, const bf16* __restrict__ dy, int H, int W,
                                               int Cin, int pix_per_cta, float* __restrict__ dW,
                                               int* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char sm[];
  unsigned char* sA = sm;                 // 128 x 64
  unsigned char* sB = sm + 128 * 64 * 2;  // BN x 64
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tslot;
  const int tid = threadIdx.x, warp = tid >> 5;
  const int npix = H * W, M = 9 * Cin;
  const int m0 = blockIdx.x * 128;
  const int q0 = blockIdx.y * pix_per_cta, q1 = min(npix, q0 + pix_per_cta);
  constexpr uint32_t NCOL = BN < 32 ? 32 : BN;
  if (warp == 0) tc::tmem_alloc(&tslot, NCOL);
  if (tid == 0) tc::mbar_init(&bar);
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t taddr = tslot;
  const uint32_t idesc = tc::idesc_bf16(128, BN);
  uint32_t phase = 0;
  bool first = true;
  for (int k0 = q0; k0 < q1; k0 += 64) {
    for (int i = tid; i < 128 * 64; i += 128) {
      const int r = i % 128, k = i / 128;
      const int m = m0 + r, q = k0 + k;
      bf16 v = __float2bfloat16(0.f);
      if (m < M && q < q1) {
        const int tap = m / Cin, ci = m % Cin;
        const int y = q / W, x = q % W;
        const int src = wrapi(y + tap / 3 - 1, H) * W + wrapi(x + tap % 3 - 1, W);
        v = in[(size_t)src * Cin + ci];
      }
      *reinterpret_cast<bf16*>(sA + tc::tile_off(r, k, 64)) = v;
    }
    for (int i = tid; i < BN * 64; i += 128) {
      const int c = i % BN, k = i / BN;
      const int q = k0 + k;
      const bf16 v = q < q1 ? dy[(size_t)q * BN + c] : __float2bfloat16(0.f);
      *reinterpret_cast<bf16*>(sB + tc::tile_off(c, k, 64)) = v;
    }
    tc::fence_async_smem();
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    if (tid == 0) {
      for (int j = 0; j < 4; ++j) {
        const uint64_t ad = tc::smem_desc(tc::smem_u32(sA) + j * 256, 128, 8 * 128);
        const uint64_t bd = tc::smem_desc(tc::smem_u32(sB) + j * 256, 128, 8 * 128);
        tc::mma(taddr, ad, bd, idesc, first ? 0u : 1u);
        first = false;
      }
      tc::commit(&bar);
    }
    tc::mbar_wait(&bar, phase, err);
    phase ^= 1;
    tc::fence_after();
  }
  const int r = 32 * warp + (tid & 31);
  const int m = m0 + r;
  if (q1 > q0) {  // CTA-uniform: every warp runs the collective TMEM loads
    for (int c0 = 0; c0 < BN; c0 += (BN < 32 ? 16 : 32)) {
      float v[32];
      const uint32_t ta = taddr + ((uint32_t)(32 * warp) << 16) + c0;
      if (BN < 32) tc::tmem_ld16(ta, v);
      else tc::tmem_ld32(ta, v);
      const int nc = BN < 32 ? 16 : 32;
      if (m < M)
        for (int j = 0; j < nc; ++j) atomicAdd(&dW[(size_t)m * BN + c0 + j], v[j]);
    }
  }
  tc::fence_before();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(taddr, NCOL);
}

// ------------------------------------------------------------ elementwise --

__global__ void k_pack_input(const float* __restrict__ in, bf16* __restrict__ out, int npix, int cin, int cpad) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < npix * cpad; i += gridDim.x * blockDim.x) {
    const int p = i / cpad, c = i % cpad;
    out[i] = __float2bfloat16(c < cin ? in[(size_t)c * npix + p] : 0.f);
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
  // out is H x W, in is H/2 x W/2
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < H * W * C; i += gridDim.x * blockDim.x) {
    const int c = i % C, p = i / C, y = p / W, x = p % W;
    out[i] = in[((size_t)(y / 2) * (W / 2) + x / 2) * C + c];
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
__global__ void k_add(const bf16* __restrict__ a, const bf16* __restrict__ b, bf16* __restrict__ o, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    o[i] = __float2bfloat16(__bfloat162float(a[i]) + __bfloat162float(b[i]));
}
// d_pre = d_post * (y > 0)
__global__ void k_relu_bwd(const bf16* __restrict__ y, const bf16* __restrict__ d, bf16* __restrict__ o, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    o[i] = __bfloat162float(y[i]) > 0.f ? d[i] : __float2bfloat16(0.f);
}
// bias gradient: db[c] += sum_p d[p][c] for the cout real channels (stride cs)
__global__ void k_bias_grad(const bf16* __restrict__ d, int npix, int cs, int cout, float* __restrict__ db) {
  for (int c = blockIdx.x; c < cout; c += gridDim.x) {
    float s = 0.f;
    for (int p = threadIdx.x; p < npix; p += blockDim.x) s += __bfloat162float(d[(size_t)p * cs + c]);
    __shared__ float red[256];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
      if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
      __syncthreads();
    }
    if (threadIdx.x == 0) atomicAdd(&db[c], red[0]);
    __syncthreads();
  }
}
// MSE loss on the head output (FP32 [p][nout]) against planar targets
// [nout][p]; writes the BF16 gradient [p][cpad] and accumulates the loss.
__global__ void k_loss(const float* __restrict__ out, const float* __restrict__ tgt, int npix, int nout, int cpad,
                       bf16* __restrict__ dout, double* __restrict__ loss) {
  const float inv = 1.f / (float)(npix * nout);
  double acc = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < npix * cpad; i += gridDim.x * blockDim.x) {
    const int p = i / cpad, c = i % cpad;
    float g = 0.f;
    if (c < nout) {
      const float e = out[(size_t)p * nout + c] - tgt[(size_t)c * npix + p];
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
// [p][2] -> planar [2][p]
__global__ void k_planar2(const float* __restrict__ in, float* __restrict__ out, int npix) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < npix; p += gridDim.x * blockDim.x) {
    out[p] = in[2 * p];
    out[npix + p] = in[2 * p + 1];
  }
}
__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                       size_t n, float lr, float b1, float b2, float c1, float c2, float eps) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi, vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

// ------------------------------------------------------------- network --

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
  cudaStream_t st = nullptr;
  std::vector<void*> allocs;
  // activations (forward) per level and gradient scratch
  Tensor x0;
  std::vector<Tensor> a, s, p, u, c, e, d;   // see forward()
  Tensor b4;
  std::vector<Tensor> g1, g2, g3;             // gradient scratch per level (3 buffers)
  Tensor dhead;

  ~Net() {
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
    t.d = dalloc<bf16>(t.n());
    return t;
  }
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

  int init(int h, int w, int base_ch, int nlev, uint64_t seed) {
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
    out_f = dalloc<float>((size_t)H * W * 2);
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
  void conv(const Tensor& in, const Conv& cv, const bf16* w, int cout_p, const float* bias, int relu, bf16* out_bf,
            float* out_f32, int nout) {
    const int npix = in.h * in.w;
    const int grid = (npix + 127) / 128;
    const size_t smem = 128 * 64 * 2 + (size_t)cout_p * 64 * 2;
    switch (cout_p) {
      case 16: launch_conv<16>(grid, smem, in, w, bias, relu, out_bf, out_f32, nout); break;
      case 32: launch_conv<32>(grid, smem, in, w, bias, relu, out_bf, out_f32, nout); break;
      case 64: launch_conv<64>(grid, smem, in, w, bias, relu, out_bf, out_f32, nout); break;
      case 128: launch_conv<128>(grid, smem, in, w, bias, relu, out_bf, out_f32, nout); break;
      default: launch_conv<256>(grid, smem, in, w, bias, relu, out_bf, out_f32, nout); break;
    }
    (void)cv;
  }
  template <int BN>
  void launch_conv(int grid, size_t smem, const Tensor& in, const bf16* w, const float* bias, int relu, bf16* ob,
                   float* of, int nout) {
    static bool attr = false;
    if (!attr) {
      cudaFuncSetAttribute(k_conv<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, 128 * 64 * 2 + 256 * 64 * 2);
      attr = true;
    }
    k_conv<BN><<<grid, 128, smem, st>>>(in.d, in.h, in.w, in.c, w, bias, relu, ob, of, nout, err);
  }
  void wgrad(const Tensor& in, const bf16* dy, int coutp, float* out) {
    const int npix = in.h * in.w, M = 9 * in.c;
    const int mt = (M + 127) / 128;
    int ppc = 4096;
    while ((npix + ppc - 1) / ppc * mt < 2 * 152 && ppc > 256) ppc /= 2;
    dim3 grid(mt, (npix + ppc - 1) / ppc);
    const size_t smem = 128 * 64 * 2 + (size_t)coutp * 64 * 2;
    cudaMemsetAsync(out, 0, sizeof(float) * (size_t)M * coutp, st);
    switch (coutp) {
      case 16: launch_wgrad<16>(grid, smem, in, dy, ppc, out); break;
      case 32: launch_wgrad<32>(grid, smem, in, dy, ppc, out); break;
      case 64: launch_wgrad<64>(grid, smem, in, dy, ppc, out); break;
      case 128: launch_wgrad<128>(grid, smem, in, dy, ppc, out); break;
      default: launch_wgrad<256>(grid, smem, in, dy, ppc, out); break;
    }
  }
  template <int BN> void launch_wgrad(dim3 grid, size_t smem, const Tensor& in, const bf16* dy, int ppc, float* out) {
    static bool attr = false;
    if (!attr) {
      cudaFuncSetAttribute(k_wgrad<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, 128 * 64 * 2 + 256 * 64 * 2);
      attr = true;
    }
    k_wgrad<BN><<<grid, 128, smem, st>>>(in.d, dy, in.h, in.w, in.c, ppc, out, err);
  }
  static int blocks(size_t n) { return (int)std::min<size_t>((n + 255) / 256, 152 * 16); }

  // Forward pass; returns the head output in out_f [p][2].
  void forward(const float* input) {
    const int npix = H * W;
    k_pack_input<<<blocks((size_t)npix * 16), 256, 0, st>>>(input, x0.d, npix, 3, 16);
    int ci = 0;
    const Tensor* cur = &x0;
    for (int l = 0; l < levels; ++l) {
      const Conv& c1 = convs[ci++];
      conv(*cur, c1, c1.wb, c1.coutp, param + c1.boff, 1, a[l].d, nullptr, 0);
      const Conv& c2 = convs[ci++];
      conv(a[l], c2, c2.wb, c2.coutp, param + c2.boff, 1, s[l].d, nullptr, 0);
      if (l + 1 < levels) {
        k_pool<<<blocks(p[l].n()), 256, 0, st>>>(s[l].d, p[l].d, s[l].h, s[l].w, s[l].c);
        cur = &p[l];
      }
    }
    const Tensor* dec = &s[levels - 1];
    for (int l = levels - 2; l >= 0; --l) {
      k_up<<<blocks(u[l].n()), 256, 0, st>>>(dec->d, u[l].d, u[l].h, u[l].w, u[l].c);
      const Conv& c1 = convs[ci++];
      conv(u[l], c1, c1.wb, c1.coutp, param + c1.boff, 1, c[l].d, nullptr, 0);
      k_add<<<blocks(e[l].n()), 256, 0, st>>>(c[l].d, s[l].d, e[l].d, e[l].n());
      const Conv& c2 = convs[ci++];
      conv(e[l], c2, c2.wb, c2.coutp, param + c2.boff, 1, d[l].d, nullptr, 0);
      dec = &d[l];
    }
    const Conv& hd = convs[ci++];
    conv(*dec, hd, hd.wb, hd.coutp, param + hd.boff, 0, nullptr, out_f, 2);
  }

  // Backward of conv `cv` whose input is `in` and (post-activation) output
  // `out`: dpost -> (ReLU mask) -> wgrad (+bias grad) -> dgrad into din.
  void conv_bwd(const Conv& cv, const Tensor& in, const bf16* out, const bf16* dpost, bf16* dpre_scratch, bf16* din) {
    const size_t nout = (size_t)in.h * in.w * cv.coutp;
    const bf16* dpre = dpost;
    if (cv.relu) {
      k_relu_bwd<<<blocks(nout), 256, 0, st>>>(out, dpost, dpre_scratch, nout);
      dpre = dpre_scratch;
    }
    wgrad(in, dpre, cv.coutp, wscratch);
    k_wgrad_scatter<<<blocks((size_t)cv.cout * 9 * cv.cin), 256, 0, st>>>(wscratch, cv.cout, cv.cin, cv.coutp,
                                                                          cv.cinp, grad + cv.woff);
    k_bias_grad<<<std::min(cv.cout, 256), 256, 0, st>>>(dpre, in.h * in.w, cv.coutp, cv.cout, grad + cv.boff);
    if (din) {
      Tensor dp;
      dp.d = const_cast<bf16*>(dpre);
      dp.h = in.h;
      dp.w = in.w;
      dp.c = cv.coutp;
      conv(dp, cv, cv.wt, cv.cinp, nullptr, 0, din, nullptr, 0);
    }
  }

  // Loss + gradients (accumulated into grad, which is zeroed first).
  void backward(const float* target) {
    const int npix = H * W;
    cudaMemsetAsync(grad, 0, sizeof(float) * nparam, st);
    cudaMemsetAsync(loss, 0, sizeof(double), st);
    k_loss<<<blocks((size_t)npix * 16), 256, 0, st>>>(out_f, target, npix, 2, 16, dhead.d, loss);
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
      k_up_bwd<<<blocks((size_t)(H >> (l + 1)) * (W >> (l + 1)) * (base << (l + 1))), 256, 0, st>>>(
          g1[l].d, gnext, H >> l, W >> l, base << (l + 1));
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
        k_pool_bwd<<<blocks(s[l].n()), 256, 0, st>>>(gcur, g1[l].d, s[l].h, s[l].w, s[l].c);
        k_add<<<blocks(s[l].n()), 256, 0, st>>>(g1[l].d, g3[l].d, g1[l].d, s[l].n());
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

  void adam(float lr) {
    ++steps;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - std::pow(b1, (float)steps), c2 = 1.f - std::pow(b2, (float)steps);
    k_adam<<<blocks(nparam), 256, 0, st>>>(param, grad, adam_m, adam_v, nparam, lr, b1, b2, c1, c2, 1e-8f);
    refresh_weights();
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
  if (!net || h <= 0 || w <= 0 || base < 16 || base % 16 || levels < 1 || levels > 5 || (h >> (levels - 1)) < 2 ||
      (w >> (levels - 1)) < 2 || (h % (1 << (levels - 1))) || (w % (1 << (levels - 1))) || (base << (levels - 1)) > 256) {
    set_error("vk_nn_create: need h, w divisible by 2^(levels-1), base a multiple of 16, base*2^(levels-1) <= 256");
    return VK_E_INVALID;
  }
  *net = nullptr;
  Net* n = new Net();
  const int rc = n->init(h, w, base, levels, seed);
  if (rc != VK_OK) {
    delete n;
    set_error("vk_nn_create: allocation failed");
    return rc;
  }
  *net = new NetCtx{kNetMagic, n};
  return n->check();
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
  vk::nn::k_planar2<<<Net::blocks((size_t)npix), 256, 0, x->st>>>(x->out_f, out_dev, npix);
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

// One Adam step on the MSE loss of one sample.
extern "C" int vk_nn_train_step(void* net, const float* in_dev, const float* target_dev, float lr, double* loss_out) {
  Net* x = as_net(net);
  if (!x || !in_dev || !target_dev) { set_error("vk_nn_train_step: null argument"); return VK_E_INVALID; }
  x->forward(in_dev);
  x->backward(target_dev);
  x->adam(lr);
  if (loss_out) {
    cudaMemcpyAsync(loss_out, x->loss, sizeof(double), cudaMemcpyDeviceToHost, x->st);
    return x->check();
  }
  return VK_OK;
}
