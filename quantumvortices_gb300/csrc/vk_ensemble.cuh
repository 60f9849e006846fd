// vk_ensemble.cuh -- batched RK4 over an ensemble of independent fields of
// uneven sizes (128, 256, 512 or 1024 points per side).
//
// Every pass of the single-field stepper (X1, Y1, X2, Y2 and the final
// F^-1_x) becomes one persistent kernel over a work list of (member, row
// tile) items for ALL members: a CTA walks items blockIdx.x, +gridDim.x, ...
// and runs the same device body as the single-field kernel with that
// member's buffers.  Tiles hold RL points (R = RL/L rows), so items of
// different sizes cost about the same and a static stride balances.  One
// RK4 step (16 persistent launches) is captured as one CUDA graph.
//
// Autotuner: at set-up it times, on the (still zero) ensemble buffers, every
// compiled tile variant (x passes RL = 2048 or 4096 points, y passes
// RL = 1024 or 2048, each also with the registers capped for more CTAs per
// SM) at 1, 2, 4 and 8 CTAs per SM, per pass kind, and keeps the fastest.
// It then times one RK4 step of those four pass kernels per stage against
// one persistent kernel per stage (kb_stage: the four pass loops in one
// cooperative launch, bounded grid-wide barriers between them) and steps
// with the faster.
#pragma once
#include <algorithm>
#include <string>
#include <vector>
#include "vk_kernels.cuh"
#include "vk_solver.h"
#include "vk_stage.cuh"
#include <type_traits>

namespace vk {

template <typename T, int LL, int RL> struct GeoB {
  static constexpr int L = LL, R = RL / LL, LP = padded(LL), MINB = 2;
  static constexpr int NT = RL / 16;
};

#define VK_ENS_SWITCH(N, BODY)                      \
  switch (N) {                                      \
    case 128: { constexpr int L = 128; BODY; } break; \
    case 256: { constexpr int L = 256; BODY; } break; \
    case 512: { constexpr int L = 512; BODY; } break; \
    case 1024: { constexpr int L = 1024; BODY; } break; \
    default: break;                                 \
  }

// MB > 1: the compiler keeps the registers low enough for MB CTAs per SM
// (a variant the autotuner times against the uncapped one).
template <typename T, int RL, bool FROM_T, int MB = 1>
__global__ void __launch_bounds__(RL / 16, MB) kb_x1(const Field<T>* __restrict__ F, const int2* __restrict__ items, int n) {
  extern __shared__ __align__(16) unsigned char smraw[];
  cplx<T>* s = reinterpret_cast<cplx<T>*>(smraw);
  for (int it = blockIdx.x; it < n; it += gridDim.x) {
    const int2 w = items[it];
    const Field<T>& f = F[w.x];
    VK_ENS_SWITCH(f.c.nx, (x1_body<T, L, GeoB<T, L, RL>, FROM_T, true>(f.Ta, f.psi, f.Tb, f.twx, f.c, w.y, s)));
    __syncthreads();
  }
}

template <typename T, int RL, int MB = 1>
__global__ void __launch_bounds__(RL / 16, MB) kb_y1(const Field<T>* __restrict__ F, const int2* __restrict__ items, int n) {
  extern __shared__ __align__(16) unsigned char smraw[];
  cplx<T>* s = reinterpret_cast<cplx<T>*>(smraw);
  for (int it = blockIdx.x; it < n; it += gridDim.x) {
    const int2 w = items[it];
    const Field<T>& f = F[w.x];
    VK_ENS_SWITCH(f.c.ny, (y1_body<T, L, GeoB<T, L, RL>>(f.Tb, f.Tc, f.twy, f.c, w.y, s)));
    __syncthreads();
  }
}

template <typename T, int RL, int MB = 1>
__global__ void __launch_bounds__(RL / 16, MB) kb_x2(const Field<T>* __restrict__ F, const int2* __restrict__ items, int n) {
  extern __shared__ __align__(16) unsigned char smraw[];
  cplx<T>* s = reinterpret_cast<cplx<T>*>(smraw);
  for (int it = blockIdx.x; it < n; it += gridDim.x) {
    const int2 w = items[it];
    const Field<T>& f = F[w.x];
    VK_ENS_SWITCH(f.c.nx, (x2_body<T, L, GeoB<T, L, RL>, +1, true, false>(f.Tc, f.psi, (const T*)nullptr, f.Td,
                                                                            f.twx, f.c, w.y, s)));
    __syncthreads();
  }
}

template <typename T, int RL, int STAGE, int MB = 1>
__global__ void __launch_bounds__(RL / 16, MB) kb_y2(const Field<T>* __restrict__ F, const int2* __restrict__ items, int n) {
  extern __shared__ __align__(16) unsigned char smraw[];
  cplx<T>* s = reinterpret_cast<cplx<T>*>(smraw);
  for (int it = blockIdx.x; it < n; it += gridDim.x) {
    const int2 w = items[it];
    const Field<T>& f = F[w.x];
    VK_ENS_SWITCH(f.c.ny, (y2_rk4_body<T, L, GeoB<T, L, RL>, STAGE>(f.Td, f.kpsi, f.str1, f.str2, f.Ta, f.twy, f.c,
                                                                      w.y, s)));
    __syncthreads();
  }
}

template <typename T, int RL>
__global__ void __launch_bounds__(RL / 16) kb_xinv(const Field<T>* __restrict__ F, const int2* __restrict__ items, int n) {
  extern __shared__ __align__(16) unsigned char smraw[];
  cplx<T>* s = reinterpret_cast<cplx<T>*>(smraw);
  for (int it = blockIdx.x; it < n; it += gridDim.x) {
    const int2 w = items[it];
    const Field<T>& f = F[w.x];
    VK_ENS_SWITCH(f.c.nx, (xinv_body<T, L, GeoB<T, L, RL>, true>(f.Ta, f.psi, f.twx, T(f.c.scale), f.c.K, w.y, s)));
    __syncthreads();
  }
}

// One RK4 stage of every member in one cooperative launch: the four pass
// loops of the kernels above with grid-wide barriers between them; every
// pass takes tiles of RL points, so one block size serves all four.
template <typename T, int RL, int STAGE, bool FROM_T>
__global__ void __launch_bounds__(RL / 16) kb_stage(const Field<T>* __restrict__ F, const int2* __restrict__ ix,
                                                   int nix, const int2* __restrict__ iy1, int niy1,
                                                   const int2* __restrict__ iy2, int niy2, GridBarrier* bar,
                                                   unsigned long long limit) {
  extern __shared__ __align__(16) unsigned char smraw[];
  cplx<T>* s = reinterpret_cast<cplx<T>*>(smraw);
  for (int it = blockIdx.x; it < nix; it += gridDim.x) {
    const int2 w = ix[it];
    const Field<T>& f = F[w.x];
    VK_ENS_SWITCH(f.c.nx, (x1_body<T, L, GeoB<T, L, RL>, FROM_T, true>(f.Ta, f.psi, f.Tb, f.twx, f.c, w.y, s)));
    __syncthreads();
  }
  if (!grid_sync(bar, limit, 3 * (STAGE - 1))) return;
  for (int it = blockIdx.x; it < niy1; it += gridDim.x) {
    const int2 w = iy1[it];
    const Field<T>& f = F[w.x];
    VK_ENS_SWITCH(f.c.ny, (y1_body<T, L, GeoB<T, L, RL>>(f.Tb, f.Tc, f.twy, f.c, w.y, s)));
    __syncthreads();
  }
  if (!grid_sync(bar, limit, 3 * (STAGE - 1) + 1)) return;
  for (int it = blockIdx.x; it < nix; it += gridDim.x) {
    const int2 w = ix[it];
    const Field<T>& f = F[w.x];
    VK_ENS_SWITCH(f.c.nx, (x2_body<T, L, GeoB<T, L, RL>, +1, true, false>(f.Tc, f.psi, (const T*)nullptr, f.Td,
                                                                            f.twx, f.c, w.y, s)));
    __syncthreads();
  }
  if (!grid_sync(bar, limit, 3 * (STAGE - 1) + 2)) return;
  for (int it = blockIdx.x; it < niy2; it += gridDim.x) {
    const int2 w = iy2[it];
    const Field<T>& f = F[w.x];
    VK_ENS_SWITCH(f.c.ny, (y2_rk4_body<T, L, GeoB<T, L, RL>, STAGE>(f.Td, f.kpsi, f.str1, f.str2, f.Ta, f.twy, f.c,
                                                                      w.y, s)));
    __syncthreads();
  }
}

// Pass kinds the autotuner decides separately.
enum EnsPass { EP_X1 = 0, EP_Y1, EP_X2, EP_Y2, EP_XINV, EP_N };

template <typename T>
class Ensemble {
  typedef cplx<T> C;

 public:
  std::vector<SolverBase*> owned;
  std::vector<Field<T>> fields;
  int n = 0;
  cudaStream_t st = nullptr;
  Field<T>* dF = nullptr;
  // work lists per pass kind and tile variant: [kind][variant]
  int2* dItems[EP_N][2] = {};
  int nItems[EP_N][2] = {};
  // tile variants: 0 and 1 the tile sizes below (registers uncapped), 2 the
  // tile of variant 0 with the registers capped for more CTAs per SM
  static constexpr int NVAR = 3;
  static int list_of(int v) { return v == 2 ? 0 : v; }
  int variant[EP_N] = {0, 0, 0, 0, 0};
  int grid[EP_N] = {0, 0, 0, 0, 0};
  int sms = 152;
  bool masked = false;
  cudaGraphExec_t gstep = nullptr;
  int64_t launches = 0, gstep_n = 0;
  std::string report;
  // persistent stage kernel (kb_stage, tiles of kFusedRL points)
  static constexpr int kFusedRL = 2048;
  GridBarrier* bar = nullptr;
  int fused_grid = 0;
  bool fused = false;
  unsigned long long spin_limit = 1ull << 24;

  static constexpr int XRL[2] = {2048, 4096};
  static constexpr int YRL[2] = {1024, 2048};

  int init(const vk_params* ps, int nmem) {
    n = nmem;
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    for (int m = 0; m < n; ++m) {
      const int nx = ps[m].nx, ny = ps[m].ny;
      auto ok = [](int v) { return v == 128 || v == 256 || v == 512 || v == 1024; };
      if (!ok(nx) || !ok(ny) || ps[m].n_particles != 0) {
        set_error("vk_ens_init: members need nx, ny in {128, 256, 512, 1024} and no particles");
        return VK_E_INVALID;
      }
      int rc = VK_OK;
      SolverBase* sb = std::is_same<T, double>::value ? make_solver_f64(ps[m], &rc) : make_solver_f32(ps[m], &rc);
      if (!sb) return rc ? rc : VK_E_CUDA;
      owned.push_back(sb);
      Field<T> f;
      if ((rc = sb->field_view(&f, sizeof(f)))) return rc;
      fields.push_back(f);
    }
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc(&dF, sizeof(Field<T>) * n) != cudaSuccess ||
        cudaMemcpy(dF, fields.data(), sizeof(Field<T>) * n, cudaMemcpyHostToDevice) != cudaSuccess) {
      set_error("vk_ens_init: device allocation failed");
      return VK_E_NOMEM;
    }
    int rc = build_lists();
    if (rc) return rc;
    return autotune();
  }

  ~Ensemble() {
    for (auto* o : owned) delete o;
    if (gstep) cudaGraphExecDestroy(gstep);
    for (auto& a : dItems)
      for (auto* b : a)
        if (b) cudaFree(b);
    if (dF) cudaFree(dF);
    if (bar) cudaFree(bar);
    if (st) cudaStreamDestroy(st);
  }

  static int rows_x(int L, int v) { return XRL[list_of(v)] / L; }
  static int rows_y(int L, int v) { return YRL[list_of(v)] / L; }

  int build_lists() {
    for (int kind = 0; kind < EP_N; ++kind)
      for (int v = 0; v < 2; ++v) {
        // per member tile counts, then round-robin interleave across members
        std::vector<int> cnt(n);
        int tot = 0;
        for (int m = 0; m < n; ++m) {
          const StepConsts& c = fields[m].c;
          const bool xk = (kind == EP_X1 || kind == EP_X2 || kind == EP_XINV);
          const int R = xk ? rows_x(c.nx, v) : rows_y(c.ny, v);
          const int rows = xk ? c.ny : (kind == EP_Y1 ? c.K + 1 : 2 * c.K + 1);
          cnt[m] = (rows + R - 1) / R;
          tot += cnt[m];
        }
        std::vector<int2> items;
        items.reserve(tot);
        const int mx = *std::max_element(cnt.begin(), cnt.end());
        for (int t = 0; t < mx; ++t)
          for (int m = 0; m < n; ++m)
            if (t < cnt[m]) items.push_back(make_int2(m, t));
        if (cudaMalloc(&dItems[kind][v], sizeof(int2) * items.size()) != cudaSuccess ||
            cudaMemcpy(dItems[kind][v], items.data(), sizeof(int2) * items.size(), cudaMemcpyHostToDevice) !=
                cudaSuccess) {
          set_error("vk_ens_init: work list upload failed");
          return VK_E_NOMEM;
        }
        nItems[kind][v] = (int)items.size();
      }
    return VK_OK;
  }

  template <typename K> void launch(K kern, int g, int threads, size_t smem, int kind, int v) {
    ensure_smem_attr((const void*)kern, smem);
    kern<<<g, threads, smem, st>>>(dF, dItems[kind][list_of(v)], nItems[kind][list_of(v)]);
    ++launches;
  }

  void pass(int kind, int stage, bool from_t, int v, int g) {
    constexpr size_t E = sizeof(C);
    if (kind == EP_X1) {
      if (v == 2) {
        const size_t sm = E * 2048 * 17 / 16;
        if (from_t) launch(kb_x1<T, 2048, true, 3>, g, 128, sm, kind, v);
        else launch(kb_x1<T, 2048, false, 3>, g, 128, sm, kind, v);
      } else if (v == 0) {
        const size_t sm = E * 2048 * 17 / 16;
        if (from_t) launch(kb_x1<T, 2048, true>, g, 128, sm, kind, v);
        else launch(kb_x1<T, 2048, false>, g, 128, sm, kind, v);
      } else {
        const size_t sm = E * 4096 * 17 / 16;
        if (from_t) launch(kb_x1<T, 4096, true>, g, 256, sm, kind, v);
        else launch(kb_x1<T, 4096, false>, g, 256, sm, kind, v);
      }
    } else if (kind == EP_Y1) {
      if (v == 2) launch(kb_y1<T, 1024, 6>, g, 64, E * 1024 * 17 / 16, kind, v);
      else if (v == 0) launch(kb_y1<T, 1024>, g, 64, E * 1024 * 17 / 16, kind, v);
      else launch(kb_y1<T, 2048>, g, 128, E * 2048 * 17 / 16, kind, v);
    } else if (kind == EP_X2) {
      if (v == 2) launch(kb_x2<T, 2048, 3>, g, 128, E * 2048 * 17 / 16, kind, v);
      else if (v == 0) launch(kb_x2<T, 2048>, g, 128, E * 2048 * 17 / 16, kind, v);
      else launch(kb_x2<T, 4096>, g, 256, E * 4096 * 17 / 16, kind, v);
    } else if (kind == EP_Y2) {
      const size_t sm0 = E * 1024 * 17 / 16, sm1 = E * 2048 * 17 / 16;
      if (v == 2) {
        switch (stage) {
          case 1: launch(kb_y2<T, 1024, 1, 6>, g, 64, sm0, kind, v); break;
          case 2: launch(kb_y2<T, 1024, 2, 6>, g, 64, sm0, kind, v); break;
          case 3: launch(kb_y2<T, 1024, 3, 6>, g, 64, sm0, kind, v); break;
          default: launch(kb_y2<T, 1024, 4, 6>, g, 64, sm0, kind, v); break;
        }
        return;
      }
      switch (stage) {
        case 1: v == 0 ? launch(kb_y2<T, 1024, 1>, g, 64, sm0, kind, v) : launch(kb_y2<T, 2048, 1>, g, 128, sm1, kind, v); break;
        case 2: v == 0 ? launch(kb_y2<T, 1024, 2>, g, 64, sm0, kind, v) : launch(kb_y2<T, 2048, 2>, g, 128, sm1, kind, v); break;
        case 3: v == 0 ? launch(kb_y2<T, 1024, 3>, g, 64, sm0, kind, v) : launch(kb_y2<T, 2048, 3>, g, 128, sm1, kind, v); break;
        default: v == 0 ? launch(kb_y2<T, 1024, 4>, g, 64, sm0, kind, v) : launch(kb_y2<T, 2048, 4>, g, 128, sm1, kind, v); break;
      }
    } else {
      if (v != 1) launch(kb_xinv<T, 2048>, g, 128, E * 2048 * 17 / 16, kind, v);
      else launch(kb_xinv<T, 4096>, g, 256, E * 4096 * 17 / 16, kind, v);
    }
  }

  template <int STAGE, bool FROM_T> void launch_stage() {
    constexpr int RL = kFusedRL;
    // x lists of tile variant 0 and y lists of variant 1 hold RL-point tiles
    static_assert(XRL[0] == RL && YRL[1] == RL, "fused tiles");
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(fused_grid);
    cfg.blockDim = dim3(RL / 16);
    cfg.dynamicSmemBytes = sizeof(C) * RL * 17 / 16;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeCooperative;
    at[0].val.cooperative = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kb_stage<T, RL, STAGE, FROM_T>, (const Field<T>*)dF, (const int2*)dItems[EP_X1][0],
                       nItems[EP_X1][0], (const int2*)dItems[EP_Y1][1], nItems[EP_Y1][1],
                       (const int2*)dItems[EP_Y2][1], nItems[EP_Y2][1], bar, spin_limit);
    ++launches;
  }
  void step_fused(bool first) {
    if (first) launch_stage<1, false>();
    else launch_stage<1, true>();
    launch_stage<2, true>();
    launch_stage<3, true>();
    launch_stage<4, true>();
  }
  // Sets fused_grid (0 when a cooperative launch of kb_stage is not possible).
  int init_fused() {
    int dev = 0, coop = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
    const char* lim = std::getenv("VK_SPIN_LIMIT");
    if (lim) spin_limit = std::strtoull(lim, nullptr, 10);
    if (!coop) return VK_OK;
    const size_t smem = sizeof(C) * kFusedRL * 17 / 16;
    int occ = 1 << 30;
    auto fit = [&](const void* fn) {
      int b = 0;
      ensure_smem_attr(fn, smem);
      if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, fn, kFusedRL / 16, smem) != cudaSuccess) b = 0;
      occ = std::min(occ, b);
    };
    fit((const void*)kb_stage<T, kFusedRL, 1, false>);
    fit((const void*)kb_stage<T, kFusedRL, 1, true>);
    fit((const void*)kb_stage<T, kFusedRL, 2, true>);
    fit((const void*)kb_stage<T, kFusedRL, 3, true>);
    fit((const void*)kb_stage<T, kFusedRL, 4, true>);
    cudaGetLastError();
    if (occ <= 0) return VK_OK;
    fused_grid = occ * sms;
    if (cudaMalloc(&bar, sizeof(GridBarrier)) != cudaSuccess || cudaMemset(bar, 0, sizeof(GridBarrier)) != cudaSuccess) {
      set_error("vk_ens_init: barrier allocation failed");
      return VK_E_NOMEM;
    }
    return VK_OK;
  }
  // A barrier wait that ran out: report it once and reset the barrier.
  int barrier_check() {
    if (!bar) return VK_OK;
    GridBarrier h;
    if (cudaMemcpyAsync(&h, bar, sizeof(h), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess) {
      set_error("vk_ens: stream error");
      return VK_E_CUDA;
    }
    if (h.err == 0) return VK_OK;
    cudaMemsetAsync(bar, 0, sizeof(GridBarrier), st);
    cudaStreamSynchronize(st);
    set_error("vk_ens: a CTA of the persistent stage kernel gave up waiting at grid barrier " +
              std::to_string(h.err - 1) + " (the members' fields are not valid; set them again)");
    return VK_E_CUDA;
  }

  void step(bool first) {
    if (fused) {
      step_fused(first);
      return;
    }
    for (int stage = 1; stage <= 4; ++stage) {
      pass(EP_X1, stage, !(first && stage == 1), variant[EP_X1], grid[EP_X1]);
      pass(EP_Y1, stage, true, variant[EP_Y1], grid[EP_Y1]);
      pass(EP_X2, stage, true, variant[EP_X2], grid[EP_X2]);
      pass(EP_Y2, stage, true, variant[EP_Y2], grid[EP_Y2]);
    }
  }

  // Times each (variant, CTAs per SM) per pass kind on the current buffers.
  int autotune() {
    cudaEvent_t a, b;
    if (cudaEventCreate(&a) || cudaEventCreate(&b)) {
      set_error("vk_ens: event creation failed");
      return VK_E_CUDA;
    }
    const int per_sm[4] = {1, 2, 4, 8};
    const char* names[EP_N] = {"x1", "y1", "x2", "y2", "xinv"};
    report.clear();
    for (int kind = 0; kind < EP_N; ++kind) {
      float best = 1e30f;
      for (int v = 0; v < (kind == EP_XINV ? 2 : NVAR); ++v)
        for (int k = 0; k < 4; ++k) {
          const int g = sms * per_sm[k];
          pass(kind, 2, true, v, g);  // warm
          cudaEventRecord(a, st);
          for (int r = 0; r < 3; ++r) pass(kind, 2, true, v, g);
          cudaEventRecord(b, st);
          cudaEventSynchronize(b);
          float ms = 0.f;
          cudaEventElapsedTime(&ms, a, b);
          if (ms < best) {
            best = ms;
            variant[kind] = v;
            grid[kind] = g;
          }
        }
      char buf[160];
      snprintf(buf, sizeof(buf), "%s: tile %d points%s, %d CTAs (%.1f us/launch); ", names[kind],
               (kind == EP_Y1 || kind == EP_Y2) ? YRL[list_of(variant[kind])] : XRL[list_of(variant[kind])],
               variant[kind] == 2 ? " (registers capped)" : "", grid[kind], 1e3f * best / 3.f);
      report += buf;
    }
    // one RK4 step: the chosen pass kernels against the persistent stage kernel
    int rc = init_fused();
    if (rc) {
      cudaEventDestroy(a);
      cudaEventDestroy(b);
      return rc;
    }
    if (fused_grid > 0) {
      float tsep = 0.f, tfus = 0.f;
      for (int f = 0; f < 2; ++f) {
        fused = f == 1;
        step(false);  // warm
        cudaEventRecord(a, st);
        for (int r = 0; r < 2; ++r) step(false);
        cudaEventRecord(b, st);
        cudaEventSynchronize(b);
        cudaEventElapsedTime(f ? &tfus : &tsep, a, b);
      }
      const char* env = std::getenv("VK_FUSED");
      fused = env ? env[0] != '0' : tfus < tsep;
      rc = barrier_check();
      if (rc) {
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        return rc;
      }
      char buf[200];
      snprintf(buf, sizeof(buf), "step: pass kernels %.1f us, persistent stage kernel (%d CTAs) %.1f us -> %s",
               1e3f * tsep / 2.f, fused_grid, 1e3f * tfus / 2.f, fused ? "persistent" : "pass kernels");
      report += buf;
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
      set_error(std::string("vk_ens autotune: ") + cudaGetErrorString(e));
      return VK_E_CUDA;
    }
    return VK_OK;
  }

  int rk4(int nsteps) {
    if (nsteps <= 0) return VK_OK;
    for (int m = 0; m < n; ++m)
      if (!owned[m]->kpsi_is_masked()) {
        const StepConsts& c = fields[m].c;
        k_mask_four<T><<<512, 256, 0, st>>>(fields[m].kpsi, c.nx, c.ny, c.k2max);
        ++launches;
      }
    for (int s = 0; s < nsteps; ++s) {
      if (s == 0) {
        step(true);
        continue;
      }
      if (!gstep) {
        const int64_t l0 = launches;
        cudaGraph_t g = nullptr;
        if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
          step(false);
          if (cudaStreamEndCapture(st, &g) != cudaSuccess || cudaGraphInstantiate(&gstep, g, 0) != cudaSuccess)
            gstep = nullptr;
          if (g) cudaGraphDestroy(g);
        }
        gstep_n = launches - l0;
        launches = l0;
        cudaGetLastError();
      }
      if (gstep) {
        if (cudaGraphLaunch(gstep, st) != cudaSuccess) {
          set_error("vk_ens_gpe_rk4: graph launch failed");
          return VK_E_CUDA;
        }
        launches += gstep_n;
      } else {
        step(false);
      }
    }
    pass(EP_XINV, 0, true, variant[EP_XINV], grid[EP_XINV]);
    for (int m = 0; m < n; ++m) owned[m]->mark_rk4_done();
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
      set_error(std::string("vk_ens_gpe_rk4: ") + cudaGetErrorString(e));
      return VK_E_CUDA;
    }
    return VK_OK;
  }
};

}  // namespace vk
