// Host build of the FP64 pass bodies of quantumvortices_gb300/csrc/vk_kernels.cuh
// (x1 / x2 on row pairs and on single rows, y1, the RK4 y2 stage) with a
// one-thread geometry: every loop over the block's threads covers all
// elements and every stage reads all its inputs before it writes, so the
// bodies compute exactly what a CTA computes.  Fields are raw complex128
// files in a work directory; tests/test_kernel_bodies.py writes the inputs,
// runs a pass over all row tiles and checks the outputs against numpy.
//
//   kernel_bodies_host x1 L ny single|pair DIR      Ta -> psi, Tb
//   kernel_bodies_host x2 L ny single|pair +1|-1 DIR  Tc, psi -> Td
//   kernel_bodies_host y1 L DIR                      Tb -> Tc        (L x L grid)
//   kernel_bodies_host y2 L STAGE DIR                Td, kpsi, str1, str2 -> kpsi, str1, str2, Ta
//   kernel_bodies_host y2a L DIR                     Td, kpsi -> kpsi, Ta, part (ARGLE, residual sums)
//   kernel_bodies_host x2p L ny DIR                  Tc, psi, vpot -> Td (RK4 with a potential)
#include <cuda_runtime.h>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

static struct { int x; } threadIdx = {0}, blockIdx = {0}, blockDim = {1}, gridDim = {1};
static inline void __syncthreads() {}
static inline void __syncwarp() {}
#define __ldg(p) (*(p))
#define __launch_bounds__(...)
#include "vk_kernels.cuh"

using namespace vk;
typedef double2 C;

template <int LL, int RR> struct G1 {
  static constexpr int L = LL, R = RR, LP = padded(LL), MINB = 1, NT = 1;
};

static std::string dir;
static std::vector<C> load(const char* name, size_t n) {
  std::vector<C> v(n);
  FILE* f = std::fopen((dir + "/" + name).c_str(), "rb");
  if (!f || std::fread(v.data(), sizeof(C), n, f) != n) { std::fprintf(stderr, "read %s\n", name); std::exit(2); }
  std::fclose(f);
  return v;
}
static void save(const char* name, const std::vector<C>& v) {
  FILE* f = std::fopen((dir + "/" + name).c_str(), "wb");
  if (!f || std::fwrite(v.data(), sizeof(C), v.size(), f) != v.size()) { std::fprintf(stderr, "write %s\n", name); std::exit(2); }
  std::fclose(f);
}

static std::vector<double> load_real(const char* name, size_t n) {
  std::vector<double> v(n);
  FILE* f = std::fopen((dir + "/" + name).c_str(), "rb");
  if (!f || std::fread(v.data(), sizeof(double), n, f) != n) { std::fprintf(stderr, "read %s\n", name); std::exit(2); }
  std::fclose(f);
  return v;
}
static void save_real(const char* name, const std::vector<double>& v) {
  FILE* f = std::fopen((dir + "/" + name).c_str(), "wb");
  if (!f || std::fwrite(v.data(), sizeof(double), v.size(), f) != v.size()) { std::fprintf(stderr, "write %s\n", name); std::exit(2); }
  std::fclose(f);
}

static int k2max_of(int n) {
  const double ka2 = (n / 3.0) * (n / 3.0);
  long k = (long)std::floor(ka2) + 1;
  while (k > 0 && (double)k >= ka2) --k;
  return (int)k;
}
static int kmax_of(int k2max) {
  int k = (int)std::sqrt((double)k2max);
  while ((long)(k + 1) * (k + 1) <= k2max) ++k;
  while ((long)k * k > k2max) --k;
  return k;
}

static StepConsts consts(int nx, int ny) {
  StepConsts c{};
  c.nx = nx; c.ny = ny;
  c.k2max = k2max_of(nx);  // the 2/3 rule on kalias = nx/3 (src/mod_grid.f90:63-101)
  c.K = kmax_of(c.k2max);
  c.pk = (c.K + 2) & ~1;
  c.alpha = 0.0123; c.g = 15.5; c.omega = 15.5; c.dt = 1e-3;
  c.prefac_re = -0.1; c.prefac_im = -1.0;
  c.scale = 1.0 / ((double)nx * (double)ny);
  return c;
}

static std::vector<C> twiddles(int n) {
  std::vector<C> t(n);
  const long double tp = 6.283185307179586476925286766559L;
  for (int k = 0; k < n; ++k) { t[k].x = (double)std::cos(-tp * k / n); t[k].y = (double)std::sin(-tp * k / n); }
  return t;
}

template <int L> static int run(int argc, char** argv) {
  const std::string pass = argv[1];
  const std::vector<C> tw = twiddles(L);
  std::vector<C> s(2 * padded(L) + 64);
  if (pass == "x1") {
    const int ny = std::atoi(argv[3]);
    const bool single = std::string(argv[4]) == "single";
    const StepConsts c = consts(L, ny);
    std::vector<C> Ta = load("Ta.bin", (size_t)ny * L), psi((size_t)ny * L), Tb((size_t)(c.K + 1) * ny);
    if (single)
      for (int y = 0; y < ny; ++y) x1_single_body<double, L, G1<L, 2>, true, true>(Ta.data(), psi.data(), Tb.data(), tw.data(), c, y, s.data());
    else
      for (int t = 0; t < ny / 2; ++t) x1_body<double, L, G1<L, 2>, true, true>(Ta.data(), psi.data(), Tb.data(), tw.data(), c, t, s.data());
    save("psi.bin", psi);
    save("Tb.bin", Tb);
  } else if (pass == "x2") {
    const int ny = std::atoi(argv[3]);
    const bool single = std::string(argv[4]) == "single";
    const int sign = std::atoi(argv[5]);
    const StepConsts c = consts(L, ny);
    std::vector<C> Tc = load("Tc.bin", (size_t)ny * c.pk), psi = load("psi.bin", (size_t)ny * L), Td((size_t)L * ny);
    for (int t = 0; t < (single ? ny : ny / 2); ++t) {
      if (sign > 0) {
        if (single) x2_single_body<double, L, G1<L, 2>, +1, true, false, true>(Tc.data(), psi.data(), nullptr, Td.data(), tw.data(), c, t, s.data());
        else x2_body<double, L, G1<L, 2>, +1, true, false>(Tc.data(), psi.data(), nullptr, Td.data(), tw.data(), c, t, s.data());
      } else {
        if (single) x2_single_body<double, L, G1<L, 2>, -1, false, false, true>(Tc.data(), psi.data(), nullptr, Td.data(), tw.data(), c, t, s.data());
        else x2_body<double, L, G1<L, 2>, -1, false, false>(Tc.data(), psi.data(), nullptr, Td.data(), tw.data(), c, t, s.data());
      }
    }
    save("Td.bin", Td);
  } else if (pass == "y1") {
    const StepConsts c = consts(L, L);
    std::vector<C> Tb = load("Tb.bin", (size_t)(c.K + 1) * L), Tc((size_t)L * c.pk);
    for (int t = 0; t <= c.K; ++t) y1_body<double, L, G1<L, 1>>(Tb.data(), Tc.data(), tw.data(), c, t, s.data());
    save("Tc.bin", Tc);
  } else if (pass == "y2") {
    const int stage = std::atoi(argv[3]);
    const StepConsts c = consts(L, L);
    const size_t n2 = (size_t)L * L;
    std::vector<C> Td = load("Td.bin", n2), kpsi = load("kpsi.bin", n2), s1 = load("str1.bin", n2), s2 = load("str2.bin", n2), Ta(n2);
    for (int t = 0; t < 2 * c.K + 1; ++t) {
      switch (stage) {
        case 1: y2_rk4_body<double, L, G1<L, 1>, 1>(Td.data(), kpsi.data(), s1.data(), s2.data(), Ta.data(), tw.data(), c, t, s.data()); break;
        case 2: y2_rk4_body<double, L, G1<L, 1>, 2>(Td.data(), kpsi.data(), s1.data(), s2.data(), Ta.data(), tw.data(), c, t, s.data()); break;
        case 3: y2_rk4_body<double, L, G1<L, 1>, 3>(Td.data(), kpsi.data(), s1.data(), s2.data(), Ta.data(), tw.data(), c, t, s.data()); break;
        default: y2_rk4_body<double, L, G1<L, 1>, 4>(Td.data(), kpsi.data(), s1.data(), s2.data(), Ta.data(), tw.data(), c, t, s.data()); break;
      }
    }
    save("kpsi.bin", kpsi);
    save("str1.bin", s1);
    save("str2.bin", s2);
    save("Ta.bin", Ta);
  } else if (pass == "y2a") {
    const StepConsts c = consts(L, L);
    const size_t n2 = (size_t)L * L;
    std::vector<C> Td = load("Td.bin", n2), kpsi = load("kpsi.bin", n2), Ta(n2);
    std::vector<double> part(3 * (size_t)L);
    for (int t = 0; t < L; ++t)
      y2_argle_body<double, L, G1<L, 1>, true>(Td.data(), kpsi.data(), Ta.data(), tw.data(), part.data(), c, t, s.data());
    save("kpsi.bin", kpsi);
    save("Ta.bin", Ta);
    save_real("part.bin", part);
  } else if (pass == "x2p") {
    const int ny = std::atoi(argv[3]);
    const StepConsts c = consts(L, ny);
    std::vector<C> Tc = load("Tc.bin", (size_t)ny * c.pk), psi = load("psi.bin", (size_t)ny * L), Td((size_t)L * ny);
    const std::vector<double> vpot = load_real("vpot.bin", (size_t)ny * L);
    for (int t = 0; t < ny / 2; ++t)
      x2_body<double, L, G1<L, 2>, +1, true, true>(Tc.data(), psi.data(), vpot.data(), Td.data(), tw.data(), c, t, s.data());
    save("Td.bin", Td);
  } else {
    return 2;
  }
  return 0;
}

int main(int argc, char** argv) {
  if (argc < 4) return 2;
  dir = argv[argc - 1];
  const int L = std::atoi(argv[2]);
  switch (L) {
    case 128: return run<128>(argc, argv);
    case 256: return run<256>(argc, argv);
    case 1024: return run<1024>(argc, argv);
    default: return 3;
  }
}
