// Host build of the row-FFT arithmetic of quantumvortices_gb300/csrc/vk_fft.cuh:
// the radix codelets, the twiddled first butterfly layer and whole Stockham
// transforms (one emulated thread, so every stage reads all its inputs before
// it writes) against a direct long-double DFT.  Prints one line per case:
//   <case> <max |error|> <max |X|>
// Built by tests/test_fft_codelets.py with g++ and the CUDA headers.
#include <cuda_runtime.h>
#include <cmath>
#include <complex>
#include <cstdio>
#include <vector>

// CUDA built-ins the header names: one thread, no barriers needed.
static struct { int x; } threadIdx = {0};
static inline void __syncthreads() {}
static inline void __syncwarp() {}
#define __ldg(p) (*(p))
#include "vk_fft.cuh"

using namespace vk;
typedef std::complex<long double> CL;

template <typename T> static cplx<T> input(int m, int seed) {
  cplx<T> v;
  v.x = T(std::sin(1.37 * m + 0.29 * seed) + 0.25 * std::cos(0.011 * m * m));
  v.y = T(std::cos(0.73 * m - 0.41 * seed));
  return v;
}

template <typename T> static void report(const char* name, const cplx<T>* got, const std::vector<CL>& ref) {
  long double err = 0, mx = 0;
  for (size_t k = 0; k < ref.size(); ++k) {
    err = std::fmax(err, std::abs(CL(got[k].x, got[k].y) - ref[k]));
    mx = std::fmax(mx, std::abs(ref[k]));
  }
  std::printf("%s %.6Le %.6Le\n", name, err, mx);
}

// X(k) = sum_m x(m) exp(DIR 2 pi i m k / n), x(m) = pre(m) * input(m)
template <typename T, class Pre> static std::vector<CL> direct(int n, int dir, int seed, Pre pre) {
  std::vector<CL> out(n);
  const long double tp = 6.283185307179586476925286766559L;
  for (int k = 0; k < n; ++k) {
    CL s = 0;
    for (int m = 0; m < n; ++m) {
      const cplx<T> v = input<T>(m, seed);
      s += pre(m) * CL(v.x, v.y) * std::polar(1.0L, dir * tp * (long double)((long long)m * k % n) / n);
    }
    out[k] = s;
  }
  return out;
}

template <int RAD, int DIR> static void codelet() {
  cplx<double> v[RAD];
  for (int m = 0; m < RAD; ++m) v[m] = input<double>(m, RAD + DIR);
  dft<RAD, DIR>(v);
  char name[64];
  std::snprintf(name, sizeof name, "dft%d_dir%+d", RAD, DIR);
  report<double>(name, v, direct<double>(RAD, DIR, RAD + DIR, [](int) { return CL(1); }));
}

// First layer with table twiddles w(m) (w(0) = 1), then the tail.
template <int RAD, int DIR> static void twiddled() {
  cplx<double> v[RAD], w[RAD];
  auto wl = [](int m) { return std::polar(1.0L, DIR * 0.173L * m); };
  for (int m = 0; m < RAD; ++m) {
    v[m] = input<double>(m, 7 * RAD);
    w[m].x = (double)wl(m).real();
    w[m].y = (double)wl(m).imag();
  }
  for (int m = 0; m < RAD / 2; ++m) {
    if (m > 0) v[m] = cmul(v[m], w[m]);
    bfly_tw(v[m], v[m + RAD / 2], w[m + RAD / 2]);
  }
  dft_tail<RAD, DIR>(v);
  char name[64];
  std::snprintf(name, sizeof name, "tw%d_dir%+d", RAD, DIR);
  report<double>(name, v, direct<double>(RAD, DIR, 7 * RAD, [&](int m) { return m ? wl(m) : CL(1); }));
}

// Whole transform of L points through the Stockham stages of plan P on the
// table of a TWS*L-point transform.
template <typename T, int L, int DIR, int TWS, class P> static void transform(const char* tag) {
  std::vector<cplx<T>> tw(TWS * L), s(padded(L));
  const long double tp = 6.283185307179586476925286766559L;
  for (int k = 0; k < TWS * L; ++k) {
    tw[k].x = (T)std::cos(-tp * k / (TWS * L));
    tw[k].y = (T)std::sin(-tp * k / (TWS * L));
  }
  for (int m = 0; m < L; ++m) s[pidx(m)] = input<T>(m, L);
  run_stages<T, L, 1, 1, DIR, 1, 1, TWS>(s.data(), tw.data(), P());
  std::vector<cplx<T>> out(L);
  for (int k = 0; k < L; ++k) out[k] = s[pidx(k)];
  char name[96];
  std::snprintf(name, sizeof name, "%s_%s_L%d_dir%+d_tws%d", sizeof(T) == 8 ? "f64" : "f32", tag, L, DIR, TWS);
  report<T>(name, out.data(), direct<T>(L, DIR, L, [](int) { return CL(1); }));
}

int main() {
  codelet<2, -1>(); codelet<2, 1>(); codelet<4, -1>(); codelet<4, 1>();
  codelet<8, -1>(); codelet<8, 1>(); codelet<16, -1>(); codelet<16, 1>();
  twiddled<2, -1>(); twiddled<2, 1>(); twiddled<4, -1>(); twiddled<4, 1>();
  twiddled<8, -1>(); twiddled<8, 1>(); twiddled<16, -1>(); twiddled<16, 1>();
  transform<double, 1024, -1, 1, PlanFor<1024, 16>::type>("r16");
  transform<double, 1024, +1, 1, PlanFor<1024, 16>::type>("r16");
  transform<double, 1024, -1, 1, PlanFor<1024, 8>::type>("r8");
  transform<double, 1024, +1, 1, PlanFor<1024, 4>::type>("r4");
  transform<double, 512, -1, 2, PlanFor<512, 8>::type>("r8");
  transform<double, 512, +1, 2, PlanFor<512, 4>::type>("r4");
  transform<double, 2048, -1, 1, PlanFor<2048, 16>::type>("r16");
  transform<double, 256, +1, 1, PlanFor<256, 16>::type>("r16");
  transform<double, 32, -1, 1, PlanFor<32, 16>::type>("r16");
  transform<float, 1024, -1, 1, PlanFor<1024, 16>::type>("r16");
  transform<float, 512, +1, 2, PlanFor<512, 8>::type>("r8");
  return 0;
}
