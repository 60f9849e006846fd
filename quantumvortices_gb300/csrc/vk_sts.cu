// vk_sts.cu -- spatio-temporal spectra on the GPU (the -DGPSTS path).
//
// The reference appends kpsi(:, kx=0) and the kpsi plane to files every
// ststeps (sts_gpe, src/diagnostics.f90:636-695) and computes the spectra
// offline (Run/CompSTS/driver.f90:132-265): every mode's time series is
// multiplied by the Hann window w(t) = (1 - cos(2 pi t/(Nt-1)))/2
// (:194-196, :236-238), transformed along time with FFTW_FORWARD (:132, :240),
// and |X|^2 stsnorm is kept per (kx=0, ky) line (:198-200) and summed over the
// shells nint(|k|) (:243-255), stsnorm = (1/Nt)^2 (1/(Nx Ny))^2 (:123).
//
// Here the records stay in HBM: a ring of nt FP64 kpsi planes, [t][kx][ky].
//   k_sts_time   one CTA per R modes: the R time series are staged in shared
//                memory (windowed), transformed by the row-FFT engine
//                (length nt), and |X|^2 stsnorm is written back in place
//                (into .x of the same slots).
//   k_sts_bin    one CTA per frequency: the kx = 0 line is copied out and each
//                shell is summed by one thread over a host-built list of its
//                modes in (kx, ky) order -- the reference's loop order, so the
//                shell sums are deterministic.
#include <cmath>
#include <cstring>
#include <string>
#include <vector>
#include "vk_kernels.cuh"
#include "vk_solver.h"

namespace vk {

template <int L>
__global__ void __launch_bounds__(GeoX<double, L>::NT, GeoX<double, L>::MINB)
    k_sts_time(double2* __restrict__ ring, size_t nmodes, const double* __restrict__ hann,
               const double2* __restrict__ tw, double stsnorm) {
  typedef GeoX<double, L> G;
  extern __shared__ __align__(16) unsigned char smraw[];
  double2* s = reinterpret_cast<double2*>(smraw);
  const size_t m0 = (size_t)blockIdx.x * G::R;
  // element e -> (mode r, time t) with r fastest: R consecutive modes of one
  // record are contiguous in the ring
  for (int e = threadIdx.x; e < G::R * L; e += G::NT) {
    const int r = e % G::R, t = e / G::R;
    const double2 v = ring[(size_t)t * nmodes + m0 + r];
    const double w = hann[t];
    s[r * G::LP + pidx(t)] = make_double2(w * v.x, w * v.y);
  }
  __syncthreads();
  fft_rows<double, L, G::R, G::NT, -1>(s, tw);
  for (int e = threadIdx.x; e < G::R * L; e += G::NT) {
    const int r = e % G::R, t = e / G::R;
    const double2 v = s[r * G::LP + pidx(t)];
    const double a = hypot(v.x, v.y);  // Fortran ABS of a complex
    ring[(size_t)t * nmodes + m0 + r].x = stsnorm * (a * a);
  }
}

// One CTA per frequency w: sts1d[w][ky] = P[w][kx=0][ky]; sts2d[w][m] = sum of
// P[w][mode] over the modes listed for shell m (in increasing mode index).
__global__ void k_sts_bin(const double2* __restrict__ ring, size_t nmodes, int ny, const int* __restrict__ shell_ptr,
                          const int* __restrict__ shell_modes, int nsh, double* __restrict__ sts1d,
                          double* __restrict__ sts2d) {
  const size_t w = blockIdx.x;
  const double2* P = ring + w * nmodes;
  for (int ky = threadIdx.x; ky < ny; ky += blockDim.x) sts1d[w * ny + ky] = P[ky].x;
  for (int m = threadIdx.x; m < nsh; m += blockDim.x) {
    double acc = 0.0;
    for (int j = shell_ptr[m]; j < shell_ptr[m + 1]; ++j) acc += P[shell_modes[j]].x;
    sts2d[w * nsh + m] = acc;
  }
}

namespace {

class Sts final : public StsBase {
 public:
  ~Sts() override {
    if (ring_) cudaFree(ring_);
    if (hann_) cudaFree(hann_);
    if (tw_) cudaFree(tw_);
    if (ptr_) cudaFree(ptr_);
    if (modes_) cudaFree(modes_);
    if (o1_) cudaFree(o1_);
    if (o2_) cudaFree(o2_);
  }

  int init(int nx, int ny, int nt, cudaStream_t st) {
    nx_ = nx;
    ny_ = ny;
    nt_ = nt;
    st_ = st;
    nmodes_ = (size_t)nx * ny;
    nsh_ = nx / 3 + 1;  // written shells 0..INT(Nx/3) (Run/CompSTS/driver.f90:262)
    if (cudaMalloc(&ring_, sizeof(double2) * nmodes_ * nt) != cudaSuccess) {
      ring_ = nullptr;
      cudaGetLastError();
      set_error("vk_sts_begin: cannot allocate " + std::to_string(sizeof(double2) * nmodes_ * nt) + " bytes");
      return VK_E_NOMEM;
    }
    // Hann window, time-FFT twiddles, shell lists (host, FP64)
    std::vector<double> hann(nt), tw(2 * (size_t)nt);
    const double pi = 4.0 * std::atan(1.0);
    for (int t = 0; t < nt; ++t) hann[t] = 0.5 * (1.0 - std::cos(2.0 * pi * t / (nt - 1)));
    twiddle_table(nt, tw.data());
    std::vector<int> cnt(nsh_ + 1, 0), shell(nmodes_, -1);
    for (int kx = 0; kx < nx; ++kx)
      for (int ky = 0; ky < ny; ++ky) {
        const int k1 = kx - nx * ((kx + 1) / (nx / 2 + 1));  // (i1-1) - Nx*(i1/Nxhp), i1 = kx+1
        const int k2 = ky - ny * ((ky + 1) / (ny / 2 + 1));
        const long ksq = (long)k1 * k1 + (long)k2 * k2;
        const long m = std::lround(std::sqrt((double)ksq));  // NINT; sqrt of an integer is never x.5
        if (m < nsh_) {
          shell[(size_t)kx * ny + ky] = (int)m;
          ++cnt[m + 1];
        }
      }
    for (int m = 0; m < nsh_; ++m) cnt[m + 1] += cnt[m];
    std::vector<int> modes(cnt[nsh_]), fill(cnt.begin(), cnt.end() - 1);
    for (size_t i = 0; i < nmodes_; ++i)
      if (shell[i] >= 0) modes[fill[shell[i]]++] = (int)i;
    const bool ok = cudaMalloc(&hann_, sizeof(double) * nt) == cudaSuccess &&
                    cudaMalloc(&tw_, sizeof(double2) * nt) == cudaSuccess &&
                    cudaMalloc(&ptr_, sizeof(int) * (nsh_ + 1)) == cudaSuccess &&
                    cudaMalloc(&modes_, sizeof(int) * std::max<size_t>(modes.size(), 1)) == cudaSuccess &&
                    cudaMalloc(&o1_, sizeof(double) * (size_t)nt * ny) == cudaSuccess &&
                    cudaMalloc(&o2_, sizeof(double) * (size_t)nt * nsh_) == cudaSuccess;
    if (!ok) {
      cudaGetLastError();
      set_error("vk_sts_begin: out of device memory");
      return VK_E_NOMEM;
    }
    cudaMemcpy(hann_, hann.data(), sizeof(double) * nt, cudaMemcpyHostToDevice);
    cudaMemcpy(tw_, tw.data(), sizeof(double2) * nt, cudaMemcpyHostToDevice);
    cudaMemcpy(ptr_, cnt.data(), sizeof(int) * (nsh_ + 1), cudaMemcpyHostToDevice);
    if (!modes.empty()) cudaMemcpy(modes_, modes.data(), sizeof(int) * modes.size(), cudaMemcpyHostToDevice);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
      set_error(std::string("vk_sts_begin: ") + cudaGetErrorString(e));
      return VK_E_CUDA;
    }
    return VK_OK;
  }

  int record(SolverBase* s) override {
    if (count_ >= nt_) {
      set_error("vk_sts_record: the ring is full (" + std::to_string(nt_) + " records)");
      return VK_E_STATE;
    }
    const int rc = s->snapshot_kpsi_f64(ring_ + (size_t)count_ * nmodes_);
    if (rc == VK_OK) ++count_;
    return rc;
  }
  int count() const override { return count_; }

  int spectra(double* sts1d, double* sts2d) override {
    if (count_ != nt_) {
      set_error("vk_sts_spectra: " + std::to_string(count_) + " of " + std::to_string(nt_) + " records");
      return VK_E_STATE;
    }
    const double a = 1.0 / (double)nt_, b = 1.0 / (double)nmodes_;
    const double stsnorm = (a * a) * (b * b);  // (one/Ntt)**2*(one/(Nx*Ny))**2
    int rc = VK_OK;
    switch (nt_) {
      case 16: rc = time_pass<16>(stsnorm); break;
      case 32: rc = time_pass<32>(stsnorm); break;
      case 64: rc = time_pass<64>(stsnorm); break;
      case 128: rc = time_pass<128>(stsnorm); break;
      case 256: rc = time_pass<256>(stsnorm); break;
      case 512: rc = time_pass<512>(stsnorm); break;
      case 1024: rc = time_pass<1024>(stsnorm); break;
      case 2048: rc = time_pass<2048>(stsnorm); break;
      case 4096: rc = time_pass<4096>(stsnorm); break;
      default: set_error("vk_sts_spectra: bad record count"); return VK_E_INVALID;
    }
    if (rc != VK_OK) return rc;
    k_sts_bin<<<nt_, 256, 0, st_>>>(ring_, nmodes_, ny_, ptr_, modes_, nsh_, o1_, o2_);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(sts1d, o1_, sizeof(double) * (size_t)nt_ * ny_, cudaMemcpyDeviceToHost, st_);
    if (e == cudaSuccess) e = cudaMemcpyAsync(sts2d, o2_, sizeof(double) * (size_t)nt_ * nsh_, cudaMemcpyDeviceToHost, st_);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st_);
    count_ = 0;  // the ring now holds |X|^2, not records
    if (e != cudaSuccess) {
      set_error(std::string("vk_sts_spectra: ") + cudaGetErrorString(e));
      return VK_E_CUDA;
    }
    return VK_OK;
  }

 private:
  template <int L> int time_pass(double stsnorm) {
    typedef GeoX<double, L> G;
    const size_t smem = sizeof(double2) * G::R * G::LP;
    ensure_smem_attr((const void*)k_sts_time<L>, smem);
    const size_t grid = nmodes_ / G::R;  // nmodes is a power of two >= 256, R <= 16
    k_sts_time<L><<<(unsigned)grid, G::NT, smem, st_>>>(ring_, nmodes_, hann_, tw_, stsnorm);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
      set_error(std::string("k_sts_time: ") + cudaGetErrorString(e));
      return VK_E_CUDA;
    }
    return VK_OK;
  }

  int nx_ = 0, ny_ = 0, nt_ = 0, nsh_ = 0, count_ = 0;
  size_t nmodes_ = 0;
  cudaStream_t st_ = nullptr;
  double2* ring_ = nullptr;
  double* hann_ = nullptr;
  double2* tw_ = nullptr;
  int *ptr_ = nullptr, *modes_ = nullptr;
  double *o1_ = nullptr, *o2_ = nullptr;
};

}  // namespace

StsBase* make_sts(int nx, int ny, int nt, void* stream, int* status) {
  Sts* s = new Sts();
  *status = s->init(nx, ny, nt, (cudaStream_t)stream);
  if (*status != VK_OK) {
    delete s;
    return nullptr;
  }
  return s;
}

}  // namespace vk
