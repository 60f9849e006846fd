// vk_noalloc.cu -- forward 2D FFT that allocates no device memory.
//
// For callers that cannot call cudaMalloc: for example a Fortran code whose
// device arrays are owned by an OpenACC / OpenMP-offload runtime (handed over
// with `host_data use_device`), or an application whose device memory belongs
// to its own pool allocator and must not be grown behind its back.  They pass
// device pointers for psi and kpsi; the transposed intermediate of the two
// row passes lives in the file-scope array below instead of a cudaMalloc'd
// buffer, and the twiddle tables live in a second file-scope array.
//
// Limits and sharing: the intermediate holds at most VK_NOALLOC_MAX_POINTS
// complex doubles (4 MiB; every GPU that loads the library keeps it until the
// process exits) and rows up to 4096 points.  All calls share the one array;
// each call overwrites every element it reads, so nothing needs clearing, but
// calls that overlap on the GPU (different streams, no ordering) race on it.
#include <cuda_runtime.h>
#include <mutex>
#include <string>
#include <vector>
#include "vk_kernels.cuh"
#include "vk_solver.h"

#define VK_NOALLOC_MAX_POINTS (512 * 512)
#define VK_NOALLOC_MAX_LEN 4096
// Twiddle tables for L = 16, 32, ..., 4096 back to back: table L starts at L-16.
#define VK_NOALLOC_TW_TOTAL (2 * VK_NOALLOC_MAX_LEN - 16)

namespace vk {
namespace {

static __device__ __align__(256) double2 g_noalloc_scratch[VK_NOALLOC_MAX_POINTS];
static __device__ __align__(256) double2 g_noalloc_tw[VK_NOALLOC_TW_TOTAL];

struct DeviceSlots {
  bool ready = false;
  double2* scratch = nullptr;  // device address of g_noalloc_scratch
  double2* tw = nullptr;       // device address of g_noalloc_tw
};

// One slot per device ordinal, in a fixed array: a slot never moves, and the
// caller gets a copy of its pointers taken under the lock.
constexpr int kMaxDevices = 64;
std::mutex g_mu;
DeviceSlots g_slots[kMaxDevices];

// Once per device, with that device current: resolve the arrays' device
// addresses (the names are host stand-ins in host code) and fill the tables.
int setup_current_device(DeviceSlots* out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    set_error(std::string("vk_fft2d_forward_noalloc: cudaGetDevice: ") + cudaGetErrorString(e));
    return VK_E_CUDA;
  }
  if (dev < 0 || dev >= kMaxDevices) {
    set_error("vk_fft2d_forward_noalloc: device ordinal beyond the 64 slots of the built-in tables");
    return VK_E_INVALID;
  }
  std::lock_guard<std::mutex> g(g_mu);
  DeviceSlots& s = g_slots[dev];
  if (!s.ready) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) {
      set_error(std::string("vk_fft2d_forward_noalloc: cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
      return VK_E_CUDA;
    }
    double2* scratch = static_cast<double2*>(p);
    e = cudaGetSymbolAddress(&p, g_noalloc_tw);
    if (e != cudaSuccess) {
      set_error(std::string("vk_fft2d_forward_noalloc: cudaGetSymbolAddress(twiddles): ") + cudaGetErrorString(e));
      return VK_E_CUDA;
    }
    double2* tw = static_cast<double2*>(p);
    std::vector<double> host(2 * (size_t)VK_NOALLOC_TW_TOTAL);
    for (int L = 16; L <= VK_NOALLOC_MAX_LEN; L *= 2) twiddle_table(L, host.data() + 2 * (size_t)(L - 16));
    e = cudaMemcpyToSymbol(g_noalloc_tw, host.data(), sizeof(double2) * VK_NOALLOC_TW_TOTAL);
    if (e != cudaSuccess) {
      set_error(std::string("vk_fft2d_forward_noalloc: cudaMemcpyToSymbol(twiddles): ") + cudaGetErrorString(e));
      return VK_E_CUDA;
    }
    s.scratch = scratch;
    s.tw = tw;
    s.ready = true;
  }
  *out = s;
  return VK_OK;
}

// Launches kern through cudaLaunchKernel, whose return code belongs to this
// launch alone (an error left behind by earlier work of the caller is neither
// reported nor cleared here).
template <typename... A>
int launch_checked(const char* what, void (*kern)(A...), int grid, int block, size_t smem, cudaStream_t st,
                   A... args) {
  if (smem > 48 * 1024) {
    const cudaError_t e =
        cudaFuncSetAttribute((const void*)kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) {
      set_error(std::string("vk_fft2d_forward_noalloc: shared-memory attribute of ") + what + ": " +
                cudaGetErrorString(e));
      return VK_E_CUDA;
    }
  }
  void* argv[] = {(void*)&args...};
  const cudaError_t e = cudaLaunchKernel((const void*)kern, dim3(grid), dim3(block), argv, smem, st);
  if (e != cudaSuccess) {
    set_error(std::string("vk_fft2d_forward_noalloc: launch of ") + what + ": " + cudaGetErrorString(e));
    return VK_E_CUDA;
  }
  return VK_OK;
}

template <typename F> bool with_len_na(int n, F&& f) {
  switch (n) {
    case 16: f(std::integral_constant<int, 16>()); return true;
    case 32: f(std::integral_constant<int, 32>()); return true;
    case 64: f(std::integral_constant<int, 64>()); return true;
    case 128: f(std::integral_constant<int, 128>()); return true;
    case 256: f(std::integral_constant<int, 256>()); return true;
    case 512: f(std::integral_constant<int, 512>()); return true;
    case 1024: f(std::integral_constant<int, 1024>()); return true;
    case 2048: f(std::integral_constant<int, 2048>()); return true;
    case 4096: f(std::integral_constant<int, 4096>()); return true;
    default: return false;
  }
}

bool pow2_len(int n) { return n >= 16 && n <= VK_NOALLOC_MAX_LEN && (n & (n - 1)) == 0; }

}  // namespace
}  // namespace vk

// No counterpart in the reference (see include/vk.h).
extern "C" int vk_fft2d_forward_noalloc(const double* psi_dev, double* kpsi_dev, int32_t nx, int32_t ny,
                                        void* stream) {
  using namespace vk;
  if (!psi_dev || !kpsi_dev) {
    set_error("vk_fft2d_forward_noalloc: null device pointer");
    return VK_E_INVALID;
  }
  if (!pow2_len(nx) || !pow2_len(ny)) {
    set_error("vk_fft2d_forward_noalloc: nx and ny must be powers of two in [16, 4096]");
    return VK_E_INVALID;
  }
  if ((long)nx * (long)ny > VK_NOALLOC_MAX_POINTS) {
    set_error("vk_fft2d_forward_noalloc: nx*ny exceeds the built-in scratch of 262144 complex points (4 MiB)");
    return VK_E_INVALID;
  }
  DeviceSlots slots;
  int rc = setup_current_device(&slots);
  if (rc) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const double2* in = reinterpret_cast<const double2*>(psi_dev);
  double2* out = reinterpret_cast<double2*>(kpsi_dev);
  double2* scratch = slots.scratch;
  const double2* twx = slots.tw + (nx - 16);
  const double2* twy = slots.tw + (ny - 16);
  with_len_na(nx, [&](auto lc) {
    constexpr int L = decltype(lc)::value;
    typedef GeoX<double, L> G;
    rc = launch_checked("the x pass", k_xfwd<double, L>, ny / G::R, G::NT, sizeof(double2) * G::R * G::LP, st, in,
                        scratch, twx, (int)ny);
  });
  if (rc) return rc;
  with_len_na(ny, [&](auto lc) {
    constexpr int L = decltype(lc)::value;
    typedef GeoY<double, L> G;
    rc = launch_checked("the y pass", k_yfwd<double, L, false>, nx / G::R, G::NT, sizeof(double2) * G::R * G::LP,
                        st, (const double2*)scratch, out, twy, (int)nx, 0, 0.0, 0.0);
  });
  return rc;
}
