// vk_diag.cuh -- diagnostics_gpe on the GPU (placeholder until the spectra
// kernels land).
#pragma once
#include "vk_kernels.cuh"
#include "vk_solver.h"

namespace vk {

template <typename T>
struct Diagnostics {
  template <typename S>
  int run(S&, double*, double*, int32_t*) {
    set_error("vk_diagnostics: not available yet");
    return VK_E_STATE;
  }
  void release() {}
};

}  // namespace vk
