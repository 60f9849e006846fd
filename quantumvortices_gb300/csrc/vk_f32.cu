// vk_f32.cu -- FP32-bulk instantiation (FP64 twiddle generation, FP64 reductions).
#include "vk_solver_impl.cuh"

namespace vk {
SolverBase* make_solver_f32(const vk_params& p, int* status) {
  Solver<float>* s = new Solver<float>(p);
  int rc = s->init();
  if (rc != VK_OK) {
    delete s;
    *status = rc;
    return nullptr;
  }
  *status = VK_OK;
  return s;
}
}  // namespace vk
