// vk_f64.cu -- plain FP64 instantiation of the solver.
#include "vk_solver_impl.cuh"

namespace vk {
SolverBase* make_solver_f64(const vk_params& p, int* status) {
  Solver<double>* s = new Solver<double>(p);
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
