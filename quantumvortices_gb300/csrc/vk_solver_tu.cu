// vk_solver_tu.cu -- one compilation of Solver<T> for one precision and one
// set of row lengths.  The build compiles this file ten times:
//   -DVK_TU_FP32=0|1      FP64 or FP32-bulk arithmetic
//   -DVK_TU_CLASS=0..4    row lengths {16, 32, 64, 128}, {128, 256, 512},
//                         {256, 512, 1024}, {512, 1024, 2048}, {1024, 2048, 4096}
// (the sets of solver_len_class in vk_host.cpp; a grid runs in the first set
// that holds both nx and ny).  Splitting by length keeps each compilation to a
// fraction of the kernel instantiations, so they compile in parallel.
#if !defined(VK_TU_FP32) || !defined(VK_TU_CLASS)
#error "compile with -DVK_TU_FP32=0|1 -DVK_TU_CLASS=0..4"
#endif

#if VK_TU_CLASS == 0
#define VK_LEN_MASK 0x0f
#elif VK_TU_CLASS == 1
#define VK_LEN_MASK 0x38
#elif VK_TU_CLASS == 2
#define VK_LEN_MASK 0x70
#elif VK_TU_CLASS == 3
#define VK_LEN_MASK 0xe0
#elif VK_TU_CLASS == 4
#define VK_LEN_MASK 0x1c0
#else
#error "VK_TU_CLASS out of range"
#endif

#define VK_PASTE_(a, b, c) a##b##_c##c
#define VK_PASTE(a, b, c) VK_PASTE_(a, b, c)
#if VK_TU_FP32
#define VK_SOLVER_NS VK_PASTE(solver_, f32, VK_TU_CLASS)
#define VK_FACTORY VK_PASTE(make_solver_, f32, VK_TU_CLASS)
typedef float vk_tu_real;
#else
#define VK_SOLVER_NS VK_PASTE(solver_, f64, VK_TU_CLASS)
#define VK_FACTORY VK_PASTE(make_solver_, f64, VK_TU_CLASS)
typedef double vk_tu_real;
#endif

#include "vk_solver_impl.cuh"

namespace vk {
SolverBase* VK_FACTORY(const vk_params& p, int* status) {
  Solver<vk_tu_real>* s = new Solver<vk_tu_real>(p);
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
