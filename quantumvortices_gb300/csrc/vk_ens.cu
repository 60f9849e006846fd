// vk_ens.cu -- ensemble (batched) stepper and its C ABI.  Compiled twice:
// -DVK_ENS_FP32=0 builds the FP64 ensemble and the C ABI, -DVK_ENS_FP32=1 the
// FP32-bulk ensemble, so the two precisions compile in parallel.
#ifndef VK_ENS_FP32
#error "compile with -DVK_ENS_FP32=0|1"
#endif
#include <cstring>
#include <string>
#include "vk_ensemble.cuh"

namespace vk {

template <typename T> constexpr int Ensemble<T>::XRL[2];
template <typename T> constexpr int Ensemble<T>::YRL[2];

template <typename T>
class EnsembleImpl : public EnsembleBase {
 public:
  Ensemble<T> e;
  int set_psi(int m, const double* psi) override {
    const int rc = e.barrier_check();  // synchronises the ensemble stream
    if (rc) return rc;
    return e.owned[m]->set_psi(psi);
  }
  int get_psi(int m, double* psi) override {
    const int rc = e.barrier_check();
    if (rc) return rc;
    return e.owned[m]->get_psi(psi);
  }
  int rk4(int nsteps) override { return e.rk4(nsteps); }
  const char* report() const override { return e.report.c_str(); }
  void* stream() override { return (void*)e.st; }
  int64_t launches() const override { return e.launches; }
  int size() const override { return e.n; }
};

template <typename T> EnsembleBase* make_ensemble(const vk_params* p, int n, int* status) {
  EnsembleImpl<T>* x = new EnsembleImpl<T>();
  const int rc = x->e.init(p, n);
  if (rc != VK_OK) {
    delete x;
    *status = rc;
    return nullptr;
  }
  *status = VK_OK;
  return x;
}
#if VK_ENS_FP32
EnsembleBase* make_ensemble_f32(const vk_params* p, int n, int* status) { return make_ensemble<float>(p, n, status); }
#else
EnsembleBase* make_ensemble_f64(const vk_params* p, int n, int* status) { return make_ensemble<double>(p, n, status); }
#endif

}  // namespace vk

#if !VK_ENS_FP32

using vk::set_error;

namespace {
struct EnsCtx {
  uint32_t magic;
  vk::EnsembleBase* e;
};
constexpr uint32_t kEnsMagic = 0x454e534du;
EnsCtx* as_ens(void* h) {
  EnsCtx* c = static_cast<EnsCtx*>(h);
  if (!c || c->magic != kEnsMagic || !c->e) {
    set_error("invalid ensemble handle");
    return nullptr;
  }
  return c;
}
}  // namespace

extern "C" int vk_ens_init(const vk_params* members, int32_t n, void** ens) {
  if (!members || !ens || n <= 0) { set_error("vk_ens_init: bad arguments"); return VK_E_INVALID; }
  *ens = nullptr;
  const int prec = members[0].precision;
  for (int i = 0; i < n; ++i)
    if (members[i].precision != prec) { set_error("vk_ens_init: members must share one precision"); return VK_E_INVALID; }
  int rc = VK_OK;
  vk::EnsembleBase* e = prec == VK_PREC_FP64 ? vk::make_ensemble_f64(members, n, &rc)
                                             : vk::make_ensemble_f32(members, n, &rc);
  if (!e) return rc ? rc : VK_E_CUDA;
  *ens = new EnsCtx{kEnsMagic, e};
  return VK_OK;
}

extern "C" int vk_ens_finalize(void* ens) {
  EnsCtx* c = as_ens(ens);
  if (!c) return VK_E_INVALID;
  delete c->e;
  c->magic = 0;
  delete c;
  return VK_OK;
}

extern "C" int vk_ens_set_psi(void* ens, int32_t m, const double* psi) {
  EnsCtx* c = as_ens(ens);
  if (!c) return VK_E_INVALID;
  if (m < 0 || m >= c->e->size() || !psi) { set_error("vk_ens_set_psi: bad member or pointer"); return VK_E_INVALID; }
  return c->e->set_psi(m, psi);
}

extern "C" int vk_ens_get_psi(void* ens, int32_t m, double* psi) {
  EnsCtx* c = as_ens(ens);
  if (!c) return VK_E_INVALID;
  if (m < 0 || m >= c->e->size() || !psi) { set_error("vk_ens_get_psi: bad member or pointer"); return VK_E_INVALID; }
  return c->e->get_psi(m, psi);
}

extern "C" int vk_ens_gpe_rk4(void* ens, int32_t nsteps) {
  EnsCtx* c = as_ens(ens);
  if (!c) return VK_E_INVALID;
  if (nsteps < 0) { set_error("vk_ens_gpe_rk4: negative step count"); return VK_E_INVALID; }
  return c->e->rk4(nsteps);
}

extern "C" int vk_ens_report(void* ens, char* buf, int32_t cap) {
  EnsCtx* c = as_ens(ens);
  if (!c) return VK_E_INVALID;
  if (!buf || cap <= 0) { set_error("vk_ens_report: bad buffer"); return VK_E_INVALID; }
  std::strncpy(buf, c->e->report(), (size_t)cap - 1);
  buf[cap - 1] = 0;
  return VK_OK;
}

extern "C" int vk_ens_get_stream(void* ens, void** stream) {
  EnsCtx* c = as_ens(ens);
  if (!c) return VK_E_INVALID;
  if (!stream) { set_error("vk_ens_get_stream: null output"); return VK_E_INVALID; }
  *stream = c->e->stream();
  return VK_OK;
}

extern "C" int vk_ens_kernel_launches(void* ens, int64_t* count) {
  EnsCtx* c = as_ens(ens);
  if (!c) return VK_E_INVALID;
  if (!count) { set_error("vk_ens_kernel_launches: null output"); return VK_E_INVALID; }
  *count = c->e->launches();
  return VK_OK;
}
#endif  // !VK_ENS_FP32
