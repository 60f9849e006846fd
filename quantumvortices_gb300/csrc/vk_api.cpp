// vk_api.cpp -- the extern "C" entry points of libvk that touch the GPU.
// Each entry point validates its arguments, forwards to the solver of the
// context's precision and returns a VK_* status (0 = OK).
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include "../../include/vk.h"
#include "vk_solver.h"

using vk::set_error;

namespace {

struct Ctx {
  uint32_t magic;
  vk_params p;
  vk::SolverBase* s;
  vk::StsBase* sts = nullptr;  // spatio-temporal spectra ring (vk_sts_begin)
};
constexpr uint32_t kMagic = 0x56494b53u;  // "VIKS"

Ctx* as_ctx(void* c) {
  Ctx* x = static_cast<Ctx*>(c);
  if (!x || x->magic != kMagic || !x->s) {
    set_error("invalid context");
    return nullptr;
  }
  return x;
}

bool pow2_in_range(int n) { return n >= 16 && n <= 4096 && (n & (n - 1)) == 0; }

}  // namespace

extern "C" int vk_init(const vk_params* p, void** ctx) {
  if (!p || !ctx) { set_error("vk_init: null argument"); return VK_E_INVALID; }
  *ctx = nullptr;
  if (!pow2_in_range(p->nx) || !pow2_in_range(p->ny)) {
    set_error("vk_init: nx, ny must be powers of two in [16, 4096]");
    return VK_E_INVALID;
  }
  if (p->precision != VK_PREC_FP64 && p->precision != VK_PREC_FP32) {
    set_error("vk_init: precision must be VK_PREC_FP64 or VK_PREC_FP32");
    return VK_E_INVALID;
  }
  if (!std::isfinite(p->dt) || !(p->dt > 0) || !std::isfinite(p->alpha) || !std::isfinite(p->gstrength) ||
      !std::isfinite(p->omega_chem) || !std::isfinite(p->disp_factor)) {
    set_error("vk_init: dt must be positive and alpha, g, omega, disp_factor finite");
    return VK_E_INVALID;
  }
  if (p->n_particles < 0) { set_error("vk_init: negative particle count"); return VK_E_INVALID; }
  Ctx* c = new (std::nothrow) Ctx();
  if (!c) { set_error("vk_init: out of host memory"); return VK_E_NOMEM; }
  c->magic = kMagic;
  c->p = *p;
  int rc = VK_OK;
  c->s = (p->precision == VK_PREC_FP64) ? vk::make_solver_f64(*p, &rc) : vk::make_solver_f32(*p, &rc);
  if (!c->s) {
    c->magic = 0;
    delete c;
    return rc ? rc : VK_E_CUDA;
  }
  *ctx = c;
  return VK_OK;
}

extern "C" int vk_finalize(void* ctx) {
  Ctx* c = as_ctx(ctx);
  if (!c) return VK_E_INVALID;
  delete c->sts;
  c->sts = nullptr;
  delete c->s;
  c->s = nullptr;
  c->magic = 0;
  delete c;
  return VK_OK;
}

#define VK_CTX_OR_FAIL(ctx)      \
  Ctx* c = as_ctx(ctx);          \
  if (!c) return VK_E_INVALID;

// NaN or Inf anywhere in a[0..n): an exponent field of all ones.  The scan
// is an OR over the bit patterns, split over the host threads (a 1024^2
// field is 16 MiB: 0.9 ms on one Grace core, 0.1 ms on all of them).
static int check_finite(const double* a, size_t n, const char* what) {
  const uint64_t exp_mask = 0x7FF0000000000000ull;
  uint64_t bad = 0;
#pragma omp parallel for reduction(| : bad) schedule(static) if (n > (1u << 18))
  for (long long i = 0; i < (long long)n; ++i) {
    uint64_t u;
    std::memcpy(&u, a + i, sizeof(u));
    bad |= (uint64_t)((u & exp_mask) == exp_mask);
  }
  if (bad) {
    set_error(std::string(what) + ": input contains NaN or Inf");
    return VK_E_NUMERIC;
  }
  return VK_OK;
}

extern "C" int vk_set_psi(void* ctx, const double* psi) {
  VK_CTX_OR_FAIL(ctx);
  if (!psi) { set_error("vk_set_psi: null psi"); return VK_E_INVALID; }
  int rc = check_finite(psi, 2 * (size_t)c->p.nx * c->p.ny, "vk_set_psi");
  if (rc) return rc;
  return c->s->set_psi(psi);
}

extern "C" int vk_set_kpsi(void* ctx, const double* kpsi) {
  VK_CTX_OR_FAIL(ctx);
  if (!kpsi) { set_error("vk_set_kpsi: null kpsi"); return VK_E_INVALID; }
  int rc = check_finite(kpsi, 2 * (size_t)c->p.nx * c->p.ny, "vk_set_kpsi");
  if (rc) return rc;
  return c->s->set_kpsi(kpsi);
}

extern "C" int vk_get_psi(void* ctx, double* out) {
  VK_CTX_OR_FAIL(ctx);
  if (!out) { set_error("vk_get_psi: null output"); return VK_E_INVALID; }
  return c->s->get_psi(out);
}

extern "C" int vk_get_kpsi(void* ctx, double* out) {
  VK_CTX_OR_FAIL(ctx);
  if (!out) { set_error("vk_get_kpsi: null output"); return VK_E_INVALID; }
  return c->s->get_kpsi(out);
}

extern "C" int vk_gpe_rk4(void* ctx, int32_t nsteps) {
  VK_CTX_OR_FAIL(ctx);
  if (nsteps < 0) { set_error("vk_gpe_rk4: negative step count"); return VK_E_INVALID; }
  return c->s->rk4(nsteps);
}

extern "C" int vk_argle(void* ctx, int32_t nsteps, double* residual_out) {
  VK_CTX_OR_FAIL(ctx);
  if (nsteps < 0) { set_error("vk_argle: negative step count"); return VK_E_INVALID; }
  return c->s->argle(nsteps, residual_out);
}

extern "C" int vk_diagnostics(void* ctx, double* scalars, double* spec, int32_t* nvort) {
  VK_CTX_OR_FAIL(ctx);
  if (!scalars || !spec) { set_error("vk_diagnostics: null output"); return VK_E_INVALID; }
  return c->s->diagnostics(scalars, spec, nvort);
}

extern "C" int vk_particles_set(void* ctx, const double* pos, const double* vel, const double* f0ext) {
  VK_CTX_OR_FAIL(ctx);
  if (c->p.n_particles <= 0) { set_error("vk_particles_set: context has no particles"); return VK_E_STATE; }
  if (!pos || !vel || !f0ext) { set_error("vk_particles_set: null argument"); return VK_E_INVALID; }
  return c->s->particles_set(pos, vel, f0ext);
}

extern "C" int vk_particles_get(void* ctx, double* pos, double* vel, double* frc) {
  VK_CTX_OR_FAIL(ctx);
  if (c->p.n_particles <= 0) { set_error("vk_particles_get: context has no particles"); return VK_E_STATE; }
  return c->s->particles_get(pos, vel, frc);
}

extern "C" int vk_get_stream(void* ctx, void** stream) {
  VK_CTX_OR_FAIL(ctx);
  if (!stream) { set_error("vk_get_stream: null output"); return VK_E_INVALID; }
  *stream = c->s->stream();
  return VK_OK;
}

extern "C" int vk_kernel_launches(void* ctx, int64_t* count) {
  VK_CTX_OR_FAIL(ctx);
  if (!count) { set_error("vk_kernel_launches: null output"); return VK_E_INVALID; }
  *count = c->s->launches();
  return VK_OK;
}

extern "C" int vk_timing_begin(void* ctx) {
  VK_CTX_OR_FAIL(ctx);
  return c->s->timing_begin();
}

extern "C" int vk_timing_end(void* ctx, int32_t cap, char* tags, double* total_ms, int64_t* counts, int32_t* ntags) {
  VK_CTX_OR_FAIL(ctx);
  if (cap < 0 || (cap > 0 && (!tags || !total_ms || !counts)) || !ntags) {
    set_error("vk_timing_end: bad output buffers");
    return VK_E_INVALID;
  }
  int n = 0;
  int rc = c->s->timing_end(cap, tags, total_ms, counts, &n);
  *ntags = n;
  return rc;
}

extern "C" int vk_set_psi_vortices(void* ctx, int32_t n_vort, uint64_t seed, double xi0, double min_sep,
                                   double* pos_out) {
  VK_CTX_OR_FAIL(ctx);
  return c->s->set_psi_vortices(n_vort, seed, xi0, min_sep, pos_out);
}

// ---- spatio-temporal spectra (sts_gpe + Run/CompSTS post-processing) ----

extern "C" int vk_sts_begin(void* ctx, int32_t nt) {
  VK_CTX_OR_FAIL(ctx);
  if (!pow2_in_range(nt)) {
    set_error("vk_sts_begin: nt must be a power of two in [16, 4096]");
    return VK_E_INVALID;
  }
  delete c->sts;
  c->sts = nullptr;
  int st = VK_OK;
  c->sts = vk::make_sts(c->p.nx, c->p.ny, nt, c->s->stream(), &st);
  return st;
}

extern "C" int vk_sts_record(void* ctx) {
  VK_CTX_OR_FAIL(ctx);
  if (!c->sts) {
    set_error("vk_sts_record: no record ring (call vk_sts_begin first)");
    return VK_E_STATE;
  }
  return c->sts->record(c->s);
}

extern "C" int vk_sts_count(void* ctx, int32_t* n) {
  VK_CTX_OR_FAIL(ctx);
  if (!n) {
    set_error("vk_sts_count: null output");
    return VK_E_INVALID;
  }
  *n = c->sts ? c->sts->count() : 0;
  return VK_OK;
}

extern "C" int vk_sts_spectra(void* ctx, double* sts1d, double* sts2d) {
  VK_CTX_OR_FAIL(ctx);
  if (!sts1d || !sts2d) {
    set_error("vk_sts_spectra: null output");
    return VK_E_INVALID;
  }
  if (!c->sts) {
    set_error("vk_sts_spectra: no record ring (call vk_sts_begin first)");
    return VK_E_STATE;
  }
  return c->sts->spectra(sts1d, sts2d);
}

extern "C" int vk_sts_end(void* ctx) {
  VK_CTX_OR_FAIL(ctx);
  delete c->sts;
  c->sts = nullptr;
  return VK_OK;
}

extern "C" int vk_set_variant(void* ctx, const vk_variant* v) {
  VK_CTX_OR_FAIL(ctx);
  if (!v) {
    set_error("vk_set_variant: null variant");
    return VK_E_INVALID;
  }
  return c->s->set_variant(v);
}

extern "C" int vk_get_chempot(void* ctx, double* omega) {
  VK_CTX_OR_FAIL(ctx);
  if (!omega) {
    set_error("vk_get_chempot: null output");
    return VK_E_INVALID;
  }
  return c->s->get_chempot(omega);
}

extern "C" int vk_dump_begin(void* ctx) {
  VK_CTX_OR_FAIL(ctx);
  return c->s->dump_begin();
}

extern "C" int vk_dump_wait(void* ctx, double* psi_phys) {
  VK_CTX_OR_FAIL(ctx);
  if (!psi_phys) {
    set_error("vk_dump_wait: null output");
    return VK_E_INVALID;
  }
  return c->s->dump_wait(psi_phys);
}
