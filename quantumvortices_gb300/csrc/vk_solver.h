// vk_solver.h -- host-side solver interface behind the C ABI.
#pragma once
#include <string>
#include <cstdint>
#include <vector>
#include "../../include/vk.h"

namespace vk {

// Thread-local error message used by vk_last_error().
void set_error(const std::string& msg);

class SolverBase {
 public:
  virtual ~SolverBase() {}
  virtual int set_psi(const double* psi) = 0;
  virtual int set_kpsi(const double* kpsi) = 0;
  virtual int set_psi_vortices(int n_vort, uint64_t seed, double xi0, double min_sep, double* pos_out) = 0;
  virtual int get_psi(double* psi) = 0;
  virtual int get_kpsi(double* kpsi) = 0;
  virtual int rk4(int nsteps) = 0;
  virtual int argle(int nsteps, double* residual) = 0;
  virtual int diagnostics(double* scalars, double* spec, int32_t* nvort) = 0;
  virtual int particles_set(const double* pos, const double* vel, const double* f0ext) = 0;
  virtual int particles_get(double* pos, double* vel, double* frc) = 0;
  virtual void* stream() = 0;
  virtual int64_t launches() const = 0;
  virtual int timing_begin() = 0;
  virtual int timing_end(int cap, char* tags, double* ms, int64_t* counts, int* ntags) = 0;
  // Ensemble support: copy this field's device view (a Field<T>), query and
  // update the state flags around batched steps.
  virtual int field_view(void* out, size_t size) = 0;
  // Copies kpsi (all nx*ny modes) as FP64 into dst (device double2), on
  // this solver's stream.
  virtual int snapshot_kpsi_f64(void* dst) = 0;
  // Compile-time branches of the reference selected at run time.
  virtual int set_variant(const vk_variant* v) = 0;
  virtual int get_chempot(double* omega) = 0;
  // Asynchronous psi dump: snapshot on the device, copy to pinned host memory
  // on a second stream; dump_wait blocks for it and copies it out.
  virtual int dump_begin() = 0;
  virtual int dump_wait(double* psi) = 0;
  virtual bool kpsi_is_masked() const = 0;
  virtual void mark_rk4_done() = 0;
};

// Factories (one per precision).  They pick the compilation of Solver<T>
// whose row-length set holds both nx and ny (solver_len_class) and fail with
// VK_E_INVALID when none does.
SolverBase* make_solver_f64(const vk_params& p, int* status);
SolverBase* make_solver_f32(const vk_params& p, int* status);
// Row-length class of an nx x ny grid: the first of the sets {16, 32, 64, 128},
// {128, 256, 512}, {256, 512, 1024}, {512, 1024, 2048}, {1024, 2048, 4096}
// holding both lengths, or -1.  Every grid with nx, ny <= 128 or with
// max/min <= 4 has one.
int solver_len_class(int nx, int ny);
#define VK_DECLARE_SOLVER_CLASS(k)                                   \
  SolverBase* make_solver_f64_c##k(const vk_params& p, int* status); \
  SolverBase* make_solver_f32_c##k(const vk_params& p, int* status);
VK_DECLARE_SOLVER_CLASS(0)
VK_DECLARE_SOLVER_CLASS(1)
VK_DECLARE_SOLVER_CLASS(2)
VK_DECLARE_SOLVER_CLASS(3)
VK_DECLARE_SOLVER_CLASS(4)
#undef VK_DECLARE_SOLVER_CLASS

// Ensembles of independent fields stepped by batched persistent kernels.
class EnsembleBase {
 public:
  virtual ~EnsembleBase() {}
  virtual int set_psi(int m, const double* psi) = 0;
  virtual int get_psi(int m, double* psi) = 0;
  virtual int rk4(int nsteps) = 0;
  virtual const char* report() const = 0;
  virtual void* stream() = 0;
  virtual int64_t launches() const = 0;
  virtual int size() const = 0;
};
EnsembleBase* make_ensemble_f64(const vk_params* p, int n, int* status);
EnsembleBase* make_ensemble_f32(const vk_params* p, int n, int* status);

// Spatio-temporal spectra recorder (vk_sts.cu).
class StsBase {
 public:
  virtual ~StsBase() {}
  virtual int record(SolverBase* s) = 0;
  virtual int count() const = 0;
  virtual int spectra(double* sts1d, double* sts2d) = 0;
};
StsBase* make_sts(int nx, int ny, int nt, void* stream, int* status);

// Host helpers shared by both precisions (vk_host.cpp).
void twiddle_table(int n, double* out_interleaved);      // exp(-2 pi i k/n), k < n
int k2max_for(int nx);                                     // largest k1^2+k2^2 kept by the 2/3 rule
int kmax_for(int k2max);                                   // largest |k| with k^2 <= k2max
int vortex_positions(int n_vort, uint64_t seed, double min_sep, std::vector<double>& px,
                     std::vector<double>& py, std::vector<int>& qc);

}  // namespace vk
