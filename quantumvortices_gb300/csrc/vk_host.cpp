// vk_host.cpp -- host-only parts of libvk: parameter handling, the
// reference's file formats, FFT tables and the seeded vortex initial state.
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>
#include "../../include/vk.h"
#include "vk_solver.h"

namespace vk {

static thread_local std::string g_err;
void set_error(const std::string& msg) { g_err = msg; }

static const double kPi = 3.14159265358979323846264338327950288;

// cos/sin(2 pi k/n) with octant reduction to [0, pi/4].
static void cis2pi(long k, long n, double* c, double* s) {
  k %= n;
  if (k < 0) k += n;
  int negs = 0, negc = 0, swp = 0;
  if (2 * k > n) { k = n - k; negs = 1; }
  if ((n % 2 == 0) && 4 * k > n) { k = n / 2 - k; negc = 1; }
  if ((n % 4 == 0) && 8 * k > n) { k = n / 4 - k; swp = 1; }
  const double th = 2.0 * kPi * (double)k / (double)n;
  double cc = std::cos(th), ss = std::sin(th);
  if (swp) std::swap(cc, ss);
  if (negc) cc = -cc;
  if (negs) ss = -ss;
  *c = cc;
  *s = ss;
}

void twiddle_table(int n, double* out) {
  for (int k = 0; k < n; ++k) {
    double c, s;
    cis2pi(k, n, &c, &s);
    out[2 * k] = c;
    out[2 * k + 1] = -s;
  }
}

// IF (ksqr .GE. kalias**2) with kalias = REAL(Nx)/3 (src/mod_grid.f90:92,
// src/gpe.f90:571): the largest integer k1^2+k2^2 that survives.
int k2max_for(int nx) {
  const double kalias = (double)nx / 3.0;
  const double ka2 = kalias * kalias;
  long k = (long)std::floor(ka2) + 1;
  while (k > 0 && (double)k >= ka2) --k;
  return (int)k;
}

int kmax_for(int k2max) {
  int k = (int)std::sqrt((double)k2max);
  while ((long)(k + 1) * (k + 1) <= k2max) ++k;
  while ((long)k * k > k2max) --k;
  return k;
}

// Bit i of a mask: row length 16 << i.  Must match VK_LEN_MASK in vk_solver_tu.cu.
static const int kLenClassMask[5] = {0x0f, 0x38, 0x70, 0xe0, 0x1c0};

int solver_len_class(int nx, int ny) {
  auto bit = [](int n) {
    for (int i = 0; i < 9; ++i)
      if (n == (16 << i)) return 1 << i;
    return 0;
  };
  const int want = bit(nx) | bit(ny);
  if (!bit(nx) || !bit(ny)) return -1;
  for (int c = 0; c < 5; ++c)
    if ((kLenClassMask[c] & want) == want) return c;
  return -1;
}

typedef SolverBase* (*SolverFactory)(const vk_params&, int*);
static const SolverFactory kF64[5] = {make_solver_f64_c0, make_solver_f64_c1, make_solver_f64_c2,
                                      make_solver_f64_c3, make_solver_f64_c4};
static const SolverFactory kF32[5] = {make_solver_f32_c0, make_solver_f32_c1, make_solver_f32_c2,
                                      make_solver_f32_c3, make_solver_f32_c4};

static SolverBase* make_solver_in_class(const SolverFactory* table, const vk_params& p, int* status) {
  const int c = solver_len_class(p.nx, p.ny);
  if (c < 0) {
    set_error("vk_init: no row-length class holds both nx and ny (classes {16..128}, {128..512}, {256..1024}, "
              "{512..2048}, {1024..4096})");
    *status = VK_E_INVALID;
    return nullptr;
  }
  return table[c](p, status);
}
SolverBase* make_solver_f64(const vk_params& p, int* status) { return make_solver_in_class(kF64, p, status); }
SolverBase* make_solver_f32(const vk_params& p, int* status) { return make_solver_in_class(kF32, p, status); }

}  // namespace vk

using vk::set_error;
static const double kPi = 3.14159265358979323846264338327950288;

extern "C" const char* vk_last_error(void) { return vk::g_err.c_str(); }

// nshell = int(1.414*Nx/2.0d0) + 1 (src/mod_grid.f90:77): 1.414 is a default
// REAL literal, so 1.414*Nx is evaluated in single precision.
extern "C" int32_t vk_nshell(int32_t nx) {
  const float prod = 1.414f * (float)nx;
  return (int32_t)((double)prod / 2.0) + 1;
}

// ------------------------------------------------------------ namelists --

namespace {

std::string lower(std::string s) {
  for (auto& ch : s) ch = (char)std::tolower((unsigned char)ch);
  return s;
}

// Parses every &group ... / block of a Fortran namelist file into
// group -> (key -> raw value).  '!' starts a comment; keys are case-blind.
bool parse_namelist_file(const char* path, std::map<std::string, std::map<std::string, std::string>>& out) {
  std::ifstream f(path);
  if (!f) return false;
  std::string line, group;
  while (std::getline(f, line)) {
    const size_t bang = line.find('!');
    if (bang != std::string::npos) line = line.substr(0, bang);
    std::string t = line;
    // trim
    size_t a = t.find_first_not_of(" \t\r");
    if (a == std::string::npos) continue;
    t = t.substr(a);
    if (t[0] == '&') {
      size_t e = t.find_first_of(" \t\r", 1);
      group = lower(t.substr(1, e == std::string::npos ? std::string::npos : e - 1));
      continue;
    }
    if (t[0] == '/') { group.clear(); continue; }
    if (group.empty()) continue;
    // key=value pairs separated by commas
    std::stringstream ss(t);
    std::string item;
    while (std::getline(ss, item, ',')) {
      size_t eq = item.find('=');
      if (eq == std::string::npos) continue;
      std::string k = item.substr(0, eq), v = item.substr(eq + 1);
      auto trim = [](std::string s) {
        size_t b = s.find_first_not_of(" \t\r"), e = s.find_last_not_of(" \t\r");
        return b == std::string::npos ? std::string() : s.substr(b, e - b + 1);
      };
      out[group][lower(trim(k))] = trim(v);
    }
  }
  return true;
}

// Fortran real literal (1.0d-3, 0.2d0, 5) -> double; longest valid prefix.
bool fortran_real(const std::string& v, double* out) {
  std::string s = v;
  for (auto& ch : s)
    if (ch == 'd' || ch == 'D') ch = 'e';
  char* end = nullptr;
  const double x = std::strtod(s.c_str(), &end);
  if (end == s.c_str()) return false;
  *out = x;
  return true;
}

template <typename F>
void get(const std::map<std::string, std::map<std::string, std::string>>& nl, const char* grp, const char* key, F set) {
  auto g = nl.find(grp);
  if (g == nl.end()) return;
  auto k = g->second.find(key);
  if (k == g->second.end()) return;
  double x;
  if (fortran_real(k->second, &x)) set(x);
}

}  // namespace

extern "C" int vk_read_namelists(const char* parameter_txt, const char* parameter_gpe_txt, vk_namelist* out) {
  if (!out) { set_error("vk_read_namelists: null output"); return VK_E_INVALID; }
  std::memset(out, 0, sizeof(*out));
  // defaults matching the shipped parameter files where a key is absent
  out->csound = 1.0;
  out->rho_avg = 1.0;
  out->xi = 1.0;
  std::map<std::string, std::map<std::string, std::string>> nl;
  if (parameter_txt && !parse_namelist_file(parameter_txt, nl)) {
    set_error(std::string("cannot open ") + parameter_txt);
    return VK_E_IO;
  }
  if (parameter_gpe_txt && !parse_namelist_file(parameter_gpe_txt, nl)) {
    set_error(std::string("cannot open ") + parameter_gpe_txt);
    return VK_E_IO;
  }
  get(nl, "resolution", "nx", [&](double x) { out->nx = (int32_t)x; });
  get(nl, "resolution", "ny", [&](double x) { out->ny = (int32_t)x; });
  get(nl, "tparam", "dt_fix", [&](double x) { out->dt_fix = x; });
  get(nl, "tparam", "maxiter", [&](double x) { out->maxiter = (int32_t)x; });
  get(nl, "tparam", "fsteps", [&](double x) { out->fsteps = (int32_t)x; });
  get(nl, "tparam", "ssteps", [&](double x) { out->ssteps = (int32_t)x; });
  get(nl, "tparam", "gsteps", [&](double x) { out->gsteps = (int32_t)x; });
  get(nl, "ckprst", "nrst", [&](double x) { out->nrst = (int32_t)x; });
  get(nl, "ckprst", "sprst", [&](double x) { out->sprst = (int32_t)x; });
  get(nl, "ckprst", "strst", [&](double x) { out->strst = (int32_t)x; });
  get(nl, "tparam", "ststeps", [&](double x) { out->ststeps = (int32_t)x; });
  get(nl, "gpparam", "xi", [&](double x) { out->xi = x; });
  get(nl, "gpparam", "csound", [&](double x) { out->csound = x; });
  get(nl, "gpparam", "rho_avg", [&](double x) { out->rho_avg = x; });
  get(nl, "gpparam", "disp_factor", [&](double x) { out->disp_factor = x; });
  get(nl, "gpotoc", "k_otoc_gp", [&](double x) { out->k_otoc_gp = x; });
  get(nl, "gpotoc", "eps_otoc_gp", [&](double x) { out->eps_otoc_gp = x; });
  get(nl, "gpparticle", "gp_n_obj", [&](double x) { out->gp_n_obj = (int32_t)x; });
  get(nl, "gpparticle", "gp_mass_part", [&](double x) { out->gp_mass_part = x; });
  get(nl, "gpparticle", "ppotd", [&](double x) { out->ppotd = x; });
  get(nl, "gpparticle", "ppotv0", [&](double x) { out->ppotv0 = x; });
  get(nl, "gpparticle", "ppotthick", [&](double x) { out->ppotthick = x; });
  get(nl, "gpforceparam", "famp_gp", [&](double x) { out->famp_gp = x; });
  get(nl, "gpforceparam", "kf1_gp", [&](double x) { out->kf1_gp = x; });
  get(nl, "gpforceparam", "kf2_gp", [&](double x) { out->kf2_gp = x; });
  get(nl, "gphypvis", "vishypo_gp", [&](double x) { out->vishypo_gp = x; });
  get(nl, "gphypvis", "vishype_gp", [&](double x) { out->vishype_gp = x; });
  get(nl, "gpcounterflow", "vnx", [&](double x) { out->vnx = x; });
  get(nl, "gpcounterflow", "vny", [&](double x) { out->vny = x; });
  get(nl, "gpfinitet", "oneybeta", [&](double x) { out->oneybeta = x; });
  get(nl, "gpfinitet", "nun", [&](double x) { out->nun = x; });
  get(nl, "gpfinitet", "chempot0", [&](double x) { out->chempot0 = x; });
  get(nl, "selftruncation", "ktrunc", [&](double x) { out->ktrunc = x; });
  get(nl, "fileparam", "nsplit_orignal", [&](double x) { out->nsplit_orignal = (int32_t)x; });
  get(nl, "fileparam", "nsplit_current", [&](double x) { out->nsplit_current = (int32_t)x; });
  return VK_OK;
}

extern "C" int vk_variant_derive(const vk_namelist* nl, int32_t flags, uint64_t seed, vk_variant* out) {
  if (!nl || !out) { set_error("vk_variant_derive: null argument"); return VK_E_INVALID; }
  std::memset(out, 0, sizeof(*out));
  const double kdx = 1.0;  // 2 pi / lengthx with lengthx = 2 pi (src/mod_grid.f90)
  out->flags = flags;
  out->famp_gp = nl->famp_gp;
  out->kf1_gp = nl->kf1_gp * kdx;
  out->kf2_gp = nl->kf2_gp * kdx;
  out->vishypo_gp = nl->vishypo_gp;
  out->vishype_gp = nl->vishype_gp;
  out->vnx = nl->vnx;
  out->vny = nl->vny;
  out->oneybeta = nl->oneybeta;
  out->nuN = nl->nun;
  out->chempot0 = nl->chempot0;
  out->ktrunc = nl->ktrunc;
  out->seed = seed;
  return VK_OK;
}

static bool pow2_in_range(int n) { return n >= 16 && n <= 4096 && (n & (n - 1)) == 0; }

extern "C" int vk_params_derive(const vk_namelist* nl, int32_t precision, int32_t otoc, vk_params* p) {
  if (!nl || !p) { set_error("vk_params_derive: null argument"); return VK_E_INVALID; }
  if (!pow2_in_range(nl->nx) || !pow2_in_range(nl->ny)) {
    set_error("Nx, Ny must be powers of two in [16, 4096]");
    return VK_E_INVALID;
  }
  if (!(nl->csound > 0) || !(nl->xi > 0) || !(nl->rho_avg > 0)) {
    set_error("xi, csound and rho_avg must be positive");
    return VK_E_INVALID;
  }
  std::memset(p, 0, sizeof(*p));
  p->nx = nl->nx;
  p->ny = nl->ny;
  p->precision = precision;
  p->otoc = otoc;
  p->dt = nl->dt_fix;  // dt = dt_fix (src/driver.f90:272)
  // set_grid: dx = lengthx/Nx with lengthx = two*pi (src/mod_grid.f90:79-82)
  const double dx = (2.0 * kPi) / nl->nx;
  // src/driver.f90:362-370
  const double xi = nl->xi * dx;
  const double alpha = nl->csound * xi * std::sqrt(nl->rho_avg / 2.0);
  const double g = (nl->csound * nl->csound) / (2.0 * alpha);
  p->xi = xi;
  p->alpha = alpha;
  p->gstrength = g;
  p->omega_chem = g;
  p->disp_factor = nl->disp_factor;
  p->k_otoc_gp = nl->k_otoc_gp;
  p->eps_otoc_gp = nl->eps_otoc_gp;
  // particles: src/driver.f90:391-392
  p->n_particles = nl->gp_n_obj;
  p->ppot_v0 = nl->ppotv0 * g;
  p->ppot_d = nl->ppotd * xi;
  p->gp_mass_part = nl->gp_mass_part;
  return VK_OK;
}

// ------------------------------------------------------------- wf files --
// Fortran sequential unformatted: each record is <int32 len> payload <int32 len>.

static bool write_record(std::FILE* f, const void* data, uint32_t len) {
  return std::fwrite(&len, 4, 1, f) == 1 && (len == 0 || std::fwrite(data, 1, len, f) == len) &&
         std::fwrite(&len, 4, 1, f) == 1;
}

extern "C" int vk_write_wf(const char* path, int32_t iopoint, double time, double dt, int32_t nx, int32_t ny,
                           const double* psi) {
  if (!path || !psi || nx <= 0 || ny <= 0) { set_error("vk_write_wf: bad argument"); return VK_E_INVALID; }
  std::FILE* f = std::fopen(path, "wb");
  if (!f) { set_error(std::string("vk_write_wf: cannot create ") + path); return VK_E_IO; }
  unsigned char hdr[20];
  std::memcpy(hdr, &iopoint, 4);
  std::memcpy(hdr + 4, &time, 8);
  std::memcpy(hdr + 12, &dt, 8);
  bool ok = write_record(f, hdr, 20);
  for (int32_t y = 0; ok && y < ny; ++y) ok = write_record(f, psi + (size_t)2 * nx * y, (uint32_t)(16u * nx));
  if (std::fclose(f) != 0) ok = false;
  if (!ok) { set_error(std::string("vk_write_wf: write failed on ") + path); return VK_E_IO; }
  return VK_OK;
}

static bool read_record(std::FILE* f, void* data, uint32_t expect) {
  uint32_t a = 0, b = 0;
  if (std::fread(&a, 4, 1, f) != 1 || a != expect) return false;
  if (std::fread(data, 1, expect, f) != expect) return false;
  if (std::fread(&b, 4, 1, f) != 1 || b != expect) return false;
  return true;
}

extern "C" int vk_read_wf(const char* path, int32_t nx, int32_t ny, int32_t* iopoint, double* time, double* dt,
                          double* psi) {
  if (!path || !psi || nx <= 0 || ny <= 0) { set_error("vk_read_wf: bad argument"); return VK_E_INVALID; }
  std::FILE* f = std::fopen(path, "rb");
  if (!f) { set_error(std::string("vk_read_wf: cannot open ") + path); return VK_E_IO; }
  unsigned char hdr[20];
  if (!read_record(f, hdr, 20)) {
    std::fclose(f);
    set_error(std::string("vk_read_wf: bad header record in ") + path);
    return VK_E_IO;
  }
  int32_t io;
  double t, d;
  std::memcpy(&io, hdr, 4);
  std::memcpy(&t, hdr + 4, 8);
  std::memcpy(&d, hdr + 12, 8);
  for (int32_t y = 0; y < ny; ++y) {
    if (!read_record(f, psi + (size_t)2 * nx * y, (uint32_t)(16u * nx))) {
      std::fclose(f);
      set_error(std::string("vk_read_wf: truncated or wrong record length in ") + path);
      return VK_E_IO;
    }
  }
  std::fclose(f);
  if (iopoint) *iopoint = io;
  if (time) *time = t;
  if (dt) *dt = d;
  return VK_OK;
}

// Regrouping of a field written by nsplit ranks (src/io_fields.f90:121-146,
// -DIOEVERYPROC with nsplit_orignal > nsplit_current = 1): files
// <prefix>p1.dat .. <prefix>p<nsplit>.dat, each a header record and ny/nsplit
// rows of nx complex128, concatenated along y in file order.
extern "C" int vk_read_wf_split(const char* prefix, int32_t nsplit, int32_t nx, int32_t ny, int32_t* iopoint,
                                double* time, double* dt, double* psi) {
  if (!prefix || !psi || nsplit <= 0 || nx <= 0 || ny <= 0 || ny % nsplit != 0) {
    set_error("vk_read_wf_split: bad argument (ny must be a multiple of nsplit)");
    return VK_E_INVALID;
  }
  const int32_t rows = ny / nsplit;
  for (int32_t j = 1; j <= nsplit; ++j) {
    const std::string path = std::string(prefix) + "p" + std::to_string(j) + ".dat";
    const int rc = vk_read_wf(path.c_str(), nx, rows, iopoint, time, dt, psi + (size_t)2 * nx * rows * (j - 1));
    if (rc != VK_OK) return rc;
  }
  return VK_OK;
}

// ------------------------------------------------------ vortex initial state --

namespace {
struct SplitMix64 {
  uint64_t s;
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
};

inline double wrap_pi(double d) {  // into (-pi, pi]
  const double L = 2.0 * kPi;
  d = std::fmod(d, L);
  if (d > kPi) d -= L;
  if (d <= -kPi) d += L;
  return d;
}
}  // namespace

// Phase of a neutral vortex set on the 2pi-periodic square: each vortex
// contributes arg theta_1((z - z_j)/2 | q = e^{-pi}) (the odd Jacobi theta
// function, zeros exactly at the periodic images of z_j), and the linear
// term -y * sum_j q_j x_j / (2 pi) cancels the quasi-periodicity in y.
namespace vk {
// Seeded neutral vortex positions: SplitMix64(seed) uniform on [0,2pi)^2,
// periodic minimum separation min_sep; charge +1 for the first half, -1 after.
int vortex_positions(int n_vort, uint64_t seed, double min_sep, std::vector<double>& px, std::vector<double>& py,
                     std::vector<int>& qc) {
  const double L = 2.0 * kPi;
  px.assign(n_vort, 0.0);
  py.assign(n_vort, 0.0);
  qc.assign(n_vort, 0);
  SplitMix64 rng{seed};
  for (int j = 0; j < n_vort; ++j) {
    int tries = 0;
    for (;;) {
      const double x = L * rng.uniform(), y = L * rng.uniform();
      bool ok = true;
      for (int i = 0; i < j && ok; ++i) {
        const double dx = wrap_pi(x - px[i]), dy = wrap_pi(y - py[i]);
        if (std::sqrt(dx * dx + dy * dy) < min_sep) ok = false;
      }
      if (ok) { px[j] = x; py[j] = y; break; }
      if (++tries > 1000000) {
        set_error("vortex IC: cannot place vortices with this minimum separation");
        return VK_E_INVALID;
      }
    }
    qc[j] = (j < n_vort / 2) ? +1 : -1;
  }
  return VK_OK;
}
}  // namespace vk

extern "C" int vk_ic_vortices(int32_t nx, int32_t ny, int32_t n_vort, uint64_t seed, double xi0, double min_sep,
                              double* psi, double* pos_out) {
  if (!psi || nx <= 0 || ny <= 0 || n_vort < 0 || (n_vort % 2) != 0 || !(xi0 > 0)) {
    set_error("vk_ic_vortices: need an even (neutral) vortex count, positive xi0 and a grid");
    return VK_E_INVALID;
  }
  const double L = 2.0 * kPi;
  std::vector<double> px, py;
  std::vector<int> qc;
  int prc = vk::vortex_positions(n_vort, seed, min_sep, px, py, qc);
  if (prc) return prc;
  double S = 0.0;
  for (int j = 0; j < n_vort; ++j) S += qc[j] * px[j];
  const int NT = 9;  // theta product terms: q^{2n} e^{2 pi} < 1e-20 for n = 9
  const double qn = std::exp(-kPi);
  double q2n[NT + 1];
  for (int n = 1; n <= NT; ++n) q2n[n] = std::pow(qn, 2.0 * n);
  const double dxg = L / nx, dyg = L / ny;
#pragma omp parallel for schedule(static)
  for (int y = 0; y < ny; ++y) {
    const double yy = y * dyg;
    for (int x = 0; x < nx; ++x) {
      const double xx = x * dxg;
      double amp = 1.0, pr = 1.0, pi_ = 0.0;
      for (int j = 0; j < n_vort; ++j) {
        const double ddx = xx - px[j], ddy = yy - py[j];
        const double wx = wrap_pi(ddx), wy = wrap_pi(ddy);
        const double r = std::sqrt(wx * wx + wy * wy) / xi0;
        amp *= r / std::sqrt(2.0 + r * r);
        // theta_1(v), v = (ddx + i ddy)/2: sin(v) * prod (1 - q^2n e^{2iv})(1 - q^2n e^{-2iv})
        const double a = 0.5 * ddx, b = 0.5 * ddy;
        double fr = std::sin(a) * std::cosh(b), fi = std::cos(a) * std::sinh(b);
        const double c2 = std::cos(ddx), s2 = std::sin(ddx);
        const double em = std::exp(-ddy), ep = std::exp(ddy);  // |e^{2iv}| = e^{-ddy}
        for (int n = 1; n <= NT; ++n) {
          const double r1 = q2n[n] * em, r2 = q2n[n] * ep;
          // (1 - r1 e^{i ddx}) (1 - r2 e^{-i ddx})
          const double ar = 1.0 - r1 * c2, ai = -r1 * s2;
          const double br = 1.0 - r2 * c2, bi = r2 * s2;
          const double tr = ar * br - ai * bi, ti = ar * bi + ai * br;
          const double nr = fr * tr - fi * ti, ni = fr * ti + fi * tr;
          fr = nr;
          fi = ni;
        }
        const double m = std::hypot(fr, fi);
        if (m > 0) {
          fr /= m;
          fi /= m;
        } else {
          fr = 1.0;
          fi = 0.0;
        }
        if (qc[j] < 0) fi = -fi;
        const double nr = pr * fr - pi_ * fi, ni = pr * fi + pi_ * fr;
        pr = nr;
        pi_ = ni;
      }
      const double lin = -yy * S / L;
      const double cr = std::cos(lin), ci = std::sin(lin);
      const double fr = pr * cr - pi_ * ci, fi = pr * ci + pi_ * cr;
      const double m = std::hypot(fr, fi);
      psi[2 * ((size_t)y * nx + x)] = amp * fr / m;
      psi[2 * ((size_t)y * nx + x) + 1] = amp * fi / m;
    }
  }
  if (pos_out)
    for (int j = 0; j < n_vort; ++j) {
      pos_out[2 * j] = px[j];
      pos_out[2 * j + 1] = py[j];
    }
  return VK_OK;
}
