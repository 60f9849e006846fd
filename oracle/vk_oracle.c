/*
 * vk_oracle.c -- CPU FP64 restatement of the VIKSHOBHA 2D GPE hot path.
 *
 * TEST INFRASTRUCTURE ONLY (the checker, never the product): loaded by
 * tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg.
 * PARITY UNPINNED against the reference binary (Fortran+FFTW+MPI cannot be
 * built on these machines; the reference has no tests or golden vectors).
 *
 * Every routine follows the reference line by line, in the same arithmetic
 * order where that is visible in the source; the comments cite the file and
 * lines (paths relative to the reference project root).  The FFT is this
 * file's own radix-2 FP64 transform (FFTW 3.3.8's plan-dependent rounding is
 * not reproducible); tests cross-check it against numpy.fft.
 *
 * One deliberate deviation: the uninitialised
 * `ksqr` used as the dealias test in translate_particle_potential
 * (src/gpe_particle.f90:275, declared :206) is replaced by the intended
 * k1^2+k2^2 of the current mode.
 */
#include "vk_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct { double re, im; } cx;

static inline cx cmul(cx a, cx b) { cx r = {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; return r; }
static inline cx cadd(cx a, cx b) { cx r = {a.re + b.re, a.im + b.im}; return r; }
static inline cx csub(cx a, cx b) { cx r = {a.re - b.re, a.im - b.im}; return r; }
static inline cx crmul(double s, cx a) { cx r = {s * a.re, s * a.im}; return r; }
static inline cx cconj(cx a) { cx r = {a.re, -a.im}; return r; }
/* Fortran ABS() of a complex is the modulus (hypot). */
static inline double cabs_f(cx a) { return hypot(a.re, a.im); }

static const double PI = 3.14159265358979323846264338327950288;

struct vko_state {
  vko_params p;
  int nx, ny;
  size_t n2;
  double lx, ly, dx, dy, dvol, kalias, ka2, fftwscale, nparticle;
  int nshell;
  int *kwn1, *kwn2;
  cx *psi, *kpsi, *nlin, *cmpxtmp, *str1, *str2, *tmp1, *tmp2, *tmp3;
  cx *vobj, *trans_vobj;
  /* FFT tables */
  cx *twx, *twy;
  int *brx, *bry;
  cx *work;
  /* particles (gpe_particle.f90, mod_gpparticles.f90) */
  int np;
  double *pos, *vel, *frc, *f0ext, *tpos, *tvel, *ku[4], *kq[4], *shortrange;
  double gpfrcpart[2];
  double gpdeltaE, gpr0obj; /* set by shortrange_repulsion (gpe_particle.f90:395-396) */
  /* -DGPE_FRCDISP (gpe.f90:623-658): hypo/hyperviscosity, random-phase forcing */
  int frcdisp;
  double vishypo, vishype, famp, kf1, kf2;
  uint64_t seed, ctr; /* forcing phases: uniform(seed, ctr, mode), ctr = RHS evaluations so far */
  /* ARGLE flow terms: 1 = -DGPE_ADVECTION (Taylor-Green), 2 = -DGPE_COUNTERFLOW */
  int flow;
  double vnx, vny;
  /* -DGPE_SGLE (gpe.f90:149-178, 199-219, 226-274) and -DGPE_SELFTRUNC */
  int sgle, selftrunc;
  double noisesigma, nuN, ktrunc;
};

/* Counter-based uniform [0,1) for the forcing phases: the GPU kernels use
 * the same definition (SplitMix64 finaliser of seed, counter and mode).  It
 * stands in for the reference's RANDOM_NUMBER, whose stream is compiler
 * dependent: parity with the reference is statistical for the forcing. */
static inline uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
static inline double frc_uniform(uint64_t seed, uint64_t ctr, uint64_t mode) {
  return (double)(mix64(mix64(seed ^ (ctr * 0xD1B54A32D192ED03ull)) + mode) >> 11) * (1.0 / 9007199254740992.0);
}

/* Standard normal pair for the SGLE noise at point idx (Box-Muller on two
 * counter-based uniforms; the reference uses the polar method on
 * RANDOM_NUMBER, so parity with it is statistical). */
static inline void sgle_normals(uint64_t seed, uint64_t ctr, uint64_t idx, double* v1, double* v2) {
  const double u1 = 1.0 - frc_uniform(seed, ctr, 2 * idx), u2 = frc_uniform(seed, ctr, 2 * idx + 1);
  const double r = sqrt(-2.0 * log(u1));
  *v1 = r * cos(2.0 * PI * u2);
  *v2 = r * sin(2.0 * PI * u2);
}

/* ---------------------------------------------------------------- grid -- */

/* nshell = int(1.414*Nx/2.0d0) + 1 (mod_grid.f90:77): 1.414 is a default
 * (single precision) literal, so the product 1.414*Nx is a REAL*4. */
int32_t vko_nshell(int32_t nx) {
  float prod = 1.414f * (float)nx;
  return (int32_t)((double)prod / 2.0) + 1;
}
/* kalias = REAL(Nx)/3 (mod_grid.f90:92). */
double vko_kalias(int32_t nx) { return (double)nx / 3.0; }
/* kwn(i) = (i-1) - N*(i/(N/2+1)) (pspectral.f90:20-29), i 1-based. */
int32_t vko_kwn(int32_t n, int32_t i) { return (i - 1) - n * (i / (n / 2 + 1)); }

/* cos/sin(2*pi*k/n) with octant reduction, so the tables are accurate to
 * the last bit libm gives for an angle in [0, pi/4]. */
static void cis2pi(long k, long n, double* c, double* s) {
  k %= n;
  if (k < 0) k += n;
  int negs = 0, negc = 0, swp = 0;
  if (2 * k > n) { k = n - k; negs = 1; }
  if ((n % 2 == 0) && 4 * k > n) { k = n / 2 - k; negc = 1; }
  if ((n % 4 == 0) && 8 * k > n) { k = n / 4 - k; swp = 1; }
  double th = 2.0 * PI * (double)k / (double)n;
  double cc = cos(th), ss = sin(th);
  if (swp) { double t = cc; cc = ss; ss = t; }
  if (negc) cc = -cc;
  if (negs) ss = -ss;
  *c = cc;
  *s = ss;
}

static void make_fft_tables(int n, cx** tw, int** br) {
  *tw = (cx*)malloc(sizeof(cx) * (size_t)(n > 1 ? n / 2 : 1));
  *br = (int*)malloc(sizeof(int) * (size_t)n);
  for (int k = 0; k < n / 2; ++k) {
    double c, s;
    cis2pi(k, n, &c, &s);
    (*tw)[k].re = c;
    (*tw)[k].im = -s; /* e^{-2 pi i k/n}: FFTW_FORWARD sign */
  }
  int lg = 0;
  while ((1 << lg) < n) ++lg;
  for (int i = 0; i < n; ++i) {
    int r = 0;
    for (int b = 0; b < lg; ++b)
      if (i & (1 << b)) r |= 1 << (lg - 1 - b);
    (*br)[i] = r;
  }
}

/* In-place radix-2 DIT FFT of length n, sign -1 (forward) or +1 (backward),
 * unnormalised like FFTW. */
static void fft1d(cx* a, int n, const cx* tw, const int* br, int sign) {
  for (int i = 0; i < n; ++i) {
    int j = br[i];
    if (i < j) { cx t = a[i]; a[i] = a[j]; a[j] = t; }
  }
  for (int len = 2; len <= n; len <<= 1) {
    int half = len >> 1, step = n / len;
    for (int i = 0; i < n; i += len) {
      for (int k = 0; k < half; ++k) {
        cx w = tw[k * step];
        if (sign > 0) w.im = -w.im;
        cx u = a[i + k];
        cx v = cmul(a[i + k + half], w);
        a[i + k] = cadd(u, v);
        a[i + k + half] = csub(u, v);
      }
    }
  }
}

/* Forward: phys[y][x] -> four[kx][ky] (FFTW_MPI_TRANSPOSED_OUT layout). */
static void fft_fwd(vko_state* s, const cx* in, cx* out) {
  const int nx = s->nx, ny = s->ny;
  cx* w = s->work;
#pragma omp parallel for schedule(static)
  for (int y = 0; y < ny; ++y) {
    memcpy(w + (size_t)y * nx, in + (size_t)y * nx, sizeof(cx) * nx);
    fft1d(w + (size_t)y * nx, nx, s->twx, s->brx, -1);
  }
#pragma omp parallel for schedule(static)
  for (int kx = 0; kx < nx; ++kx) {
    cx* o = out + (size_t)kx * ny;
    for (int y = 0; y < ny; ++y) o[y] = w[(size_t)y * nx + kx];
    fft1d(o, ny, s->twy, s->bry, -1);
  }
}

/* Backward: four[kx][ky] -> phys[y][x], then the separate fftwscale pass
 * `psi = fftwscale*psi` (mod_fft.f90:485-486 and siblings). */
static void fft_inv(vko_state* s, const cx* in, cx* out) {
  const int nx = s->nx, ny = s->ny;
  cx* w = s->work;
#pragma omp parallel for schedule(static)
  for (int kx = 0; kx < nx; ++kx) {
    memcpy(w + (size_t)kx * ny, in + (size_t)kx * ny, sizeof(cx) * ny);
    fft1d(w + (size_t)kx * ny, ny, s->twy, s->bry, +1);
  }
#pragma omp parallel for schedule(static)
  for (int y = 0; y < ny; ++y) {
    cx* o = out + (size_t)y * nx;
    for (int kx = 0; kx < nx; ++kx) o[kx] = w[(size_t)kx * ny + y];
    fft1d(o, nx, s->twx, s->brx, +1);
    for (int x = 0; x < nx; ++x) o[x] = crmul(s->fftwscale, o[x]);
  }
}

void vko_fft_forward(vko_state* s, const double* phys, double* four) { fft_fwd(s, (const cx*)phys, (cx*)four); }
void vko_fft_inverse(vko_state* s, const double* four, double* phys) { fft_inv(s, (const cx*)four, (cx*)phys); }

/* -------------------------------------------------------------- set-up -- */

static cx* calloc_cx(size_t n) { return (cx*)calloc(n, sizeof(cx)); }

vko_state* vko_create(const vko_params* p) {
  vko_state* s = (vko_state*)calloc(1, sizeof(vko_state));
  s->p = *p;
  s->nx = p->nx;
  s->ny = p->ny;
  s->n2 = (size_t)p->nx * (size_t)p->ny;
  /* set_grid (mod_grid.f90:63-101) */
  s->lx = 2.0 * PI;
  s->ly = 2.0 * PI;
  s->dx = s->lx / s->nx;
  s->dy = s->ly / s->ny;
  s->dvol = s->dx * s->dy;
  s->kalias = vko_kalias(s->nx);
  s->ka2 = s->kalias * s->kalias;
  s->nshell = vko_nshell(s->nx);
  /* fftwscale = one/(REAL(Nx)*REAL(Ny)) (mod_fft.f90:414) */
  s->fftwscale = 1.0 / ((double)s->nx * (double)s->ny);
  s->nparticle = s->lx * s->ly; /* driver.f90:362 */
  s->kwn1 = (int*)malloc(sizeof(int) * s->nx);
  s->kwn2 = (int*)malloc(sizeof(int) * s->ny);
  for (int i = 1; i <= s->nx; ++i) s->kwn1[i - 1] = vko_kwn(s->nx, i);
  for (int i = 1; i <= s->ny; ++i) s->kwn2[i - 1] = vko_kwn(s->ny, i);
  size_t n2 = s->n2;
  s->psi = calloc_cx(n2);
  s->kpsi = calloc_cx(n2);
  s->nlin = calloc_cx(n2);
  s->cmpxtmp = calloc_cx(n2);
  s->str1 = calloc_cx(n2);
  s->str2 = calloc_cx(n2);
  s->tmp1 = calloc_cx(n2);
  s->tmp2 = calloc_cx(n2);
  s->tmp3 = calloc_cx(n2);
  s->work = calloc_cx(n2);
  make_fft_tables(s->nx, &s->twx, &s->brx);
  make_fft_tables(s->ny, &s->twy, &s->bry);
  s->np = p->n_particles;
  if (s->np > 0) {
    int np = s->np;
    s->vobj = calloc_cx(n2);
    s->trans_vobj = calloc_cx(n2);
    s->pos = (double*)calloc((size_t)2 * np, sizeof(double));
    s->vel = (double*)calloc((size_t)2 * np, sizeof(double));
    s->frc = (double*)calloc((size_t)2 * np, sizeof(double));
    s->f0ext = (double*)calloc((size_t)2 * np, sizeof(double));
    s->tpos = (double*)calloc((size_t)2 * np, sizeof(double));
    s->tvel = (double*)calloc((size_t)2 * np, sizeof(double));
    s->shortrange = (double*)calloc((size_t)2 * np, sizeof(double));
    for (int k = 0; k < 4; ++k) {
      s->ku[k] = (double*)calloc((size_t)2 * np, sizeof(double));
      s->kq[k] = (double*)calloc((size_t)2 * np, sizeof(double));
    }
  }
  return s;
}

void vko_destroy(vko_state* s) {
  if (!s) return;
  free(s->kwn1); free(s->kwn2);
  free(s->psi); free(s->kpsi); free(s->nlin); free(s->cmpxtmp);
  free(s->str1); free(s->str2); free(s->tmp1); free(s->tmp2); free(s->tmp3);
  free(s->work); free(s->twx); free(s->twy); free(s->brx); free(s->bry);
  free(s->vobj); free(s->trans_vobj);
  free(s->pos); free(s->vel); free(s->frc); free(s->f0ext); free(s->tpos); free(s->tvel);
  free(s->shortrange);
  for (int k = 0; k < 4; ++k) { free(s->ku[k]); free(s->kq[k]); }
  free(s);
}

void vko_set_threads(int32_t n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

/* ---- seeded vortex initial state (new component) ---------------------- */

static uint64_t ic_splitmix(uint64_t* state) {
  uint64_t z = (*state += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

static double ic_unit(uint64_t* state) { return (double)(ic_splitmix(state) >> 11) / 9007199254740992.0; }

/* periodic difference on [0, 2pi) folded into (-pi, pi] */
static double ic_fold(double d) {
  const double pi = 3.14159265358979323846264338327950288;
  d = fmod(d, 2.0 * pi);
  if (d > pi) d -= 2.0 * pi;
  if (d <= -pi) d += 2.0 * pi;
  return d;
}

int32_t vko_ic_vortices(int32_t nx, int32_t ny, int32_t n_vort, uint64_t seed, double xi0, double min_sep,
                        double* psi, double* pos) {
  const double pi = 3.14159265358979323846264338327950288;
  if (nx <= 0 || ny <= 0 || n_vort < 0 || (n_vort & 1) || !(xi0 > 0.0) || !psi) return -1;
  double* vx = (double*)malloc(sizeof(double) * (n_vort + 1));
  double* vy = (double*)malloc(sizeof(double) * (n_vort + 1));
  uint64_t st = seed;
  for (int j = 0; j < n_vort; ++j) {
    long tries = 0;
    for (;;) {
      const double x = 2.0 * pi * ic_unit(&st), y = 2.0 * pi * ic_unit(&st);
      int far = 1;
      for (int i = 0; i < j && far; ++i) {
        const double ex = ic_fold(x - vx[i]), ey = ic_fold(y - vy[i]);
        far = sqrt(ex * ex + ey * ey) >= min_sep;
      }
      if (far) { vx[j] = x; vy[j] = y; break; }
      if (++tries > 1000000) { free(vx); free(vy); return -1; }
    }
  }
  /* sum of q_j x_j: the linear phase -y S/(2 pi) cancels the theta
     function's quasi-periodicity along y */
  double S = 0.0;
  for (int j = 0; j < n_vort; ++j) S += (j < n_vort / 2 ? 1.0 : -1.0) * vx[j];
  double q2[10];
  for (int m = 1; m <= 9; ++m) q2[m] = exp(-2.0 * pi * m);  /* q^{2m}, q = e^{-pi} */
#pragma omp parallel for schedule(static)
  for (int y = 0; y < ny; ++y) {
    const double yy = 2.0 * pi * y / ny;
    for (int x = 0; x < nx; ++x) {
      const double xx = 2.0 * pi * x / nx;
      double amp = 1.0;
      cx ph = {1.0, 0.0};
      for (int j = 0; j < n_vort; ++j) {
        const double ddx = xx - vx[j], ddy = yy - vy[j];
        const double fx = ic_fold(ddx), fy = ic_fold(ddy);
        const double r = sqrt(fx * fx + fy * fy) / xi0;
        amp *= r / sqrt(2.0 + r * r);
        /* theta_1(v | q), v = (ddx + i ddy)/2, up to a positive factor:
           sin v * prod_m (1 - q^2m e^{2iv}) (1 - q^2m e^{-2iv}) */
        cx th = {sin(0.5 * ddx) * cosh(0.5 * ddy), cos(0.5 * ddx) * sinh(0.5 * ddy)};
        const double c = cos(ddx), sn = sin(ddx), dn = exp(-ddy), up = exp(ddy);
        for (int m = 1; m <= 9; ++m) {
          const cx f1 = {1.0 - q2[m] * dn * c, -q2[m] * dn * sn};
          const cx f2 = {1.0 - q2[m] * up * c, q2[m] * up * sn};
          th = cmul(th, cmul(f1, f2));
        }
        const double mod = hypot(th.re, th.im);
        cx u = {1.0, 0.0};
        if (mod > 0.0) { u.re = th.re / mod; u.im = th.im / mod; }
        if (j >= n_vort / 2) u.im = -u.im;
        ph = cmul(ph, u);
      }
      const cx lin = {cos(-yy * S / (2.0 * pi)), sin(-yy * S / (2.0 * pi))};
      ph = cmul(ph, lin);
      const double mod = hypot(ph.re, ph.im);
      psi[2 * ((size_t)y * nx + x)] = amp * ph.re / mod;
      psi[2 * ((size_t)y * nx + x) + 1] = amp * ph.im / mod;
    }
  }
  if (pos)
    for (int j = 0; j < n_vort; ++j) { pos[2 * j] = vx[j]; pos[2 * j + 1] = vy[j]; }
  free(vx);
  free(vy);
  return 0;
}

static inline int masked(const vko_state* s, int k1, int k2) {
  int ksqr = k1 * k1 + k2 * k2;
  return (double)ksqr >= s->ka2; /* IF (ksqr .GE. kalias**2) */
}

/* ----------------------------------------------------------- particles -- */

/* particle_potential (gpe_particle.f90:3-90): origin-centred Gaussian on
 * the sin chart, forward FFT, dealiased -> cgp_four_vobj. */
static void particle_potential(vko_state* s) {
  const int nx = s->nx, ny = s->ny;
  double c1 = 2 * PI / (2.0 * s->lx);
  double c2 = 2 * PI / (2.0 * s->ly);
  double d = s->p.ppot_d, v0 = s->p.ppot_v0;
  for (int y = 0; y < ny; ++y) {
    double yy = y * s->dy;
    for (int x = 0; x < nx; ++x) {
      double xx = x * s->dx;
      double sx = sin(c1 * xx), sy = sin(c2 * yy);
      double xprd = (1.0 / c1) * (sx + (1.0 / 6.0) * (sx * sx * sx) + (1.0 / 40.0) * (sx * sx * sx * sx * sx));
      double yprd = (1.0 / c2) * (sy + (1.0 / 6.0) * (sy * sy * sy) + (1.0 / 40.0) * (sy * sy * sy * sy * sy));
      double rprd = sqrt(xprd * xprd + yprd * yprd);
      double v = v0 * exp(-(rprd * rprd) / (2.0 * (d * d)));
      s->cmpxtmp[(size_t)y * nx + x].re = v;
      s->cmpxtmp[(size_t)y * nx + x].im = 0.0;
    }
  }
  fft_fwd(s, s->cmpxtmp, s->cmpxtmp);
  for (int kx = 0; kx < nx; ++kx)
    for (int ky = 0; ky < ny; ++ky) {
      size_t i = (size_t)kx * ny + ky;
      if (masked(s, s->kwn1[kx], s->kwn2[ky])) s->cmpxtmp[i].re = s->cmpxtmp[i].im = 0.0;
      s->vobj[i] = s->cmpxtmp[i];
      s->cmpxtmp[i].re = s->cmpxtmp[i].im = 0.0;
    }
}

/* exp(-zi*theta) as gfortran evaluates EXP of a purely imaginary argument. */
static inline cx expmi(double th) { cx r = {cos(th), -sin(th)}; return r; }

static inline double ipow(double x, int n) {
  double r = 1.0;
  for (int i = 0; i < n; ++i) r *= x;
  return r;
}

/* shortrange_repulsion (gpe_particle.f90:378-427). */
static void shortrange_repulsion(vko_state* s) {
  s->gpdeltaE = (double)0.062f; /* default-real literal */
  s->gpr0obj = 4.0 * s->p.xi;
  double r0obj12 = ipow(s->gpr0obj, 12);
  double rf = 384.0 * s->gpdeltaE * ipow(PI, 12) * r0obj12 / ipow(s->lx, 12);
  int np = s->np;
  for (int i = 0; i < 2 * np; ++i) s->shortrange[i] = 0.0;
  for (int i1 = 0; i1 < np; ++i1)
    for (int i2 = 0; i2 < np; ++i2) {
      double x = s->pos[2 * i1] - s->pos[2 * i2];
      double y = s->pos[2 * i1 + 1] - s->pos[2 * i2 + 1];
      double den = ipow(-3 + cos(x) + cos(y), 7);
      double f1 = -rf * sin(x) / den;
      double f2 = -rf * sin(y) / den; /* the y factor also uses L_x (:401) */
      if (i1 == i2) f1 = f2 = 0.0;
      s->shortrange[2 * i1] += f1;
      s->shortrange[2 * i1 + 1] += f2;
    }
  if (np == 1) s->shortrange[0] = s->shortrange[1] = 0.0;
}

/* translate_particle_potential (gpe_particle.f90:186-376). */
static void translate_particle_potential(vko_state* s, int particle_trans) {
  const int nx = s->nx, ny = s->ny;
  if (particle_trans >= 1 && particle_trans <= s->np) {
    int ip = particle_trans - 1;
    for (int kx = 0; kx < nx; ++kx)
      for (int ky = 0; ky < ny; ++ky) {
        double kxr = s->kwn1[kx], kyr = s->kwn2[ky];
        cx e = expmi(kxr * s->pos[2 * ip] + kyr * s->pos[2 * ip + 1]);
        size_t i = (size_t)kx * ny + ky;
        s->trans_vobj[i] = cmul(e, s->vobj[i]);
      }
    fft_inv(s, s->trans_vobj, s->trans_vobj);
    shortrange_repulsion(s);
    for (size_t i = 0; i < s->n2; ++i) {
      double a = cabs_f(s->psi[i]);
      s->cmpxtmp[i].re = a * a;
      s->cmpxtmp[i].im = 0.0;
    }
    fft_fwd(s, s->cmpxtmp, s->cmpxtmp);
    for (int kx = 0; kx < nx; ++kx)
      for (int ky = 0; ky < ny; ++ky) {
        size_t i = (size_t)kx * ny + ky;
        /* intended mask (the reference's ksqr is uninitialised here, :275) */
        if (masked(s, s->kwn1[kx], s->kwn2[ky])) s->cmpxtmp[i].re = s->cmpxtmp[i].im = 0.0;
        cx ikx = {0.0, (double)s->kwn1[kx]}, iky = {0.0, (double)s->kwn2[ky]};
        s->tmp1[i] = cmul(ikx, s->cmpxtmp[i]);
        s->tmp2[i] = cmul(iky, s->cmpxtmp[i]);
      }
    fft_inv(s, s->tmp1, s->tmp1);
    fft_inv(s, s->tmp2, s->tmp2);
    double f1 = 0.0, f2 = 0.0;
    double ta = 2.0 * s->p.alpha;
    for (size_t i = 0; i < s->n2; ++i) {
      f1 = f1 - cmul(crmul(ta, s->tmp1[i]), s->trans_vobj[i]).re;
      f2 = f2 - cmul(crmul(ta, s->tmp2[i]), s->trans_vobj[i]).re;
    }
    f1 *= s->dvol;
    f2 *= s->dvol;
    s->gpfrcpart[0] = f1 + s->shortrange[2 * ip] + s->f0ext[2 * ip];
    s->gpfrcpart[1] = f2 + s->shortrange[2 * ip + 1] + s->f0ext[2 * ip + 1];
  }
  if (particle_trans == 0) {
    for (int kx = 0; kx < nx; ++kx)
      for (int ky = 0; ky < ny; ++ky) {
        double kxr = s->kwn1[kx], kyr = s->kwn2[ky];
        cx sum = {0.0, 0.0};
        for (int ip = 0; ip < s->np; ++ip) sum = cadd(sum, expmi(kxr * s->pos[2 * ip] + kyr * s->pos[2 * ip + 1]));
        size_t i = (size_t)kx * ny + ky;
        s->trans_vobj[i] = cmul(sum, s->vobj[i]);
      }
    fft_inv(s, s->trans_vobj, s->trans_vobj);
  }
}

/* gp_particle_motion_rk4 (gpe_particle.f90:429-531). */
static void particle_motion_rk4(vko_state* s, int stage) {
  int np = s->np;
  double dt = s->p.dt, m = s->p.gp_mass_part;
  if (stage == 1)
    for (int i = 0; i < 2 * np; ++i) { s->tvel[i] = s->vel[i]; s->tpos[i] = s->pos[i]; }
  for (int ip = 0; ip < np; ++ip) {
    translate_particle_potential(s, ip + 1);
    for (int d = 0; d < 2; ++d) {
      int i = 2 * ip + d;
      double ku = dt * s->gpfrcpart[d] / m;
      double kq = dt * s->vel[i];
      s->ku[stage - 1][i] = ku;
      s->kq[stage - 1][i] = kq;
      if (stage == 1 || stage == 2) {
        s->vel[i] = s->tvel[i] + 0.5 * ku;
        s->pos[i] = s->tpos[i] + 0.5 * kq;
      } else if (stage == 3) {
        s->vel[i] = s->tvel[i] + ku;
        s->pos[i] = s->tpos[i] + kq;
      } else {
        s->vel[i] = s->tvel[i] + (1.0 / 6.0) * (s->ku[0][i] + 2.0 * s->ku[1][i] + 2.0 * s->ku[2][i] + s->ku[3][i]);
        s->pos[i] = s->tpos[i] + (1.0 / 6.0) * (s->kq[0][i] + 2.0 * s->kq[1][i] + 2.0 * s->kq[2][i] + s->kq[3][i]);
      }
    }
  }
}

void vko_particles_set(vko_state* s, const double* pos, const double* vel, const double* f0ext) {
  if (s->np <= 0) return;
  memcpy(s->pos, pos, sizeof(double) * 2 * s->np);
  memcpy(s->vel, vel, sizeof(double) * 2 * s->np);
  memcpy(s->f0ext, f0ext, sizeof(double) * 2 * s->np);
  particle_potential(s);
}

void vko_particles_get(const vko_state* s, double* pos, double* vel, double* frc) {
  if (s->np <= 0) return;
  if (pos) memcpy(pos, s->pos, sizeof(double) * 2 * s->np);
  if (vel) memcpy(vel, s->vel, sizeof(double) * 2 * s->np);
  if (frc) memcpy(frc, s->frc, sizeof(double) * 2 * s->np);
}

void vko_particle_forces(vko_state* s, double* frc) {
  for (int ip = 0; ip < s->np; ++ip) {
    translate_particle_potential(s, ip + 1);
    s->frc[2 * ip] = s->gpfrcpart[0];
    s->frc[2 * ip + 1] = s->gpfrcpart[1];
  }
  if (frc) memcpy(frc, s->frc, sizeof(double) * 2 * s->np);
}

/* ---------------------------------------------------------- GPE state -- */

/* restart_from_argle_data (initial_config.f90:630-771, 1-rank branch
 * :727-741): psi <- file, kpsi <- F[psi].  Then ic_OTOC_gpe
 * (initial_config.f90:295-368) when -DGPOTOC is on. */
void vko_set_psi(vko_state* s, const double* psi_phys, int32_t otoc, double k_otoc, double eps_otoc) {
  memcpy(s->psi, psi_phys, sizeof(cx) * s->n2);
  fft_fwd(s, s->psi, s->kpsi);
  if (otoc) {
    const int nx = s->nx, ny = s->ny;
    for (int kx = 0; kx < nx; ++kx)
      for (int ky = 0; ky < ny; ++ky) {
        double kxr = s->kwn1[kx], kyr = s->kwn2[ky];
        double rk = sqrt(kxr * kxr + kyr * kyr);
        int mshl = (int)lround(rk); /* nint */
        size_t i = (size_t)kx * ny + ky;
        if ((double)mshl == k_otoc) s->kpsi[i] = crmul(1.0 + eps_otoc, s->kpsi[i]);
        if (masked(s, s->kwn1[kx], s->kwn2[ky])) s->kpsi[i].re = s->kpsi[i].im = 0.0;
      }
    fft_inv(s, s->kpsi, s->psi);
  }
}

void vko_get_psi(const vko_state* s, double* out) { memcpy(out, s->psi, sizeof(cx) * s->n2); }
void vko_get_kpsi(const vko_state* s, double* out) { memcpy(out, s->kpsi, sizeof(cx) * s->n2); }
void vko_set_kpsi(vko_state* s, const double* kpsi) { memcpy(s->kpsi, kpsi, sizeof(cx) * s->n2); }

/* gpe_rhs (gpe.f90:498-671): result in s->nlin (Fourier view). */
static void gpe_rhs(vko_state* s) {
  const int nx = s->nx, ny = s->ny;
  const double alpha = s->p.alpha, g = s->p.gstrength, om = s->p.omega_chem;
  /* prefacrhs = (one-zi*disp_factor)/zi  (:529) */
  cx prefac = {-s->p.disp_factor, -1.0};
  if (s->np > 0) translate_particle_potential(s, 0); /* :540-543 */
  for (size_t i = 0; i < s->n2; ++i) { /* :546-550 */
    double a = cabs_f(s->psi[i]);
    s->nlin[i].re = a * a;
    s->nlin[i].im = 0.0;
  }
  fft_fwd(s, s->nlin, s->nlin); /* :553 */
#pragma omp parallel for schedule(static)
  for (int kx = 0; kx < nx; ++kx) { /* :557-576 */
    double kxr = s->kwn1[kx];
    for (int ky = 0; ky < ny; ++ky) {
      double kyr = s->kwn2[ky];
      double kr2 = kxr * kxr + kyr * kyr;
      size_t i = (size_t)kx * ny + ky;
      s->tmp1[i] = crmul(alpha * kr2 - om, s->kpsi[i]);
      if (masked(s, s->kwn1[kx], s->kwn2[ky])) s->nlin[i].re = s->nlin[i].im = 0.0;
    }
  }
  fft_inv(s, s->nlin, s->nlin); /* :579 */
#pragma omp parallel for schedule(static)
  for (size_t i = 0; i < s->n2; ++i) { /* :583-594 */
    cx t = cmul(crmul(g, s->nlin[i]), s->psi[i]);
    if (s->np > 0) t = cadd(t, cmul(s->trans_vobj[i], s->psi[i]));
    s->nlin[i] = t;
  }
  fft_fwd(s, s->nlin, s->nlin); /* :607 */
#pragma omp parallel for schedule(static)
  for (int kx = 0; kx < nx; ++kx) { /* :609-669 */
    for (int ky = 0; ky < ny; ++ky) {
      size_t i = (size_t)kx * ny + ky;
      s->nlin[i] = cmul(prefac, cadd(s->tmp1[i], s->nlin[i]));
      if (s->frcdisp) { /* -DGPE_FRCDISP, :623-658 */
        const int k1 = s->kwn1[kx], k2 = s->kwn2[ky];
        const int ksqr = k1 * k1 + k2 * k2;
        const double kr2 = (double)k1 * k1 + (double)k2 * k2;
        const double x2 = kr2 * kr2, x4 = x2 * x2, x8 = x4 * x4; /* kradius2**8 */
        if (ksqr != 0) s->nlin[i] = csub(s->nlin[i], crmul(s->vishypo * (1.0 / x8), s->kpsi[i]));
        s->nlin[i] = csub(s->nlin[i], crmul(s->vishype * x8, s->kpsi[i]));
        if ((double)ksqr >= s->kf1 * s->kf1 && (double)ksqr <= s->kf2 * s->kf2) {
          const double ran = 2.0 * PI * frc_uniform(s->seed, s->ctr, i);
          s->nlin[i].re += s->famp * cos(ran);
          s->nlin[i].im += s->famp * sin(ran);
        }
      }
      if (masked(s, s->kwn1[kx], s->kwn2[ky])) s->nlin[i].re = s->nlin[i].im = 0.0;
    }
  }
  if (s->frcdisp) ++s->ctr;
}

void vko_set_frcdisp(vko_state* s, int32_t on, double vishypo, double vishype, double famp, double kf1,
                     double kf2, uint64_t seed) {
  s->frcdisp = on;
  s->vishypo = vishypo;
  s->vishype = vishype;
  s->famp = famp;
  s->kf1 = kf1;
  s->kf2 = kf2;
  s->seed = seed;
  s->ctr = 0;
}

/* One RK4 stage update (gpe.f90:366-387, 401-421, 435-455, 469-489). */
static void rk4_update(vko_state* s, int stage) {
  const int nx = s->nx, ny = s->ny;
  const double dt = s->p.dt;
  const double oney6 = 1.0 / 6.0, half = 0.5, two = 2.0;
  double c2 = (stage == 1 || stage == 4) ? dt * oney6 : dt * oney6 * two;
  double c1 = (stage == 3) ? dt : dt * half;
#pragma omp parallel for schedule(static)
  for (int kx = 0; kx < nx; ++kx)
    for (int ky = 0; ky < ny; ++ky) {
      size_t i = (size_t)kx * ny + ky;
      s->str2[i] = cadd(s->str2[i], crmul(c2, s->nlin[i]));
      if (stage < 4)
        s->kpsi[i] = cadd(s->str1[i], crmul(c1, s->nlin[i]));
      else
        s->kpsi[i] = cadd(s->str1[i], s->str2[i]);
      if (masked(s, s->kwn1[kx], s->kwn2[ky])) s->kpsi[i].re = s->kpsi[i].im = 0.0;
    }
}

/* gpe_rk4 (gpe.f90:310-494). */
static void gpe_rk4_step(vko_state* s) {
  const int nx = s->nx, ny = s->ny;
  for (int kx = 0; kx < nx; ++kx) /* :338-355 */
    for (int ky = 0; ky < ny; ++ky) {
      size_t i = (size_t)kx * ny + ky;
      if (masked(s, s->kwn1[kx], s->kwn2[ky])) s->kpsi[i].re = s->kpsi[i].im = 0.0;
      s->str1[i] = s->kpsi[i];
      s->str2[i].re = s->str2[i].im = 0.0;
    }
  for (int stage = 1; stage <= 4; ++stage) {
    gpe_rhs(s);
    if (s->np > 0) particle_motion_rk4(s, stage);
    rk4_update(s, stage);
    fft_inv(s, s->kpsi, s->psi);
  }
}

void vko_gpe_rk4(vko_state* s, int32_t nsteps) {
  for (int i = 0; i < nsteps; ++i) gpe_rk4_step(s);
}

/* ARGLE (gpe.f90:5-224), non-SGLE branch, plus the new residual and the
 * optional renormalisation (neither exists in the reference). */
static double argle_step(vko_state* s) {
  const int nx = s->nx, ny = s->ny;
  const double alpha = s->p.alpha, g = s->p.gstrength, dt = s->p.dt;
  fft_inv(s, s->kpsi, s->psi); /* :42 */
  if (s->sgle) {
    /* noise (:149-165) and the ad hoc chemical potential (:189, :226-264);
     * the norm uses psi of this step, so computing it first changes nothing */
    const double f = (1.0 / sqrt(s->dvol)) * s->noisesigma;
    double norm = 0.0;
    for (size_t i = 0; i < s->n2; ++i) {
      double v1, v2;
      sgle_normals(s->seed, s->ctr, i, &v1, &v2);
      s->cmpxtmp[i].re = v1 * f;
      s->cmpxtmp[i].im = v2 * f;
      const double a = cabs_f(s->psi[i]);
      norm = norm + a * a;
    }
    norm = norm * s->dvol;
    s->p.omega_chem = s->p.omega_chem - dt * (s->nuN / (s->lx * s->ly)) * (norm - s->nparticle);
    fft_fwd(s, s->cmpxtmp, s->cmpxtmp); /* :192 */
    ++s->ctr;
  }
  const double om = s->p.omega_chem;
  if (s->np > 0) translate_particle_potential(s, 0); /* :50-53 */
  if (s->flow) { /* :78-81, 93-96: gradients of psi in physical space */
    for (int kx = 0; kx < nx; ++kx)
      for (int ky = 0; ky < ny; ++ky) {
        size_t i = (size_t)kx * ny + ky;
        cx ikx = {0.0, (double)s->kwn1[kx]}, iky = {0.0, (double)s->kwn2[ky]};
        s->tmp1[i] = cmul(ikx, s->kpsi[i]);
        s->tmp2[i] = cmul(iky, s->kpsi[i]);
      }
    fft_inv(s, s->tmp1, s->tmp1);
    fft_inv(s, s->tmp2, s->tmp2);
  }
  for (size_t i = 0; i < s->n2; ++i) { /* :56-60 */
    double a = cabs_f(s->psi[i]);
    s->nlin[i].re = a * a;
    s->nlin[i].im = 0.0;
  }
  fft_fwd(s, s->nlin, s->nlin); /* :63 */
  for (int kx = 0; kx < nx; ++kx) /* :67-89 */
    for (int ky = 0; ky < ny; ++ky) {
      size_t i = (size_t)kx * ny + ky;
      if (masked(s, s->kwn1[kx], s->kwn2[ky])) s->nlin[i].re = s->nlin[i].im = 0.0;
    }
  fft_inv(s, s->nlin, s->nlin); /* :98 */
#pragma omp parallel for schedule(static)
  for (size_t i = 0; i < s->n2; ++i) { /* :101-112 */
    cx t = cmul(crmul(-g, s->nlin[i]), s->psi[i]);
    if (s->np > 0) t = cadd(t, cmul(crmul(-1.0, s->trans_vobj[i]), s->psi[i]));
    if (s->flow == 1) { /* :115-131, x = (i1-1) dx, y = (i2-1) dy */
      const double x = (double)(i % (size_t)nx) * s->dx, y = (double)(i / (size_t)nx) * s->dy;
      const double uadx = sin(x) * cos(y), uady = -cos(x) * sin(y);
      cx v = cadd(crmul(uadx, s->tmp1[i]), crmul(uady, s->tmp2[i]));
      cx miv = {v.im, -v.re}; /* -zi*(uadx*aa1+uady*aa2) */
      t = cadd(t, miv);
      t = csub(t, crmul((0.5 * 0.5) * (1.0 / alpha) * (uadx * uadx + uady * uady), s->psi[i]));
    } else if (s->flow == 2) { /* :135-145 */
      cx v = cadd(crmul(s->vnx, s->tmp1[i]), crmul(s->vny, s->tmp2[i]));
      cx miv = {v.im, -v.re};
      t = cadd(t, miv);
    }
    s->nlin[i] = t;
  }
  fft_fwd(s, s->nlin, s->nlin); /* :170 */
  double dsum = 0.0, osum = 0.0, nsum = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : dsum, osum, nsum)
  for (int kx = 0; kx < nx; ++kx) { /* :182-222 */
    double kxr = s->kwn1[kx];
    for (int ky = 0; ky < ny; ++ky) {
      double kyr = s->kwn2[ky];
      double kr2 = kxr * kxr + kyr * kyr;
      size_t i = (size_t)kx * ny + ky;
      cx old = s->kpsi[i];
      cx t1 = cadd(s->nlin[i], crmul(om, old));
      double t2 = 1.0 + alpha * kr2 * dt;
      cx nw = cadd(old, crmul(dt, t1));
      if (s->sgle) { /* :199-212 */
        cx noise = crmul(sqrt(dt), s->cmpxtmp[i]);
        if (masked(s, s->kwn1[kx], s->kwn2[ky])) noise.re = noise.im = 0.0;
        nw = cadd(nw, noise);
      }
      nw.re /= t2;
      nw.im /= t2;
      if (s->sgle && s->selftrunc && kr2 > s->ktrunc * s->ktrunc) nw.re = nw.im = 0.0; /* :213-217 */
      s->kpsi[i] = nw;
      cx dd = csub(nw, old);
      dsum += dd.re * dd.re + dd.im * dd.im;
      osum += old.re * old.re + old.im * old.im;
      nsum += nw.re * nw.re + nw.im * nw.im;
    }
  }
  if (s->p.renorm) {
    /* norm of psi = F^-1 kpsi by Parseval: dvol/(nx ny) * sum |kpsi|^2 */
    double norm = s->dvol * s->fftwscale * nsum;
    double f = sqrt(s->nparticle / norm);
    for (size_t i = 0; i < s->n2; ++i) s->kpsi[i] = crmul(f, s->kpsi[i]);
  }
  return sqrt(dsum) / (dt * sqrt(osum));
}

void vko_set_sgle(vko_state* s, int32_t on, double oneybeta, double nuN, double chempot0, int32_t selftrunc,
                  double ktrunc, uint64_t seed) {
  s->sgle = on;
  s->noisesigma = sqrt((1.0 / (2.0 * s->p.alpha)) * oneybeta); /* driver.f90:376 */
  s->nuN = nuN;
  s->selftrunc = selftrunc;
  s->ktrunc = ktrunc;
  s->seed = seed;
  s->ctr = 0;
  if (on) s->p.omega_chem = chempot0; /* driver.f90:372 */
}
double vko_chempot(const vko_state* s) { return s->p.omega_chem; }

void vko_set_argle_flow(vko_state* s, int32_t mode, double vnx, double vny) {
  s->flow = mode;
  s->vnx = vnx;
  s->vny = vny;
}

void vko_argle(vko_state* s, int32_t nsteps, double* residual) {
  double r = 0.0;
  for (int i = 0; i < nsteps; ++i) r = argle_step(s);
  if (residual) *residual = r;
}

/* -------------------------------------------------------- diagnostics -- */

/* diagnostics_gpe (diagnostics.f90:4-571) for one rank. */
void vko_diagnostics(vko_state* s, double* scalars, double* spec) {
  const int nx = s->nx, ny = s->ny, ns = s->nshell;
  const double alpha = s->p.alpha, g = s->p.gstrength, om = s->p.omega_chem;
  const double half = 0.5, two = 2.0;
  const double area = s->lx * s->ly;
  for (int kx = 0; kx < nx; ++kx) /* :55-67 */
    for (int ky = 0; ky < ny; ++ky) {
      size_t i = (size_t)kx * ny + ky;
      cx ikx = {0.0, (double)s->kwn1[kx]}, iky = {0.0, (double)s->kwn2[ky]};
      s->tmp1[i] = cmul(ikx, s->kpsi[i]);
      s->tmp2[i] = cmul(iky, s->kpsi[i]);
    }
  fft_inv(s, s->tmp1, s->tmp1); /* :70-71 */
  fft_inv(s, s->tmp2, s->tmp2);
  if (s->np > 0) translate_particle_potential(s, 0); /* :73-77 */
  double momx = 0.0, momy = 0.0;
  for (size_t i = 0; i < s->n2; ++i) { /* :84-103 */
    cx aa1 = cmul(cconj(s->psi[i]), s->tmp1[i]);
    cx aa2 = cmul(cconj(s->psi[i]), s->tmp2[i]);
    momx += aa1.im;
    momy += aa2.im;
    double a = cabs_f(s->psi[i]);
    s->nlin[i].re = a * a;
    s->nlin[i].im = 0.0;
  }
  momx = two * alpha * momx * s->dvol / area; /* :105-106 */
  momy = two * alpha * momy * s->dvol / area;
  fft_fwd(s, s->nlin, s->nlin); /* :117 */
  for (int kx = 0; kx < nx; ++kx) /* :126-146 */
    for (int ky = 0; ky < ny; ++ky) {
      size_t i = (size_t)kx * ny + ky;
      if (masked(s, s->kwn1[kx], s->kwn2[ky])) s->nlin[i].re = s->nlin[i].im = 0.0;
      s->str1[i] = s->nlin[i];
    }
  fft_inv(s, s->nlin, s->nlin); /* :149 */
  double egrad = 0.0, echem = 0.0, eintr = 0.0, eppot = 0.0, norm = 0.0;
  for (size_t i = 0; i < s->n2; ++i) { /* :165-183 */
    double a1 = cabs_f(s->tmp1[i]), a2 = cabs_f(s->tmp2[i]), ap = cabs_f(s->psi[i]);
    egrad = egrad + alpha * (a1 * a1 + a2 * a2);
    echem = echem + om * (ap * ap);
    eintr = eintr + half * g * cabs_f(s->nlin[i]) * (ap * ap);
    if (s->np > 0) eppot = eppot + s->trans_vobj[i].re * s->nlin[i].re;
    norm = norm + ap * ap;
  }
  egrad = two * alpha * egrad * s->dvol / area; /* :187-207 */
  echem = two * alpha * echem * s->dvol / area;
  eintr = two * alpha * eintr * s->dvol / area;
  eppot = two * alpha * eppot * s->dvol / area;
  norm = norm * s->dvol;
  double eobj_kin = 0.0, esrep = 0.0;
  if (s->np > 0) { /* :209-239 */
    double fac = 64.0 * s->gpdeltaE * ipow(PI, 12) * ipow(s->gpr0obj, 12) / ipow(s->lx, 12);
    for (int i1 = 0; i1 < s->np; ++i1) {
      for (int d = 0; d < 2; ++d) eobj_kin += s->vel[2 * i1 + d] * s->vel[2 * i1 + d];
      for (int i2 = 0; i2 < s->np; ++i2) {
        double x = s->pos[2 * i1] - s->pos[2 * i2], y = s->pos[2 * i1 + 1] - s->pos[2 * i2 + 1];
        double erep = fac / ipow(-3 + cos(x) + cos(y), 6);
        if (i1 == i2) erep = 0.0;
        esrep += erep;
      }
    }
    eobj_kin = half * s->p.gp_mass_part * eobj_kin;
    esrep = half * esrep;
    if (s->np == 1) esrep = 0.0;
  }
  double etot = egrad + eintr; /* :244 */
  const double smlnum = (double)1e-30f; /* REAL(GP), PARAMETER:: smlnum = 1e-30 (:43) */
  for (size_t i = 0; i < s->n2; ++i) { /* :265-275 */
    double rholoc = cabs_f(s->psi[i]) + smlnum;
    cx a = cmul(cconj(s->psi[i]), s->tmp1[i]);
    cx b = cmul(cconj(s->psi[i]), s->tmp2[i]);
    s->tmp1[i].re = a.re / rholoc; s->tmp1[i].im = a.im / rholoc;
    s->tmp2[i].re = b.re / rholoc; s->tmp2[i].im = b.im / rholoc;
  }
  for (size_t i = 0; i < s->n2; ++i) { /* :303-317 (hh = one) */
    double hh = 1.0;
    s->cmpxtmp[i].re = hh * s->tmp1[i].re; s->cmpxtmp[i].im = 0.0;
    s->tmp3[i].re = hh * s->tmp2[i].re; s->tmp3[i].im = 0.0;
    double i1 = s->tmp1[i].im, i2 = s->tmp2[i].im;
    s->tmp1[i].re = two * alpha * i1 * hh; s->tmp1[i].im = 0.0;
    s->tmp2[i].re = two * alpha * i2 * hh; s->tmp2[i].im = 0.0;
  }
  fft_fwd(s, s->tmp1, s->tmp1); /* :320-325 */
  fft_fwd(s, s->tmp2, s->tmp2);
  fft_fwd(s, s->cmpxtmp, s->cmpxtmp);
  fft_fwd(s, s->tmp3, s->tmp3);
  double enorm = (1.0 / ((double)nx * (double)ny));
  enorm = enorm * enorm; /* :328 */
  for (int i = 0; i < (ns + 1) * 6; ++i) spec[i] = 0.0;
  for (int kx = 0; kx < nx; ++kx) { /* :332-402 */
    int k1 = s->kwn1[kx];
    double kxr = k1;
    for (int ky = 0; ky < ny; ++ky) {
      int k2 = s->kwn2[ky];
      double kyr = k2;
      size_t i = (size_t)kx * ny + ky;
      double rk2 = kxr * kxr + kyr * kyr;
      double rk = sqrt(rk2);
      int mshl = (int)lround(rk);
      double kr2 = kxr * kxr + kyr * kyr;
      cx aa1 = s->tmp1[i], aa2 = s->tmp2[i];
      cx bb1 = {0.0, 0.0}, bb2 = {0.0, 0.0};
      if (!(k1 == 0 && k2 == 0)) {
        cx m1 = {0.0, -(kxr / kr2)}, m2 = {0.0, -(kyr / kr2)};
        bb1 = cmul(m1, aa1);
        bb2 = cmul(m2, aa2);
      }
      cx bb = cadd(bb1, bb2);
      cx ikx = {0.0, kxr}, iky = {0.0, kyr};
      cx cc1 = cmul(ikx, bb), cc2 = cmul(iky, bb);
      cx dd1 = csub(aa1, cc1), dd2 = csub(aa2, cc2);
      cx ee1 = s->cmpxtmp[i], ee2 = s->tmp3[i];
      cx ff = s->str1[i], gg = s->kpsi[i];
      double x1 = cabs_f(aa1), x2 = cabs_f(aa2);
      double ekint = enorm * (x1 * x1 + x2 * x2);
      x1 = cabs_f(cc1); x2 = cabs_f(cc2);
      double ekinc = enorm * (x1 * x1 + x2 * x2);
      x1 = cabs_f(dd1); x2 = cabs_f(dd2);
      double ekini = enorm * (x1 * x1 + x2 * x2);
      x1 = cabs_f(ee1); x2 = cabs_f(ee2);
      double equnt = enorm * (x1 * x1 + x2 * x2);
      x1 = cabs_f(ff);
      double eint = enorm * (x1 * x1);
      x1 = cabs_f(gg);
      double eocc = enorm * (x1 * x1);
      if (masked(s, k1, k2)) ekint = ekini = ekinc = equnt = eint = eocc = 0.0;
      spec[0 * (ns + 1) + mshl] += ekint * half;
      spec[1 * (ns + 1) + mshl] += ekini * half;
      spec[2 * (ns + 1) + mshl] += ekinc * half;
      spec[3 * (ns + 1) + mshl] += equnt * two * (alpha * alpha);
      spec[4 * (ns + 1) + mshl] += eint * half * g * two * alpha;
      spec[5 * (ns + 1) + mshl] += eocc;
    }
  }
  scalars[0] = momx; scalars[1] = momy; scalars[2] = egrad; scalars[3] = echem;
  scalars[4] = eintr; scalars[5] = etot; scalars[6] = norm; scalars[7] = eppot;
  scalars[8] = eobj_kin; scalars[9] = esrep;
  /* particle forces for the text output (:526-533) */
  if (s->np > 0) vko_particle_forces(s, NULL);
}

/* ------------------------------------------------------ vortex counter -- */

static inline double carg_diff(cx a, cx b) { /* arg(conj(a)*b) in (-pi, pi] */
  cx p = cmul(cconj(a), b);
  return atan2(p.im, p.re);
}

void vko_count_vortices(const vko_state* s, int32_t* n_plus, int32_t* n_minus) {
  const int nx = s->nx, ny = s->ny;
  int np = 0, nm = 0;
  for (int y = 0; y < ny; ++y) {
    int y1 = (y + 1) % ny;
    for (int x = 0; x < nx; ++x) {
      int x1 = (x + 1) % nx;
      cx a = s->psi[(size_t)y * nx + x], b = s->psi[(size_t)y * nx + x1];
      cx c = s->psi[(size_t)y1 * nx + x1], d = s->psi[(size_t)y1 * nx + x];
      double w = carg_diff(a, b) + carg_diff(b, c) + carg_diff(c, d) + carg_diff(d, a);
      long q = lround(w / (2.0 * PI));
      if (q > 0) np += (int)q;
      if (q < 0) nm += (int)(-q);
    }
  }
  *n_plus = np;
  *n_minus = nm;
}
