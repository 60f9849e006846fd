// vk_driver.cpp -- the reference's driver + solve loop over libvk.
//
// Host program replacing `PROGRAM driver` (src/driver.f90) and `solve`
// (src/solve.f90) for one GPU: reads parameter.txt / parameter_gpe.txt from
// the working directory, loads restart/wf/wf<nrst>p1.dat
// (restart_from_argle_data, src/initial_config.f90:630-771) and, with
// particles, restart/part/gp{pos,vel,f0ext}.dat_nrst<nrst>
// (initialize_particles, src/gpe_particle.f90:92-141), then runs the solve
// loop with the reference's output cadence and file layout:
//   data/wf/wf<n>p1.dat                      every fsteps (io_fields)
//   data/energy1.dat_nrst0, norm, mom        every gsteps (diagnostics.f90:242-261)
//   data/energy.dat_nrst0, n0.dat_nrst0      every gsteps (quantglobal_gpe)
//   spectra/spec<n>.dat                      every ssteps (spectrum_gpe)
//   data/gpobj_{pos,vel,frc}_<i>.dat_nrst0, egpobj, momgpobj  (particles)
//   data/gp{pos,vel,f0ext}_ckp.dat_nrst0     every fsteps (gppart_checkpoint)
//   run_info.dat                             wall time
// With --sts NT (the -DGPSTS build), every ststeps (sts_gpe):
//   data/sts_time.dat_nrst0, data/sts1d/kpsi_x0_nrst0.dat, data/sts2d/kpsi_nrst0p1.dat
// and every NT records the Run/CompSTS spectra data/sts1d_kx0_nrst<strst>.dat,
// data/sts2d_nrst<strst>.dat (computed on the GPU).
// Text files use Fortran's E15.6 edit descriptor.  Output points between
// which no file is written are stepped with one vk_gpe_rk4 call.
//
// --frcdisp / --advection / --counterflow / --sgle / --selftrunc select the
// reference's compile-time branches (-DGPE_FRCDISP etc.) with their namelist
// parameters; with --argle --sgle, data/cpot_sgle.dat_nrst0 every fsteps.
// With &fileparam nsplit_orignal > 1 the restart field is regrouped from
// restart/wf/wf<nrst>p1..p<nsplit>.dat.
//
// Usage: vikshobha_gb300 [--argle] [--fp32] [--no-otoc] [--steps N] [--sts NT]
//                        [--frcdisp] [--advection] [--counterflow] [--sgle] [--selftrunc]
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <sys/stat.h>
#include <thread>
#include <vector>
#include "../../include/vk.h"

namespace {

// Fortran Ew.d: [-]0.ddddddE+ee right-justified in w columns.
std::string fortran_e(double x, int w = 15, int d = 6) {
  char buf[64];
  if (x == 0.0 || !std::isfinite(x)) {
    if (!std::isfinite(x)) std::snprintf(buf, sizeof(buf), "%*s", w, std::isnan(x) ? "NaN" : (x > 0 ? "Infinity" : "-Infinity"));
    else std::snprintf(buf, sizeof(buf), "%*s", w, (std::string("0.") + std::string(d, '0') + "E+00").c_str());
    return buf;
  }
  const double ax = std::fabs(x);
  int e = (int)std::floor(std::log10(ax)) + 1;
  double m = ax / std::pow(10.0, e);
  // round the mantissa to d digits; renormalise on carry
  double scale = std::pow(10.0, d);
  double mr = std::round(m * scale);
  if (mr >= scale) { mr /= 10.0; mr = std::round(mr); e += 1; }
  if (mr < scale / 10.0) { mr *= 10.0; e -= 1; }
  char mant[32];
  std::snprintf(mant, sizeof(mant), "%0*lld", d, (long long)mr);
  char ex[16];
  if (std::abs(e) <= 99) std::snprintf(ex, sizeof(ex), "E%c%02d", e < 0 ? '-' : '+', std::abs(e));
  else std::snprintf(ex, sizeof(ex), "%c%03d", e < 0 ? '-' : '+', std::abs(e));
  std::string s = std::string(x < 0 ? "-" : "") + "0." + mant + ex;
  std::snprintf(buf, sizeof(buf), "%*s", w, s.c_str());
  return buf;
}

void append_line(const std::string& path, const std::vector<double>& vals) {
  FILE* f = std::fopen(path.c_str(), "a");
  if (!f) {
    std::fprintf(stderr, "cannot open %s\n", path.c_str());
    std::exit(2);
  }
  std::string line;
  for (double v : vals) line += fortran_e(v);
  std::fprintf(f, "%s\n", line.c_str());
  std::fclose(f);
}

void mkdirs() {
  const char* dirs[] = {"data", "data/wf", "spectra"};
  for (const char* d : dirs) mkdir(d, 0755);
}

// One Fortran sequential-unformatted record (4-byte length markers) appended.
void append_record(const std::string& path, const void* data, size_t bytes) {
  FILE* f = std::fopen(path.c_str(), "ab");
  if (!f) {
    std::fprintf(stderr, "cannot open %s\n", path.c_str());
    std::exit(1);
  }
  const uint32_t m = (uint32_t)bytes;
  std::fwrite(&m, 4, 1, f);
  std::fwrite(data, 1, bytes, f);
  std::fwrite(&m, 4, 1, f);
  std::fclose(f);
}

bool file_exists(const std::string& p) {
  struct stat st;
  return stat(p.c_str(), &st) == 0;
}

int check(int rc, const char* what) {
  if (rc != VK_OK) {
    std::fprintf(stderr, "%s failed (%d): %s\n", what, rc, vk_last_error());
    std::exit(1);
  }
  return rc;
}

// initialize_particles: lines "iopoint ptime x y" (list-directed).
void read_particle_file(const std::string& path, int np, std::vector<double>& out) {
  FILE* f = std::fopen(path.c_str(), "r");
  if (!f) {
    std::fprintf(stderr, "cannot open %s\n", path.c_str());
    std::exit(1);
  }
  out.assign(2 * (size_t)np, 0.0);
  for (int i = 0; i < np; ++i) {
    int io;
    double t, a, b;
    if (std::fscanf(f, "%d %lf %lf %lf", &io, &t, &a, &b) != 4) {
      std::fprintf(stderr, "%s: expected %d lines of 'iopoint time x y'\n", path.c_str(), np);
      std::exit(1);
    }
    out[2 * i] = a;
    out[2 * i + 1] = b;
  }
  std::fclose(f);
}

}  // namespace

int main(int argc, char** argv) {
  bool argle = false, fp32 = false, otoc = true;
  long steps_override = -1;
  int sts_nt = 0;  // -DGPSTS path: records per spatio-temporal spectrum (0 = off)
  int vflags = 0;  // -DGPE_FRCDISP / ADVECTION / COUNTERFLOW / SGLE / SELFTRUNC
  for (int i = 1; i < argc; ++i) {
    if (!std::strcmp(argv[i], "--argle")) argle = true;
    else if (!std::strcmp(argv[i], "--fp32")) fp32 = true;
    else if (!std::strcmp(argv[i], "--no-otoc")) otoc = false;
    else if (!std::strcmp(argv[i], "--steps") && i + 1 < argc) steps_override = std::atol(argv[++i]);
    else if (!std::strcmp(argv[i], "--sts") && i + 1 < argc) sts_nt = std::atoi(argv[++i]);
    else if (!std::strcmp(argv[i], "--frcdisp")) vflags |= VK_VAR_FRCDISP;
    else if (!std::strcmp(argv[i], "--advection")) vflags |= VK_VAR_ADVECTION;
    else if (!std::strcmp(argv[i], "--counterflow")) vflags |= VK_VAR_COUNTERFLOW;
    else if (!std::strcmp(argv[i], "--sgle")) vflags |= VK_VAR_SGLE;
    else if (!std::strcmp(argv[i], "--selftrunc")) vflags |= VK_VAR_SELFTRUNC;
    else {
      std::fprintf(stderr,
                   "usage: %s [--argle] [--fp32] [--no-otoc] [--steps N] [--sts NT] [--frcdisp] [--advection] "
                   "[--counterflow] [--sgle] [--selftrunc]\n",
                   argv[0]);
      return 2;
    }
  }
  const auto t0 = std::chrono::steady_clock::now();
  vk_namelist nl;
  check(vk_read_namelists("parameter.txt", file_exists("parameter_gpe.txt") ? "parameter_gpe.txt" : nullptr, &nl),
        "reading parameter.txt");
  vk_params p;
  check(vk_params_derive(&nl, fp32 ? VK_PREC_FP32 : VK_PREC_FP64, otoc ? 1 : 0, &p), "deriving parameters");
  const long maxiter = steps_override >= 0 ? steps_override : nl.maxiter;
  const int fsteps = nl.fsteps > 0 ? nl.fsteps : 1 << 30, gsteps = nl.gsteps > 0 ? nl.gsteps : 1 << 30;
  const int ssteps = nl.ssteps > 0 ? nl.ssteps : 1 << 30;
  const int ststeps = sts_nt > 0 ? (nl.ststeps > 0 ? nl.ststeps : 20) : 1 << 30;
  const int nx = p.nx, ny = p.ny, np = p.n_particles;
  const int nshell = vk_nshell(nx);
  std::printf(" VIKSHOBHA 2D GPE on one GPU: Nx %d Ny %d dt %g %s %s\n", nx, ny, p.dt, argle ? "ARGLE" : "RK4",
              fp32 ? "FP32" : "FP64");
  mkdirs();
  void* ctx = nullptr;
  check(vk_init(&p, &ctx), "vk_init");
  std::vector<double> psi(2 * (size_t)nx * ny);
  const std::string fr = "restart/wf/wf" + std::to_string(nl.nrst) + "p1.dat";
  int32_t icpoint;
  double tfile, dtfile;
  if (nl.nsplit_orignal > 1) {  // regroup the ranks' files (src/io_fields.f90:121-146)
    const std::string pre = "restart/wf/wf" + std::to_string(nl.nrst);
    check(vk_read_wf_split(pre.c_str(), nl.nsplit_orignal, nx, ny, &icpoint, &tfile, &dtfile, psi.data()),
          "reading the split restart field");
  } else {
    check(vk_read_wf(fr.c_str(), nx, ny, &icpoint, &tfile, &dtfile, psi.data()), "reading the restart field");
  }
  check(vk_set_psi(ctx, psi.data()), "vk_set_psi");
  if (vflags) {  // the compile-time branches of the reference, from the namelists
    vk_variant var;
    check(vk_variant_derive(&nl, vflags, 1, &var), "vk_variant_derive");
    check(vk_set_variant(ctx, &var), "vk_set_variant");
  }
  const std::string nrs = std::to_string(0);  // restart_from_argle_data sets nrst = 0
  if (np > 0) {
    std::vector<double> pos, vel, f0;
    const std::string suf = ".dat_nrst" + std::to_string(nl.nrst);
    read_particle_file("restart/part/gppos" + suf, np, pos);
    read_particle_file("restart/part/gpvel" + suf, np, vel);
    read_particle_file("restart/part/gpf0ext" + suf, np, f0);
    check(vk_particles_set(ctx, pos.data(), vel.data(), f0.data()), "vk_particles_set");
  }
  std::vector<double> sc(10), spec(6 * (size_t)(nshell + 1));
  std::vector<double> ppos(2 * (size_t)std::max(np, 1)), pvel(ppos.size()), pfrc(ppos.size());
  int fldpoint = 0, spcpoint = 0, stspoint = 0, stsfile = nl.strst;
  double time = 0.0;

  // sts_gpe (src/diagnostics.f90:636-695): time, the kx = 0 line and the
  // plane of kpsi appended to files; the same record goes to the GPU ring, and
  // every sts_nt records the spectra of Run/CompSTS/driver.f90 are written
  // (sts1d_kx0 / sts2d text files, one line per frequency).
  std::vector<double> kbuf;
  if (sts_nt > 0) {
    mkdir("data/sts1d", 0755);
    mkdir("data/sts2d", 0755);
    kbuf.resize(2 * (size_t)nx * ny);
    check(vk_sts_begin(ctx, sts_nt), "vk_sts_begin");
  }
  auto sts = [&](double t) {
    append_line("data/sts_time.dat_nrst" + nrs, {t});
    check(vk_get_kpsi(ctx, kbuf.data()), "vk_get_kpsi");
    append_record("data/sts1d/kpsi_x0_nrst" + nrs + ".dat", kbuf.data(), sizeof(double) * 2 * ny);
    append_record("data/sts2d/kpsi_nrst" + nrs + "p1.dat", kbuf.data(), sizeof(double) * 2 * (size_t)nx * ny);
    check(vk_sts_record(ctx), "vk_sts_record");
    int32_t cnt = 0;
    check(vk_sts_count(ctx, &cnt), "vk_sts_count");
    if (cnt == sts_nt) {
      const int nsh = nx / 3 + 1;
      std::vector<double> s1((size_t)sts_nt * ny), s2((size_t)sts_nt * nsh);
      check(vk_sts_spectra(ctx, s1.data(), s2.data()), "vk_sts_spectra");
      const std::string id = std::to_string(stsfile++);
      FILE* f1 = std::fopen(("data/sts1d_kx0_nrst" + id + ".dat").c_str(), "w");
      FILE* f2 = std::fopen(("data/sts2d_nrst" + id + ".dat").c_str(), "w");
      for (int w = 0; w < sts_nt; ++w) {
        if (f1) {
          for (int j = 0; j < ny; ++j) std::fprintf(f1, " %24.16E", s1[(size_t)w * ny + j]);
          std::fprintf(f1, "\n");
        }
        if (f2) {
          for (int j = 0; j < nsh; ++j) std::fprintf(f2, " %24.16E", s2[(size_t)w * nsh + j]);
          std::fprintf(f2, "\n");
        }
      }
      if (f1) std::fclose(f1);
      if (f2) std::fclose(f2);
    }
  };

  // io_fields: the field goes out asynchronously (vk_dump_begin); a writer
  // thread waits for the copy and writes the file while the GPU steps on.
  std::thread writer;
  std::vector<double> wbuf(2 * (size_t)nx * ny);
  auto join_writer = [&]() {
    if (writer.joinable()) writer.join();
  };
  auto io_fields = [&](int n, double t) {
    const std::string f = "data/wf/wf" + std::to_string(n) + "p1.dat";
    if (file_exists(f)) {  // the reference opens with STATUS='NEW'
      std::fprintf(stderr, "%s exists; refusing to overwrite\n", f.c_str());
      std::exit(1);
    }
    join_writer();  // one dump in flight at a time
    check(vk_dump_begin(ctx), "vk_dump_begin");
    writer = std::thread([&, f, n, t]() {
      check(vk_dump_wait(ctx, wbuf.data()), "vk_dump_wait");
      check(vk_write_wf(f.c_str(), n, t, p.dt, nx, ny, wbuf.data()), "writing the field");
    });
    if (np > 0) {
      check(vk_particles_get(ctx, ppos.data(), pvel.data(), pfrc.data()), "vk_particles_get");
      const char* names[3] = {"gppos", "gpvel", "gpf0ext"};
      for (int k = 0; k < 3; ++k) {
        if (k == 2) continue;  // f0ext is constant; written once below
        FILE* fo = std::fopen((std::string("data/") + names[k] + "_ckp.dat_nrst" + nrs).c_str(), "a");
        const std::vector<double>& v = k == 0 ? ppos : pvel;
        for (int i = 0; i < np; ++i) std::fprintf(fo, " %12d %24.16E %24.16E %24.16E\n", n, t, v[2 * i], v[2 * i + 1]);
        std::fclose(fo);
      }
    }
  };
  auto diagnostics = [&](int spoint, long jtime, double t) {
    int32_t nv[2];
    check(vk_diagnostics(ctx, sc.data(), spec.data(), nv), "vk_diagnostics");
    append_line("data/energy1.dat_nrst" + nrs, {t, sc[2], sc[3], sc[4], sc[5]});
    append_line("data/norm.dat_nrst" + nrs, {t, sc[6]});
    append_line("data/mom.dat_nrst" + nrs, {t, sc[0], sc[1]});
    // quantglobal_gpe (diagnostics.f90:588-604)
    double ek = 0, ei = 0, ec = 0, eq = 0, en = 0;
    for (int m = 1; m <= nshell; ++m) {
      ek += spec[0 * (nshell + 1) + m];
      ei += spec[1 * (nshell + 1) + m];
      ec += spec[2 * (nshell + 1) + m];
      eq += spec[3 * (nshell + 1) + m];
    }
    for (int m = 0; m <= nshell; ++m) en += spec[4 * (nshell + 1) + m];
    if (jtime % gsteps == 0) {
      append_line("data/energy.dat_nrst" + nrs, {t, ek, ei, ec, eq, en});
      append_line("data/n0.dat_nrst" + nrs, {t, spec[5 * (nshell + 1) + 0]});
    }
    if (jtime % ssteps == 0) {  // spectrum_gpe (diagnostics.f90:608-634)
      const std::string f = "spectra/spec" + std::to_string(spoint) + ".dat";
      FILE* fo = std::fopen(f.c_str(), "w");
      for (int m = 1; m <= nshell; ++m) {
        std::string line = fortran_e((double)m);
        for (int j = 0; j < 6; ++j) line += fortran_e(spec[(size_t)j * (nshell + 1) + m]);
        std::fprintf(fo, "%s\n", line.c_str());
      }
      std::fclose(fo);
    }
    append_line("data/vortices.dat_nrst" + nrs, {t, (double)nv[0], (double)nv[1]});
    if (np > 0) {
      check(vk_particles_get(ctx, ppos.data(), pvel.data(), pfrc.data()), "vk_particles_get");
      for (int i = 0; i < np; ++i) {
        const std::string id = std::to_string(i + 1);
        append_line("data/gpobj_pos_" + id + ".dat_nrst" + nrs, {t, ppos[2 * i], ppos[2 * i + 1]});
        append_line("data/gpobj_vel_" + id + ".dat_nrst" + nrs, {t, pvel[2 * i], pvel[2 * i + 1]});
        append_line("data/gpobj_frc_" + id + ".dat_nrst" + nrs, {t, pfrc[2 * i], pfrc[2 * i + 1]});
      }
      double mx = 0, my = 0;
      for (int i = 0; i < np; ++i) {
        mx += p.gp_mass_part * pvel[2 * i];
        my += p.gp_mass_part * pvel[2 * i + 1];
      }
      append_line("data/egpobj.dat_nrst" + nrs, {t, sc[7], sc[8], sc[9]});
      append_line("data/momgpobj.dat_nrst" + nrs, {t, mx, my});
    }
  };

  // solve (src/solve.f90:414-523) with nrst = 0 after restart_from_argle_data
  io_fields(fldpoint, time);
  diagnostics(spcpoint, 0, time);
  if (sts_nt > 0) sts(time);  // src/solve.f90:96-98 (nrst = 0)
  double residual = 0.0;
  long itime = 0;
  while (itime < maxiter) {
    // advance to the next output point in one call
    long next = maxiter;
    const long nf = (itime / fsteps + 1) * (long)fsteps, ng = (itime / gsteps + 1) * (long)gsteps;
    const long nst = (itime / ststeps + 1) * (long)ststeps;
    next = std::min(next, std::min(std::min(nf, ng), nst));
    const int n = (int)(next - itime);
    if (argle) check(vk_argle(ctx, n, &residual), "vk_argle");
    else check(vk_gpe_rk4(ctx, n), "vk_gpe_rk4");
    itime = next;
    time = itime * p.dt;  // time = time + dt per step
    if (itime % fsteps == 0) {
      ++fldpoint;
      io_fields(fldpoint, time);
      if (argle && (vflags & VK_VAR_SGLE)) {  // write_chempot_for_restart (src/solve.f90:112-114)
        double om = 0.0;
        check(vk_get_chempot(ctx, &om), "vk_get_chempot");
        append_line("data/cpot_sgle.dat_nrst" + nrs, {time, om});
      }
    }
    if (itime % gsteps == 0) {
      if (itime % ssteps == 0) ++spcpoint;
      diagnostics(spcpoint, itime, time);
      if (argle) append_line("data/argle_residual.dat_nrst" + nrs, {time, residual});
      if (!std::isfinite(sc[6]) || sc[6] > 1e6 * (2 * M_PI) * (2 * M_PI)) {
        std::fprintf(stderr, "norm blew up at step %ld (norm = %g)\n", itime, sc[6]);
        join_writer();
        return 3;
      }
    }
    if (itime % ststeps == 0) {  // src/solve.f90:139-144
      ++stspoint;
      sts(time);
    }
  }
  join_writer();
  check(vk_finalize(ctx), "vk_finalize");
  const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  FILE* f = std::fopen("run_info.dat", "w");
  if (f) {
    std::fprintf(f, " time taken by           0 processor   %.10f\n", secs);
    std::fclose(f);
  }
  std::printf(" done: %ld steps in %.3f s\n", itime, secs);
  return 0;
}
