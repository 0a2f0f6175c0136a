// trapbec_run.cpp -- the reference's driver program on top of libtrapbec.
//
// Mirrors the control flow of `program run` (run.f90:1-81): read the
// parameters (cparam.local, parsed at run time instead of compiled in,
// cdata.f90:3), write dims.log and the start-up banner (output.f90:9-60),
// restart from data/proc000/var.dat if it exists (initial.f90:44-57,796-818)
// or build init_cond, optionally relax in imaginary time (run.f90:19-35),
// then advance `shots` RK3 steps at a time, printing
// `itime/shots, t, maxPsi, minPsi, meanPsi, intPsi2` and writing var####.dat
// and var.dat after each block (run.f90:43-68), and finally timing.log
// (output.f90:111-118).  Errors follow emergency_stop (mpi_var.f90:164-181):
// the message goes to stdout and to a file named ERROR, and the run stops.
//
// usage: trapbec_run [cparam.local] [data directory]
#include <sys/stat.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <algorithm>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/trapbec.h"
#include "host_util.h"

namespace {

[[noreturn]] void emergency_stop(const std::string& msg) {
  std::printf(" *****FATAL ERROR ABORTING CODE*****\n %s\n", msg.c_str());
  if (FILE* f = std::fopen("ERROR", "w")) {
    std::fprintf(f, " %s\n", msg.c_str());
    std::fclose(f);
  }
  std::exit(1);
}

void check(int rc, const char* where) {
  if (rc != TRAPBEC_OK) {
    const char* detail = trapbec_last_error();
    emergency_stop(std::string(where) + ": " + trapbec_strerror(rc) + (detail && *detail ? std::string(": ") + detail : ""));
  }
}

struct RunControl {  // the run-control names of cparam.local (cparam.local:5-44)
  int shots = 100;
  int nsteps = 1000;
  std::string init_cond = "single_vortex";
  bool imaginary_time = false;
  int imag_nsteps = 0;
  bool full_binary_output = true;
  bool imaginary_output = false;
  bool vel_print = false, qpress_print = false, gnuplot_2d_print = false;
  bool add_pcurrent = false, add_ring = false, add_dipole = false, forcing = false;
  bool phase_imprint_on = false;
  int force_freq = 10;
};

bool as_bool(const std::string& v) {
  std::string s;
  for (char c : v) s += (char)std::tolower((unsigned char)c);
  return s.find("true") != std::string::npos || s == "t";
}
std::string unquote(const std::string& v) {
  if (v.size() >= 2 && (v[0] == '\'' || v[0] == '"')) return v.substr(1, v.size() - 2);
  return v;
}

bool file_exists(const std::string& p) {
  struct stat st;
  return ::stat(p.c_str(), &st) == 0;
}

// List-directed output of a real of the build's kind: 9 significant digits
// for the shipped single-precision build, 17 for the -fdefault-real-8 one.
void put_real(FILE* f, double v, bool f64) { std::fprintf(f, f64 ? " %25.16E" : " %16.8E", v); }

// 2D_slice##.log of var_print (output.f90:92-101): x, y, |Psi(z=1)|^2 per
// line, a blank line after each x; list-directed output of the build's kind.
void write_2d_slice(trapbec_ctx* ctx, const trapbec_params& p, const std::string& datadir, int q) {
  const bool f64 = p.precision == TRAPBEC_FP64;
  const size_t n = (size_t)p.nx * p.ny * p.nz;
  std::vector<double> psi(2 * n);
  std::vector<float> psif;
  if (f64) {
    check(trapbec_get_psi(ctx, psi.data(), TRAPBEC_LAYOUT_INTERIOR), "gnuplot_2D_print");
  } else {
    psif.resize(2 * n);
    check(trapbec_get_psi(ctx, psif.data(), TRAPBEC_LAYOUT_INTERIOR), "gnuplot_2D_print");
    for (size_t i = 0; i < 2 * n; ++i) psi[i] = psif[i];
  }
  char num[8];
  if (q >= 0 && q <= 99) std::snprintf(num, sizeof(num), "%02d", q);
  else std::snprintf(num, sizeof(num), "**");
  const std::string path = datadir + "/proc000/2D_slice" + num + ".log";
  FILE* f = std::fopen(path.c_str(), "w");
  if (!f) emergency_stop("cannot open " + path);
  for (int i = 0; i < p.nx; ++i) {
    const double x = (2.0 * (i + 1) - 1) / (2.0 * p.nx) * p.lx - p.lx / 2.0;   // initial.f90:40-42
    for (int j = 0; j < p.ny; ++j) {
      const double y = (2.0 * (j + 1) - 1) / (2.0 * p.ny) * p.ly - p.ly / 2.0;
      const size_t c = ((size_t)i * p.ny + j) * p.nz;   // k = 1
      const double a2 = psi[2 * c] * psi[2 * c] + psi[2 * c + 1] * psi[2 * c + 1];
      put_real(f, x, f64);
      put_real(f, y, f64);
      put_real(f, a2, f64);
      std::fprintf(f, "\n");
    }
    std::fprintf(f, "\n");
  }
  std::fclose(f);
}

}  // namespace

int main(int argc, char** argv) {
  const std::string cparam = argc > 1 ? argv[1] : "cparam.local";
  const std::string datadir = argc > 2 ? argv[2] : "./data";
  std::ifstream in(cparam);
  if (!in) emergency_stop("cannot open " + cparam);
  std::stringstream ss;
  ss << in.rdbuf();
  trapbec_params p;
  trapbec_params_default(&p);
  p.precision = TRAPBEC_FP32;  // default complex, as the shipped build
  std::vector<std::pair<std::string, std::string>> rest;
  char err[256] = {0};
  if (tbh::parse_cparam_text(ss.str().c_str(), &p, &rest, err, sizeof(err)) != TRAPBEC_OK) emergency_stop(err);
  RunControl rc;
  for (auto& kv : rest) {
    const std::string& k = kv.first;
    const std::string& v = kv.second;
    if (k == "shots") rc.shots = std::atoi(v.c_str());
    else if (k == "nsteps") rc.nsteps = std::atoi(v.c_str());
    else if (k == "init_cond") rc.init_cond = unquote(v);
    else if (k == "imaginary_time") rc.imaginary_time = as_bool(v);
    else if (k == "imag_nsteps") rc.imag_nsteps = std::atoi(v.c_str());
    else if (k == "full_binary_output") rc.full_binary_output = as_bool(v);
    else if (k == "imaginary_output") rc.imaginary_output = as_bool(v);
    else if (k == "vel_print") rc.vel_print = as_bool(v);
    else if (k == "qpress_print") rc.qpress_print = as_bool(v);
    else if (k == "add_pcurrent") rc.add_pcurrent = as_bool(v);
    else if (k == "add_ring") rc.add_ring = as_bool(v);
    else if (k == "add_dipole") rc.add_dipole = as_bool(v);
    else if (k == "forcing") rc.forcing = as_bool(v);
    else if (k == "force_freq") rc.force_freq = std::atoi(v.c_str());
    else if (k == "phase_imprint_on") rc.phase_imprint_on = as_bool(v);
    else if (k == "gnuplot_2d_print") rc.gnuplot_2d_print = as_bool(v);
  }
  if (rc.shots <= 0) emergency_stop("shots must be positive");
  if (rc.forcing && rc.force_freq <= 0) emergency_stop("force_freq must be positive");
  if (const char* prec = std::getenv("TRAPBEC_PRECISION")) p.precision = std::atoi(prec) ? TRAPBEC_FP64 : TRAPBEC_FP32;

  tbh::mkdirs(datadir + "/proc000");
  check(trapbec_write_dims(&p, datadir.c_str()), "dims_print");   // output.f90:48-60
  // initial_print (output.f90:9-46)
  std::printf(" TrapBEC code initialised\n");
  if (p.two_dim) std::printf(" WARNING: Running in 2D mode .\n");
  std::printf(" Running a %04dx%04dx%04d GPE simulation\n", p.nx, p.ny, p.nz);
  std::printf(" Dimensions: Lx=%6.2f Ly=%6.2f Lz=%6.2f\n", p.lx, p.ly, p.lz);
  std::printf(" Timestep dt:%8.3f\n", p.dt_re);
  std::printf(" Initial condition: %s\n", rc.init_cond.c_str());
  std::printf(" Running for %06d timesteps, file print every %04d\n", rc.nsteps, rc.shots);
  std::printf(" Dissipation, gamma= %g\n", p.gamma);
  if (p.advective_vx != 0.0) std::printf(" Moving frame, vx= %g\n", p.advective_vx);
  else if (p.omega_z != 0.0) std::printf(" Rotating frame, Omega= %g\n", p.omega_z);

  trapbec_ctx* ctx = nullptr;
  check(trapbec_create(&p, &ctx), "mesh_init");
  double t = 0.0;
  int nstart = 1;
  bool restarted = false;
  if (file_exists(datadir + "/proc000/var.dat") || file_exists(datadir + "/proc00/var.dat")) {
    std::printf(" attempting to restart from 001 processes, this may fail!\n");
    check(trapbec_read_restart(ctx, datadir.c_str(), &nstart, &t), "reload_data");
    std::printf(" succsesful restart, t= %g\n", t);
    restarted = true;
  } else {
    check(trapbec_init_state(ctx, rc.init_cond.c_str(), nullptr), "mesh_init: init_cond");
  }

  if (!restarted && rc.imaginary_time) {  // run.f90:19-35
    for (int itime = 1; itime <= rc.imag_nsteps;) {
      const int m = (itime + rc.shots - 1) / rc.shots * rc.shots;   // next output step
      // phase_imprint follows every imaginary step (run.f90:25)
      const int k = rc.phase_imprint_on ? 1 : std::min(m - itime + 1, rc.imag_nsteps - itime + 1);
      int done = 0;
      double ratio = 0;
      check(trapbec_step_imag(ctx, k, TRAPBEC_IMAG_REF_EULER, 0.0, &done, &ratio), "imaginary time");
      if (rc.phase_imprint_on) check(trapbec_init_state(ctx, "phase_imprint", nullptr), "phase_imprint");
      itime += k;
      const int last = itime - 1;
      if (last % rc.shots == 0) {
        std::printf(" %12d", last / rc.shots);
        put_real(stdout, ratio, p.precision == TRAPBEC_FP64);
        std::printf("\n");
        if (rc.imaginary_output)
          check(trapbec_write_var(ctx, datadir.c_str(), last, rc.shots, t, 1), "imaginary_print");
      }
    }
    std::printf(" finished imaginary time propagation\n");
  }

  // run.f90:37-40, after a restart too
  if (rc.add_pcurrent) check(trapbec_init_state(ctx, "add_pcurrent", nullptr), "setup_pcurrent");
  if (rc.add_ring) check(trapbec_init_state(ctx, "add_ring", nullptr), "setup_add_ring");
  if (rc.add_dipole) check(trapbec_init_state(ctx, "add_dipole", nullptr), "setup_add_dipole");

  // forcing draws: TRAPBEC_FORCE_SEED (default 1), draw number itime/force_freq
  const uint64_t force_seed = std::getenv("TRAPBEC_FORCE_SEED") ? std::strtoull(std::getenv("TRAPBEC_FORCE_SEED"), nullptr, 10) : 1;
  double tot_ms = 0.0;
  int timed_steps = 0;
  // The state of an output step is read back into page-locked memory on a
  // copy stream (trapbec_get_psi_async) and its var####.dat and var.dat are
  // written from there while the next block of steps runs; the files are the
  // ones var_print writes at that step (output.f90:64-75,102-108).
  const size_t state_bytes = (size_t)p.nx * p.ny * p.nz * (p.precision == TRAPBEC_FP64 ? 16 : 8);
  void* out_buf = nullptr;
  check(trapbec_host_alloc(state_bytes, &out_buf), "output buffer");
  bool out_pending = false;
  int out_last = 0;
  double out_t = 0.0;
  auto flush_output = [&]() {
    if (!out_pending) return;
    out_pending = false;
    check(trapbec_wait_psi(ctx), "var_print: read-back");
    if (rc.full_binary_output)
      check(trapbec_write_var_host(&p, datadir.c_str(), out_last, rc.shots, out_t, 0, out_buf), "var_print");
    check(trapbec_write_restart_host(&p, datadir.c_str(), out_last, out_t, out_buf), "var_print: var.dat");
  };
  for (int itime = nstart; itime <= rc.nsteps;) {   // run.f90:43-76
    int m = (itime + rc.shots - 1) / rc.shots * rc.shots;   // next output step
    if (rc.forcing) m = std::min(m, (itime + rc.force_freq - 1) / rc.force_freq * rc.force_freq);
    const int k = std::min(m - itime + 1, rc.nsteps - itime + 1);
    const int st = trapbec_step_rt_async(ctx, k, &t);
    flush_output();   // the last output's files, written while these steps run
    check(st, "RK3 step");
    double ms = 0;
    check(trapbec_last_kernel_ms(ctx, &ms), "RK3 step");   // waits for the steps
    tot_ms += ms;
    timed_steps += k;
    itime += k;
    const int last = itime - 1;
    if (last % rc.shots == 0) {
      trapbec_diag_out d;
      check(trapbec_diag(ctx, &d), "Psi_info/Psi_norm");
      std::printf(" %12d", last / rc.shots);   // run.f90:62
      for (double v : {t, d.maxpsi, d.minpsi, d.meanpsi, d.intpsi2}) put_real(stdout, v, p.precision == TRAPBEC_FP64);
      std::printf("\n");
      if (d.nonfinite) emergency_stop("non-finite values in Psi");
      // run.f90:64-66 computes the diagnostics, output.f90:73-91 writes them
      if (rc.vel_print)
        check(trapbec_write_field(ctx, datadir.c_str(), last, rc.shots, TRAPBEC_FIELD_VELOCITY), "get_phase");
      if (rc.qpress_print)
        check(trapbec_write_field(ctx, datadir.c_str(), last, rc.shots, TRAPBEC_FIELD_QPRESSURE), "get_qpressure");
      if (rc.gnuplot_2d_print) write_2d_slice(ctx, p, datadir, last / rc.shots);
      check(trapbec_get_psi_async(ctx, out_buf, TRAPBEC_LAYOUT_INTERIOR), "var_print: read-back");
      out_pending = true;
      out_last = last;
      out_t = t;
    }
    if (rc.forcing && last % rc.force_freq == 0)   // run.f90:70-74
      check(trapbec_force_random_points(ctx, force_seed, (uint64_t)(last / rc.force_freq), nullptr),
            "force_random_points");
  }
  flush_output();
  trapbec_host_free(out_buf);
  const double tpt = timed_steps ? tot_ms * 1e-3 / timed_steps : 0.0;
  check(trapbec_write_timing(&p, datadir.c_str(), tpt, 0.0), "print_timing");
  trapbec_destroy(ctx);
  return 0;
}
