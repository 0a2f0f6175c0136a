// params_io.cpp -- cparam.local parsing, defaults and the reference's output
// file layout (host C++, part of libtrapbec).
//
// cparam.local (cparam.local:1-44) is a Fortran include of declarations such
// as `real, parameter :: harm_wx=900, harm_wy=8`.  The reference compiles it
// in (cdata.f90:3); here it is parsed at run time into trapbec_params.
// Output files follow output.f90:48-118 (Fortran unformatted sequential
// records as gfortran writes them: 4-byte length markers around each record,
// split into sub-records above 2^31-9 bytes) and are readable by
// bin/gather.m:6-28.
#include <algorithm>
#include <cctype>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <sys/stat.h>
#include <vector>

#include "../../include/trapbec.h"
#include "host_util.h"

namespace {

const double HUGE_REAL = 3.4028234663852886e38;  // huge(1.) of a default real

std::string lower(std::string s) {
  for (auto& c : s) c = (char)std::tolower((unsigned char)c);
  return s;
}
std::string trim(const std::string& s) {
  size_t a = s.find_first_not_of(" \t\r\n");
  if (a == std::string::npos) return "";
  size_t b = s.find_last_not_of(" \t\r\n");
  return s.substr(a, b - a + 1);
}

// Split on commas that are not inside parentheses or quotes.
std::vector<std::string> split_top(const std::string& s) {
  std::vector<std::string> out;
  int depth = 0;
  char q = 0;
  std::string cur;
  for (char c : s) {
    if (q) {
      cur += c;
      if (c == q) q = 0;
      continue;
    }
    if (c == '\'' || c == '"') { q = c; cur += c; continue; }
    if (c == '(') depth++;
    if (c == ')') depth--;
    if (c == ',' && depth == 0) { out.push_back(cur); cur.clear(); continue; }
    cur += c;
  }
  if (!trim(cur).empty()) out.push_back(cur);
  return out;
}

bool parse_real(const std::string& v0, double* out) {
  std::string v = lower(trim(v0));
  if (v.rfind("huge(", 0) == 0) { *out = HUGE_REAL; return true; }
  for (auto& c : v) if (c == 'd') c = 'e';      // 1d0 -> 1e0
  if (v.size() > 2 && v[0] == '(' && v.back() == ')') v = v.substr(1, v.size() - 2);
  char* end = nullptr;
  errno = 0;
  double d = std::strtod(v.c_str(), &end);
  if (end == v.c_str()) return false;
  std::string rest = trim(std::string(end));
  // allow a kind suffix such as 1.0_8
  if (!rest.empty() && rest[0] == '_') rest.clear();
  if (!rest.empty()) return false;
  *out = d;
  return true;
}

bool parse_complex(const std::string& v0, double* re, double* im) {
  std::string v = trim(v0);
  if (!v.empty() && v[0] == '(') {
    size_t c = v.find(',');
    if (c == std::string::npos || v.back() != ')') return false;
    return parse_real(v.substr(1, c - 1), re) && parse_real(v.substr(c + 1, v.size() - c - 2), im);
  }
  *im = 0;
  return parse_real(v, re);
}

bool parse_logical(const std::string& v0, int* out) {
  std::string v = lower(trim(v0));
  if (v == ".true." || v == "t" || v == ".t.") { *out = 1; return true; }
  if (v == ".false." || v == "f" || v == ".f.") { *out = 0; return true; }
  return false;
}

bool parse_string(const std::string& v0, std::string* out) {
  std::string v = trim(v0);
  if (v.size() >= 2 && (v[0] == '\'' || v[0] == '"') && v.back() == v[0]) {
    *out = v.substr(1, v.size() - 2);
    return true;
  }
  return false;
}

// Names of cparam.local (cparam.local:2-44) that the time-stepping path does
// not use; they are accepted and ignored by trapbec_params_parse.
const char* IGNORED[] = {"shots", "nsteps", "init_cond", "imaginary_time", "imag_nsteps",
                         "forcing", "force_freq", "full_binary_output", "imaginary_output",
                         "gnuplot_2d_print", "qpress_print", "vel_print", "add_pcurrent",
                         "add_ring", "add_dipole", "vor_line_count", "phase_imprint_on"};

}  // namespace

namespace tbh {

int parse_cparam_text(const char* text, trapbec_params* p, std::vector<std::pair<std::string, std::string>>* rest,
                      char* errbuf, size_t errlen) {
  auto fail = [&](const std::string& m) {
    if (errbuf && errlen) std::snprintf(errbuf, errlen, "%s", m.c_str());
    set_error(m);
    return TRAPBEC_ERR_PARSE;
  };
  std::string all(text ? text : "");
  size_t pos = 0;
  int lineno = 0;
  while (pos <= all.size()) {
    size_t e = all.find('\n', pos);
    if (e == std::string::npos) e = all.size();
    std::string line = all.substr(pos, e - pos);
    pos = e + 1;
    ++lineno;
    // strip a trailing comment (a '!' outside quotes)
    {
      char q = 0;
      for (size_t i = 0; i < line.size(); ++i) {
        char c = line[i];
        if (q) { if (c == q) q = 0; continue; }
        if (c == '\'' || c == '"') q = c;
        else if (c == '!') { line = line.substr(0, i); break; }
      }
    }
    line = trim(line);
    if (line.empty()) continue;
    size_t dc = line.find("::");
    if (dc == std::string::npos) return fail("line " + std::to_string(lineno) + ": expected a declaration 'type :: name=value'");
    std::string decl = lower(trim(line.substr(0, dc)));
    std::string body = line.substr(dc + 2);
    std::string type = decl.substr(0, decl.find_first_of(" ,("));
    for (const std::string& item : split_top(body)) {
      size_t eq = item.find('=');
      if (eq == std::string::npos) return fail("line " + std::to_string(lineno) + ": '" + trim(item) + "' has no value");
      std::string name = lower(trim(item.substr(0, eq)));
      std::string val = trim(item.substr(eq + 1));
      auto bad = [&]() { return fail("line " + std::to_string(lineno) + ": bad value for " + name + ": " + val); };
      double d = 0, di = 0;
      int b = 0;
      std::string s;
      if (name == "lx" || name == "ly" || name == "lz" || name == "gamma" || name == "harm_wx" ||
          name == "harm_wy" || name == "harm_wz" || name == "potential_off" || name == "wbeam" ||
          name == "advective_vx" || name == "omega_z" || name == "t_spindown" || name == "ring_rad") {
        if (!parse_real(val, &d)) return bad();
        if (name == "lx") p->lx = d; else if (name == "ly") p->ly = d; else if (name == "lz") p->lz = d;
        else if (name == "gamma") p->gamma = d; else if (name == "harm_wx") p->harm_wx = d;
        else if (name == "harm_wy") p->harm_wy = d; else if (name == "harm_wz") p->harm_wz = d;
        else if (name == "potential_off") p->potential_off = d; else if (name == "wbeam") p->wbeam = d;
        else if (name == "advective_vx") p->advective_vx = d; else if (name == "omega_z") p->omega_z = d;
        else if (name == "t_spindown") p->t_spindown = d; else p->ring_rad = d;
      } else if (name == "nx" || name == "ny" || name == "nz" || name == "winding_number" ||
                 name == "vor_ring_count") {
        if (!parse_real(val, &d) || d != std::floor(d)) return bad();
        int v = (int)d;
        if (name == "nx") p->nx = v; else if (name == "ny") p->ny = v; else if (name == "nz") p->nz = v;
        else if (name == "winding_number") p->winding_number = v; else p->vor_ring_count = v;
      } else if (name == "dt") {
        if (!parse_complex(val, &d, &di)) return bad();
        p->dt_re = d;
        p->dt_im = di;
      } else if (name == "periodicz" || name == "two_dim" || name == "lbeam") {
        if (!parse_logical(val, &b)) return bad();
        if (name == "periodicz") p->periodicz = b; else if (name == "two_dim") p->two_dim = b; else p->lbeam = b;
      } else if (name == "boundaries") {
        if (!parse_string(val, &s)) return bad();
        s = lower(s);
        if (s == "zero") p->boundaries = TRAPBEC_BC_ZERO;
        else if (s == "solid") p->boundaries = TRAPBEC_BC_SOLID;
        else if (s == "periodic") p->boundaries = TRAPBEC_BC_PERIODIC;
        else return fail("wrong boundaries set: " + s);   // mpi_var.f90:140-141
      } else if (name == "potential") {
        if (!parse_string(val, &s)) return bad();
        s = lower(s);
        static const char* names[] = {"zero", "harmonic", "harmonic_ring", "harmonic_ring2", "barrier",
                                      "box_trap", "channel", "quartic", "sphere", "mobius", "array"};
        int k = -1;
        for (int q = 0; q < 11; ++q) if (s == names[q]) k = q;
        if (k < 0) return fail("error incorrect potential set: " + s);  // output.f90:28-29
        p->potential = k;
      } else if (name == "precision") {
        if (!parse_string(val, &s)) return bad();
        s = lower(s);
        if (s == "fp32" || s == "single") p->precision = TRAPBEC_FP32;
        else if (s == "fp64" || s == "double") p->precision = TRAPBEC_FP64;
        else return bad();
      } else if (name == "nprocx" || name == "nprocy") {
        if (!parse_real(val, &d) || d < 1) return bad();
        if (name == "nprocx") p->nprocx = (int)d; else p->nprocy = (int)d;
      } else {
        bool ign = false;
        for (const char* n : IGNORED) if (name == n) ign = true;
        if (!ign) return fail("line " + std::to_string(lineno) + ": unknown parameter " + name);
        if (rest) rest->push_back({name, val});
      }
      (void)type;
    }
  }
  return TRAPBEC_OK;
}

// ------------------------------------------------ Fortran record writer --
struct Rec {
  std::vector<char> buf;
  void put(const void* p, size_t n) { buf.insert(buf.end(), (const char*)p, (const char*)p + n); }
};

// gfortran sequential unformatted record, split into sub-records of at most
// 2147483639 bytes; a negative marker means "continued".
static bool write_record(FILE* f, const std::vector<std::pair<const void*, size_t>>& parts) {
  size_t total = 0;
  for (auto& q : parts) total += q.second;
  const size_t MAXSUB = 2147483639ULL;
  size_t done = 0;
  size_t pi = 0, po = 0;
  bool first = true;
  do {
    size_t len = std::min(MAXSUB, total - done);
    bool last = (done + len == total);
    int32_t lead = (int32_t)(last ? len : -(int64_t)len);
    int32_t trail = (int32_t)(first ? len : -(int64_t)len);
    if (std::fwrite(&lead, 4, 1, f) != 1) return false;
    size_t left = len;
    while (left) {
      size_t take = std::min(left, parts[pi].second - po);
      if (take && std::fwrite((const char*)parts[pi].first + po, 1, take, f) != take) return false;
      po += take;
      left -= take;
      if (po == parts[pi].second) { ++pi; po = 0; }
    }
    if (std::fwrite(&trail, 4, 1, f) != 1) return false;
    done += len;
    first = false;
  } while (done < total);
  return true;
}

// Read one record (following sub-records) into out.
static bool read_record(FILE* f, std::vector<char>* out) {
  out->clear();
  while (true) {
    int32_t lead;
    if (std::fread(&lead, 4, 1, f) != 1) return false;
    size_t len = (size_t)(lead < 0 ? -(int64_t)lead : lead);
    size_t old = out->size();
    out->resize(old + len);
    if (len && std::fread(out->data() + old, 1, len, f) != len) return false;
    int32_t trail;
    if (std::fread(&trail, 4, 1, f) != 1) return false;
    if (lead >= 0) return true;
  }
}

bool mkdirs(const std::string& d) {
  std::string cur;
  for (size_t i = 0; i <= d.size(); ++i) {
    if (i == d.size() || d[i] == '/') {
      if (!cur.empty()) {
        if (mkdir(cur.c_str(), 0755) != 0 && errno != EEXIST) return false;
      }
    }
    if (i < d.size()) cur += d[i];
  }
  return true;
}

int write_var_file(const std::string& path, const trapbec_params* p, double t, const void* psi,
                   size_t psi_bytes) {
  size_t sl = path.find_last_of('/');
  if (sl != std::string::npos && !mkdirs(path.substr(0, sl))) { set_error("cannot create " + path); return TRAPBEC_ERR_IO; }
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) { set_error("cannot open " + path); return TRAPBEC_ERR_IO; }
  int32_t coords[2] = {0, 0};
  bool ok;
  if (p->precision == TRAPBEC_FP64) {
    double h[4] = {p->lx, p->ly, p->lz, t};
    ok = write_record(f, {{coords, 8}, {h, 32}, {psi, psi_bytes}});
  } else {
    float h[4] = {(float)p->lx, (float)p->ly, (float)p->lz, (float)t};
    ok = write_record(f, {{coords, 8}, {h, 16}, {psi, psi_bytes}});
  }
  ok = (std::fclose(f) == 0) && ok;
  if (!ok) { set_error("write failed: " + path); return TRAPBEC_ERR_IO; }
  return TRAPBEC_OK;
}

int write_field_file(const std::string& path, const void* data, size_t bytes) {
  size_t sl = path.find_last_of('/');
  if (sl != std::string::npos && !mkdirs(path.substr(0, sl))) { set_error("cannot create " + path); return TRAPBEC_ERR_IO; }
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) { set_error("cannot open " + path); return TRAPBEC_ERR_IO; }
  int32_t coords[2] = {0, 0};
  bool ok = write_record(f, {{coords, 8}, {data, bytes}});   // output.f90:83,89: coords, field
  ok = (std::fclose(f) == 0) && ok;
  if (!ok) { set_error("write failed: " + path); return TRAPBEC_ERR_IO; }
  return TRAPBEC_OK;
}

int write_restart_file(const std::string& path, const trapbec_params* p, int itime, double t,
                       const void* psi, size_t psi_bytes) {
  size_t sl = path.find_last_of('/');
  if (sl != std::string::npos && !mkdirs(path.substr(0, sl))) { set_error("cannot create " + path); return TRAPBEC_ERR_IO; }
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) { set_error("cannot open " + path); return TRAPBEC_ERR_IO; }
  int32_t it = itime + 1;   // output.f90:105 writes itime+1
  bool ok = write_record(f, {{&it, 4}});
  if (p->precision == TRAPBEC_FP64) {
    double tt = t;
    ok = ok && write_record(f, {{&tt, 8}});
  } else {
    float tt = (float)t;
    ok = ok && write_record(f, {{&tt, 4}});
  }
  ok = ok && write_record(f, {{psi, psi_bytes}});
  ok = (std::fclose(f) == 0) && ok;
  if (!ok) { set_error("write failed: " + path); return TRAPBEC_ERR_IO; }
  return TRAPBEC_OK;
}

int read_restart_file(const std::string& path, const trapbec_params* p, int* itime, double* t,
                      void* psi, size_t psi_bytes) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) { set_error("cannot open " + path); return TRAPBEC_ERR_IO; }
  std::vector<char> r;
  int rc = TRAPBEC_OK;
  size_t rsz = p->precision == TRAPBEC_FP64 ? 8 : 4;
  if (!read_record(f, &r) || r.size() != 4) { rc = TRAPBEC_ERR_IO; set_error("restart: bad itime record"); }
  else std::memcpy(itime, r.data(), 4);
  if (rc == TRAPBEC_OK) {
    if (!read_record(f, &r) || r.size() != rsz) { rc = TRAPBEC_ERR_IO; set_error("restart: bad t record (precision mismatch?)"); }
    else if (rsz == 8) std::memcpy(t, r.data(), 8);
    else { float tf; std::memcpy(&tf, r.data(), 4); *t = tf; }
  }
  if (rc == TRAPBEC_OK) {
    if (!read_record(f, &r) || r.size() != psi_bytes) { rc = TRAPBEC_ERR_IO; set_error("restart: psi record has the wrong size"); }
    else std::memcpy(psi, r.data(), psi_bytes);
  }
  std::fclose(f);
  return rc;
}

}  // namespace tbh

extern "C" {

int trapbec_params_default(trapbec_params* p) {
  if (!p) return TRAPBEC_ERR_ARG;
  std::memset(p, 0, sizeof(*p));
  p->nx = p->ny = p->nz = 64;
  p->nprocx = p->nprocy = 1;
  p->precision = TRAPBEC_FP64;
  p->boundaries = TRAPBEC_BC_ZERO;
  p->periodicz = 0;
  p->two_dim = 0;
  p->potential = TRAPBEC_POT_HARMONIC;
  p->lbeam = 0;
  p->winding_number = 1;
  p->lx = p->ly = p->lz = 32.0;
  p->dt_re = 0.005;
  p->dt_im = 0.0;
  p->gamma = 0.0;
  p->potential_off = HUGE_REAL;
  p->wbeam = 4.0;
  p->t_spindown = HUGE_REAL;
  p->ring_rad = 10.0;
  p->vor_ring_count = 1;
  return TRAPBEC_OK;
}

int trapbec_params_parse(const char* text, trapbec_params* p, char* errbuf, size_t errlen) {
  if (!text || !p) return TRAPBEC_ERR_ARG;
  return tbh::parse_cparam_text(text, p, nullptr, errbuf, errlen);
}

// var_print / the restart writer for a state already in host memory
// (output.f90:64-75,102-108): the files trapbec_write_var and
// trapbec_write_restart write for the context's state.
int trapbec_write_var_host(const trapbec_params* p, const char* datadir, int itime, int shots, double t,
                           int imaginary, const void* psi) {
  if (!p || !datadir || !psi || shots <= 0) return TRAPBEC_ERR_ARG;
  const size_t bytes = (size_t)p->nx * p->ny * p->nz * (p->precision == TRAPBEC_FP64 ? 16 : 8);
  char name[64];
  // output.f90:65,75: "./data/proc%03d/var%04d.dat" with itime/shots
  std::snprintf(name, sizeof(name), "/proc%03d/%s%04d.dat", 0, imaginary ? "imag_var" : "var", itime / shots);
  return tbh::write_var_file(std::string(datadir) + name, p, t, psi, bytes);
}

int trapbec_write_restart_host(const trapbec_params* p, const char* datadir, int itime, double t, const void* psi) {
  if (!p || !datadir || !psi) return TRAPBEC_ERR_ARG;
  const size_t bytes = (size_t)p->nx * p->ny * p->nz * (p->precision == TRAPBEC_FP64 ? 16 : 8);
  return tbh::write_restart_file(std::string(datadir) + "/proc000/var.dat", p, itime, t, psi, bytes);
}

int trapbec_write_dims(const trapbec_params* p, const char* datadir) {  // output.f90:48-60
  if (!p || !datadir) return TRAPBEC_ERR_ARG;
  std::string d(datadir);
  if (!tbh::mkdirs(d)) { tbh::set_error("cannot create " + d); return TRAPBEC_ERR_IO; }
  FILE* f = std::fopen((d + "/dims.log").c_str(), "w");
  if (!f) { tbh::set_error("cannot open dims.log"); return TRAPBEC_ERR_IO; }
  int px = p->nprocx > 0 ? p->nprocx : 1, py = p->nprocy > 0 ? p->nprocy : 1;
  int v[8] = {p->nx, p->ny, p->nz, px, py, p->nx / px, p->ny / py, p->nz};
  for (int i = 0; i < 8; ++i) std::fprintf(f, "%12d\n", v[i]);
  std::fclose(f);
  return TRAPBEC_OK;
}

int trapbec_write_timing(const trapbec_params* p, const char* datadir, double tpt, double comm) {
  if (!p || !datadir) return TRAPBEC_ERR_ARG;  // output.f90:111-118
  std::string d(datadir);
  if (!tbh::mkdirs(d)) { tbh::set_error("cannot create " + d); return TRAPBEC_ERR_IO; }
  FILE* f = std::fopen((d + "/timing.log").c_str(), "w");
  if (!f) { tbh::set_error("cannot open timing.log"); return TRAPBEC_ERR_IO; }
  int px = p->nprocx > 0 ? p->nprocx : 1, py = p->nprocy > 0 ? p->nprocy : 1;
  std::fprintf(f, " %12lld%12d %16.8E\n", (long long)p->nx * p->ny * p->nz, px * py, tpt);
  std::fprintf(f, " ---------communication timing-----------\n");
  std::fprintf(f, " %16.8E\n", comm);
  std::fclose(f);
  return TRAPBEC_OK;
}

}  // extern "C"
