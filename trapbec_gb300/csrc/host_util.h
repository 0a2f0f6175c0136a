// host_util.h -- host-side helpers shared by the translation units of libtrapbec.
#pragma once
#include <stdint.h>
#include <string>
#include <utility>
#include <vector>

#include "../../include/trapbec.h"

namespace tbh {

void set_error(const std::string& msg);
const char* get_error();

// Seeded sequence for the host-side random draws of the initial states
// (replaces Fortran's random_number seeded from the clock, mpi_var.f90:183-209).
struct Rng {
  uint64_t s;
  static uint64_t mix(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
  }
  double next() {
    s += 0x9e3779b97f4a7c15ULL;
    return (double)(mix(s) >> 11) * (1.0 / 9007199254740992.0);
  }
};

int parse_cparam_text(const char* text, trapbec_params* p,
                      std::vector<std::pair<std::string, std::string>>* rest, char* errbuf, size_t errlen);
bool mkdirs(const std::string& d);
int write_field_file(const std::string& path, const void* data, size_t bytes);
int write_var_file(const std::string& path, const trapbec_params* p, double t, const void* psi,
                   size_t psi_bytes);
int write_restart_file(const std::string& path, const trapbec_params* p, int itime, double t,
                       const void* psi, size_t psi_bytes);
int read_restart_file(const std::string& path, const trapbec_params* p, int* itime, double* t,
                      void* psi, size_t psi_bytes);

}  // namespace tbh
