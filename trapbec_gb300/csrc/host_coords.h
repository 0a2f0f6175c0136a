// host_coords.h -- host-side coordinate and potential tables shared by the
// single-grid context and the batched solver.
#pragma once
#include <vector>

#include "../../include/trapbec.h"

namespace tbh {

// Coordinates as the reference computes them on an nprocx x nprocy grid
// (initial.f90:34-42), in the reference precision.
template <typename T>
inline void make_coords(const trapbec_params& p, std::vector<T>& xx, std::vector<T>& yy, std::vector<T>& zz) {
  int px = p.nprocx > 0 ? p.nprocx : 1, py = p.nprocy > 0 ? p.nprocy : 1;
  int nmx = p.nx / px, nmy = p.ny / py, nmz = p.nz;
  T Lx = (T)p.lx, Ly = (T)p.ly, Lz = (T)p.lz;
  xx.resize(p.nx); yy.resize(p.ny); zz.resize(p.nz);
  for (int k = 1; k <= nmz; ++k) zz[k - 1] = (T)(2 * k - 1) / ((T)2 * (T)nmz) * Lz - Lz / (T)2;
  for (int cy = 0; cy < py; ++cy)
    for (int j = 1; j <= nmy; ++j)
      yy[cy * nmy + j - 1] = (T)(2 * j - 1) / ((T)2 * (T)nmy) * Ly / (T)py + (T)cy * Ly / (T)py - Ly / (T)2;
  for (int cx = 0; cx < px; ++cx)
    for (int i = 1; i <= nmx; ++i)
      xx[cx * nmx + i - 1] = (T)(2 * i - 1) / ((T)2 * (T)nmx) * Lx / (T)px + (T)cx * Lx / (T)px - Lx / (T)2;
}


// Separable harmonic potential tables, finite_diff.f90:34:
// harm_wx*((xx(i))/Lx)**2 + harm_wy*... + harm_wz*...
template <typename T>
inline void make_harm_tables(const trapbec_params& p, const std::vector<T>& xx, const std::vector<T>& yy,
                             const std::vector<T>& zz, std::vector<T>& px, std::vector<T>& py, std::vector<T>& pz) {
  const T Lx = (T)p.lx, Ly = (T)p.ly, Lz = (T)p.lz;
  px.resize(p.nx); py.resize(p.ny); pz.resize(p.nz);
  for (int i = 0; i < p.nx; ++i) { T a = xx[i] / Lx; px[i] = (T)p.harm_wx * (a * a); }
  for (int j = 0; j < p.ny; ++j) { T a = yy[j] / Ly; py[j] = (T)p.harm_wy * (a * a); }
  for (int k = 0; k < p.nz; ++k) { T a = zz[k] / Lz; pz[k] = (T)p.harm_wz * (a * a); }
}

}  // namespace tbh
