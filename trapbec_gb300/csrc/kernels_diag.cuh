// kernels_diag.cuh -- output-time diagnostics of the reference.
//
// get_phase (diagnostic.f90:27-48): the phase atan2(Im psi, Re psi) over the
// ghosted array, then its 6th-order first derivative along x, y, z (no phase
// unwrapping, as in the reference).  get_qpressure (diagnostic.f90:50-84): the
// density |psi| over the ghosted array, its 4th-order Laplacian on indices
// 0..n+1, then the 2nd-order gradient of that at interior points.  The ghosted
// array is what ghost_comm leaves: face ghosts by the boundary rule, edge and
// corner ghosts (two or three coordinates outside) zero, because ghost_comm
// never writes them and mesh_init set them to zero.  "Edge" is meant per
// rank: with nprocx x nprocy ranks a cell next to a rank corner reads zeros
// where a single domain would read its neighbours, and the kernels reproduce
// that from the rank extents nmx = nx/nprocx, nmy = ny/nprocy (z is never
// split, mpi_var.f90:156).
#pragma once
#include "common.cuh"

namespace tb {

template <typename T> struct DiagFieldArgs {
  const c_t<T>* psi;
  T* out;            // [3][n] (component-major)
  int nx, ny, nz;
  int nmx, nmy;      // rank extents
  int bc, bcz;       // boundary rule of x/y and of z
  T hx, hy, hz;
};

// Interior index range [li, li + nmx) x [lj, lj + nmy) of the rank owning a cell.
struct RankBox { int li, lj; };
template <typename T> __device__ __forceinline__ RankBox rank_box(const DiagFieldArgs<T>& a, int i, int j) {
  return RankBox{i / a.nmx * a.nmx, j / a.nmy * a.nmy};
}

// Psi of the owning rank's ghosted array at global 0-based indices (ghosts allowed).
template <typename T>
__device__ __forceinline__ c_t<T> ghosted(const DiagFieldArgs<T>& a, RankBox rb, int i, int j, int k) {
  const int oi = (i < rb.li || i >= rb.li + a.nmx), oj = (j < rb.lj || j >= rb.lj + a.nmy);
  const int ok = (k < 0 || k >= a.nz);
  if (oi + oj + ok > 1) return mk<T>((T)0, (T)0);   // edge / corner ghost: never written
  const int ii = map_ghost(i, a.nx, a.bc), jj = map_ghost(j, a.ny, a.bc), kk = map_ghost(k, a.nz, a.bcz);
  // zero-rule ghosts map to -1; tiny extents (nz = 1 in 2D runs) can map
  // past the far end: both read as zero instead of leaving the array
  if ((ii | jj | kk) < 0 || ii >= a.nx || jj >= a.ny || kk >= a.nz) return mk<T>((T)0, (T)0);
  return a.psi[((size_t)ii * a.ny + jj) * a.nz + kk];
}

template <typename T>
__device__ __forceinline__ T phase_at(const DiagFieldArgs<T>& a, RankBox rb, int i, int j, int k) {
  const c_t<T> v = ghosted(a, rb, i, j, k);
  return atan2(v.y, v.x);
}
template <typename T>
__device__ __forceinline__ T dens_at(const DiagFieldArgs<T>& a, RankBox rb, int i, int j, int k) {
  const c_t<T> v = ghosted(a, rb, i, j, k);
  return hypot(v.x, v.y);
}

// real first_deriv (deriv.f90:5-11)
template <typename T> __device__ __forceinline__ T d1r(T m3, T m2, T m1, T p1, T p2, T p3, T h) {
  return (-m3 + (T)9 * m2 - (T)45 * m1 + (T)45 * p1 - (T)9 * p2 + p3) / ((T)60 * h);
}
// real_second_deriv, 4th order (deriv.f90:26-32)
template <typename T> __device__ __forceinline__ T d2r4(T m2, T m1, T c, T p1, T p2, T h) {
  return (-m2 + (T)16 * m1 - (T)30 * c + (T)16 * p1 - p2) / ((T)12 * (h * h));
}

template <typename T>
__global__ void velocity_kernel(DiagFieldArgs<T> a) {
  const size_t n = (size_t)a.nx * a.ny * a.nz;
  for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += (size_t)gridDim.x * blockDim.x) {
    const int k = (int)(idx % a.nz);
    const size_t r = idx / a.nz;
    const int j = (int)(r % a.ny), i = (int)(r / a.ny);
    const RankBox b = rank_box(a, i, j);
    a.out[idx] = d1r(phase_at(a, b, i - 3, j, k), phase_at(a, b, i - 2, j, k), phase_at(a, b, i - 1, j, k),
                     phase_at(a, b, i + 1, j, k), phase_at(a, b, i + 2, j, k), phase_at(a, b, i + 3, j, k), a.hx);
    a.out[n + idx] = d1r(phase_at(a, b, i, j - 3, k), phase_at(a, b, i, j - 2, k), phase_at(a, b, i, j - 1, k),
                         phase_at(a, b, i, j + 1, k), phase_at(a, b, i, j + 2, k), phase_at(a, b, i, j + 3, k), a.hy);
    a.out[2 * n + idx] = d1r(phase_at(a, b, i, j, k - 3), phase_at(a, b, i, j, k - 2), phase_at(a, b, i, j, k - 1),
                             phase_at(a, b, i, j, k + 1), phase_at(a, b, i, j, k + 2), phase_at(a, b, i, j, k + 3), a.hz);
  }
}

// laplace_rho at a point of the owning rank's index range 0..n+1
template <typename T>
__device__ __forceinline__ T lap_rho(const DiagFieldArgs<T>& a, RankBox b, int i, int j, int k) {
  const T c = dens_at(a, b, i, j, k);
  T v = d2r4(dens_at(a, b, i - 2, j, k), dens_at(a, b, i - 1, j, k), c, dens_at(a, b, i + 1, j, k),
             dens_at(a, b, i + 2, j, k), a.hx);
  v = v + d2r4(dens_at(a, b, i, j - 2, k), dens_at(a, b, i, j - 1, k), c, dens_at(a, b, i, j + 1, k),
               dens_at(a, b, i, j + 2, k), a.hy);
  v = v + d2r4(dens_at(a, b, i, j, k - 2), dens_at(a, b, i, j, k - 1), c, dens_at(a, b, i, j, k + 1),
               dens_at(a, b, i, j, k + 2), a.hz);
  return v;
}

template <typename T>
__global__ void qpressure_kernel(DiagFieldArgs<T> a) {
  const size_t n = (size_t)a.nx * a.ny * a.nz;
  for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += (size_t)gridDim.x * blockDim.x) {
    const int k = (int)(idx % a.nz);
    const size_t r = idx / a.nz;
    const int j = (int)(r % a.ny), i = (int)(r / a.ny);
    const RankBox b = rank_box(a, i, j);
    // low_first_deriv (deriv.f90:33-39) of laplace_rho
    a.out[idx] = (-lap_rho(a, b, i - 1, j, k) + lap_rho(a, b, i + 1, j, k)) / ((T)2 * a.hx);
    a.out[n + idx] = (-lap_rho(a, b, i, j - 1, k) + lap_rho(a, b, i, j + 1, k)) / ((T)2 * a.hy);
    a.out[2 * n + idx] = (-lap_rho(a, b, i, j, k - 1) + lap_rho(a, b, i, j, k + 1)) / ((T)2 * a.hz);
  }
}

}  // namespace tb
