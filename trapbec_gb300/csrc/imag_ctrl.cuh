// imag_ctrl.cuh -- finaliser kernels of the on-device imaginary-time loop.
//
// The imaginary-time relaxation (new; the reference only has the forward
// Euler step of run.f90:19-35) runs as: stage 1 (+ energy reduction of the
// incoming renormalised state) -> imag_fin_energy -> stage 2 -> stage 3
// (+ norm reduction of the new state) -> imag_fin_norm.  The finalisers run
// as one block, reduce the block partials in a fixed order (bitwise
// reproducible), and update the control block in FP64.  The stop test is on
// the energy change of consecutive states: relative, |E_n - E_{n-1}| <=
// tol |E_n|, or absolute in the caller's energy unit, |E_n - E_{n-1}| *
// escale < tol, or absolute per unit norm, |E_n - E_{n-1}| / N0 * escale <
// tol (ImagCtrl::stop_mode 0, 1, 2).
#pragma once
#include "common.cuh"
#include "kernels_simple.cuh"

namespace tb {

// Energy and mu of the incoming renormalised state, taken at exactly the
// target norm n0: the state was scaled in its own precision, so its norm
// misses n0 by that rounding (about 1e-10 relative for FP32 grids of 1e5-1e6
// cells), and the energy would carry the same noise into the convergence
// test.  The sums separate the quadratic terms (kinetic, potential,
// rotation) from the quartic one, so E(kappa psi) = kappa^2 Q + kappa^4 q4
// with kappa^2 = n0 / N is exact in FP64.
__device__ __forceinline__ void imag_energy_update(const double* r, ImagCtrl* c) {
  const double dV = c->dV;
  if (r[8] != 0.0 || !(r[0] > 0.0)) { c->nonfinite = 1; return; }
  if (c->n0 <= 0.0) c->n0 = dV * r[0];   // norm target unset: keep the initial norm
  const double k2 = c->n0 / (dV * r[0]);
  const double Q = -0.5 * r[1] + 0.5 * r[2] - 0.5 * r[4];
  const double E = dV * (k2 * Q + k2 * k2 * 0.25 * r[3]);
  const double mu = (Q + k2 * 0.5 * r[3]) / r[0];
  if (!isfinite(E)) { c->nonfinite = 1; return; }
  if (c->have_prev) {
    // relative test |dE|/|E| <= tol, or the absolute |dE| * escale < tol
    // (per unit norm: |dE| / n0 * escale < tol)
    const double dE = fabs(E - c->e_prev);
    const double rel = c->stop_mode == 0 ? dE / fabs(E) : (c->stop_mode == 2 ? dE / c->n0 : dE) * c->escale;
    c->rel = rel;
    if (c->stop_mode == 0 ? rel <= c->tol : rel < c->tol) c->converged = 1;
  }
  c->e_prev = E;
  c->have_prev = 1;
  c->energy = E;
  c->mu = mu;
}

__device__ __forceinline__ void imag_norm_update(const double* r, ImagCtrl* c) {
  const double N = c->dV * r[0];
  c->norm = N;
  if (!(N > 0.0) || !isfinite(N)) { c->nonfinite = 1; return; }
  c->scale = sqrt(c->n0 / N);
  c->step += 1;
}

static __global__ void __launch_bounds__(FIN_THREADS) imag_fin_energy_kernel(const double* __restrict__ red, int nblk,
                                                                      ImagCtrl* ctrl) {
  if (ctrl->converged || ctrl->nonfinite) return;
  __shared__ double out[NRED];
  finalize_partials(red, nblk, out);
  if (threadIdx.x == 0) imag_energy_update(out, ctrl);
}

static __global__ void __launch_bounds__(FIN_THREADS) imag_fin_norm_kernel(const double* __restrict__ red, int nblk,
                                                                    ImagCtrl* ctrl) {
  if (ctrl->converged || ctrl->nonfinite) return;
  __shared__ double out[NRED];
  finalize_partials(red, nblk, out);
  if (threadIdx.x == 0) imag_norm_update(out, ctrl);
}

}  // namespace tb
