// imag_ctrl.cuh -- finaliser kernels of the on-device imaginary-time loop.
//
// The imaginary-time relaxation (new; the reference only has the forward
// Euler step of run.f90:19-35) runs as: stage 1 (+ energy reduction of the
// incoming renormalised state) -> imag_fin_energy -> stage 2 -> stage 3
// (+ norm reduction of the new state) -> imag_fin_norm.  The finalisers run
// as one block, reduce the block partials in a fixed order (bitwise
// reproducible), and update the control block in FP64.
#pragma once
#include "common.cuh"
#include "kernels_simple.cuh"

namespace tb {

__device__ __forceinline__ void imag_energy_update(const double* r, ImagCtrl* c) {
  const double dV = c->dV;
  const double E = dV * (-0.5 * r[1] + 0.5 * r[2] + 0.25 * r[3] - 0.5 * r[4]);
  const double mu = (-0.5 * r[1] + 0.5 * r[2] + 0.5 * r[3] - 0.5 * r[4]) / r[0];
  if (!isfinite(E) || r[8] != 0.0) { c->nonfinite = 1; return; }
  if (c->n0 <= 0.0) c->n0 = dV * r[0];   // norm target unset: keep the initial norm
  if (c->have_prev) {
    const double rel = fabs(E - c->e_prev) / fabs(E);
    c->rel = rel;
    if (rel <= c->tol) c->converged = 1;
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
