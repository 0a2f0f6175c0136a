// common.cuh -- shared device-side definitions of the TrapBEC GB300 engine.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/trapbec.h"

namespace tb {

template <typename T> struct cplx;
template <> struct cplx<float> { using type = float2; };
template <> struct cplx<double> { using type = double2; };
template <typename T> using c_t = typename cplx<T>::type;

template <typename T> __host__ __device__ inline c_t<T> mk(T a, T b) { c_t<T> r; r.x = a; r.y = b; return r; }

// Potential evaluation modes inside the stage kernels.  Every reference
// potential other than the separable 'harmonic' one (and the laser) is
// evaluated by fill_potential_kernel into the Trap array and read as ARRAY.
enum PotMode : int { POT_NONE = 0, POT_HARM = 1, POT_ARR = 2 };
// Frame term of get_rhs (finite_diff.f90:126-131).
enum FrameMode : int { FRAME_NONE = 0, FRAME_ROT = 1, FRAME_ADV = 2 };
// Which parts of the 2N-storage update a stage performs.
//   S1: w = c*rhs,            psi' = psi + B*w, w stored     (run.f90:46-48)
//   S2: w = A*w + c*rhs,      psi' = psi + B*w, w stored     (run.f90:49-51)
//   S3: w = A*w + c*rhs,      psi' = psi + B*w, w not stored (run.f90:52-54)
//   EU: psi' = psi + c*rhs,   no w                           (run.f90:22)
//   DIAG: no update, no writes; reductions of the energy set only
// The deferred real-time form (tiled FP32 kernel, plain stages) splits the
// psi' = psi + B1*w1 of S1 into the next stage, which forms it on the fly:
//   S1W: w1 = c*rhs(psi0), only w1 stored
//   S2D: psi1 = psi0 + B1*w1 (same FMA as S1), then S2 from psi1; w2 goes to
//        a second w buffer because w1 is read with its ghost frame
// The psi-difference real-time form (tiled kernel, plain stages) stores no w
// at all: the two psi arrays hold the last two stage values, and a stage
// recovers the w of the stage before it from their difference,
// w_prev = (psi_k - psi_{k-1}) / B_prev (exact in exact arithmetic since
// psi_k = psi_{k-1} + B_prev*w_prev):
//   S1P: w1 = c*rhs(psi0), psi1 = psi0 + B1*w1, only psi1 stored
//   S2P: w2 = A2*w1 + c*rhs(psi1) with w1 = 3*(psi1 - psi0), psi2 = psi1 + B2*w2
//        stored over psi0 (each cell is read and written by one thread)
//   S3P: w3 = A3*w2 + c*rhs(psi2) with w2 = (psi2 - psi1)/B2, psi3 = psi2 + B3*w3
//        stored over psi1
enum StageKind : int {
  ST_S1 = 0, ST_S2 = 1, ST_S3 = 2, ST_EU = 3, ST_DIAG = 4, ST_S1W = 5, ST_S2D = 6,
  ST_S1P = 7, ST_S2P = 8, ST_S3P = 9
};

// Number of FP64 quantities a stage kernel may reduce (fused reductions).
//   0: sum|psi|^2  1: sum Re psi* lap  2: sum pot|psi|^2  3: sum |psi|^4
//   4: sum Re psi* frame  5: sum |psi|  6: max|psi|  7: min|psi|  8: nonfinite
constexpr int NRED = 9;

// Control block of the on-device imaginary-time loop (one per context or
// per batch instance).  Written by the finaliser kernels, read by the stage
// kernels, copied to the host every few steps.
struct ImagCtrl {
  double scale;     // pending renormalisation factor, applied on the next load
  double e_prev;    // energy of the previous state
  double rel;       // last |dE|/|E|
  double energy;    // energy of the last evaluated state
  double mu;        // chemical potential of the last evaluated state
  double norm;      // norm of the last state before renormalisation
  double n0;        // norm target
  double tol;       // convergence tolerance
  double dV;        // cell volume
  double escale;    // stop_mode 1: |dE| * escale < tol; 2: |dE| / n0 * escale < tol
                    // (escale converts the reference-unit energy, or energy per norm, into the caller's unit)
  int have_prev;    // e_prev is valid
  int converged;    // |dE|/|E| <= tol reached (stages become no-ops)
  int step;         // completed steps in the current call
  int nonfinite;    // a norm or energy was NaN/Inf
  int stop_mode;    // trapbec_imag_stop: 0 |dE|/|E| <= tol, 1 absolute, 2 absolute per unit norm
};

template <typename T> struct StageArgs {
  const c_t<T>* __restrict__ psi_in;
  c_t<T>* __restrict__ psi_out;
  c_t<T>* __restrict__ w;
  const T* __restrict__ xx;   // coordinates (initial.f90:34-42), length nx/ny/nz
  const T* __restrict__ yy;
  const T* __restrict__ zz;
  const T* __restrict__ px;   // harm_wx*(xx/Lx)^2 etc. (finite_diff.f90:34)
  const T* __restrict__ py;
  const T* __restrict__ pz;
  const T* __restrict__ trap; // full potential array (POT_ARR)
  double* __restrict__ red;   // per-block partials [NRED][nblocks] (may be null)
  int nx, ny, nz;
  int bc;                     // trapbec_boundaries for x and y
  int zper;                   // z periodic (periodicz or 'periodic')
  int two_dim;
  int pot_mode, frame_mode;
  int reduce;                 // 0 none, 1 = norm only (sum|psi|^2), 2 = energy set
  T ix2, iy2, iz2;            // 1/(180 h^2) per axis
  T ix1, iy1;                 // 1/(60 h)
  T c_re, c_im;               // rhs multiplier of the update
  T A, B;                     // 2N-storage coefficients of this stage
  T omega;                    // omega_z (FRAME_ROT) or 2*advective_vx (FRAME_ADV)
  T scale;                    // factor applied to psi_in on load (renormalisation)
  ImagCtrl* ctrl;             // imaginary-time control block (may be null)
  int use_ctrl_scale;         // take the load factor from ctrl->scale
  const c_t<T>* __restrict__ w_in;  // S2D: w1 (ghost fix-ups read it); w receives w2
  T B1;                       // S2D: B of stage 1 (psi1 = psi0 + B1*w1)
  T rB;                       // S2P / S3P: 1/B of the previous stage (w_prev = rB*(psi - psi_prev));
                              // w_in then points at the previous psi array
  c_t<T>* __restrict__ lo;    // compensated state: rounding remainder of psi, read and rewritten in place
};

// Stage prologue: a converged imaginary-time loop turns stages into no-ops;
// otherwise returns the load factor.
template <typename T>
__device__ __forceinline__ bool stage_skip(const StageArgs<T>& a, T* scale) {
  if (a.ctrl != nullptr) {
    const volatile ImagCtrl* c = a.ctrl;
    if (c->converged || c->nonfinite) return true;
    if (a.use_ctrl_scale) { *scale = (T)c->scale; return false; }
  }
  *scale = a.scale;
  return false;
}

// Ghost index mapping for a non-periodic / periodic axis of length n
// (ghost.f90:53-60 'zero', 'solid', periodic wrap).  Returns -1 for a zero ghost.
__device__ __forceinline__ int map_ghost(int q, int n, int bc) {
  if (q >= 0 && q < n) return q;
  if (bc == TRAPBEC_BC_PERIODIC) return q < 0 ? q + n : q - n;
  if (bc == TRAPBEC_BC_SOLID) return q < 0 ? -q : 2 * (n - 1) - q;
  return -1;
}

// D2 of a 7-point line without the 1/(180 h^2) factor (deriv.f90:19-25):
// 2(v-3+v3) - 27(v-2+v2) + 270(v-1+v1) - 490 v0, written symmetrically.
template <typename T>
__device__ __forceinline__ c_t<T> d2raw(c_t<T> m3, c_t<T> m2, c_t<T> m1, c_t<T> c0, c_t<T> p1,
                                        c_t<T> p2, c_t<T> p3) {
  c_t<T> r;
  r.x = (T)2 * (m3.x + p3.x) - (T)27 * (m2.x + p2.x) + (T)270 * (m1.x + p1.x) - (T)490 * c0.x;
  r.y = (T)2 * (m3.y + p3.y) - (T)27 * (m2.y + p2.y) + (T)270 * (m1.y + p1.y) - (T)490 * c0.y;
  return r;
}
// The same D2 in difference form, 2 ((v-3-c)+(v3-c)) - 27 (...) + 270 (...):
// equal in exact arithmetic, but the neighbour differences of a resolved
// field are (nearly) exact in floating point, so its rounding scales with the
// result instead of with 490 |c|.  Used for FP32 diagnostics only.
template <typename T>
__device__ __forceinline__ c_t<T> d2diff(c_t<T> m3, c_t<T> m2, c_t<T> m1, c_t<T> c0, c_t<T> p1,
                                         c_t<T> p2, c_t<T> p3) {
  c_t<T> r;
  r.x = (T)2 * ((m3.x - c0.x) + (p3.x - c0.x)) - (T)27 * ((m2.x - c0.x) + (p2.x - c0.x)) +
        (T)270 * ((m1.x - c0.x) + (p1.x - c0.x));
  r.y = (T)2 * ((m3.y - c0.y) + (p3.y - c0.y)) - (T)27 * ((m2.y - c0.y) + (p2.y - c0.y)) +
        (T)270 * ((m1.y - c0.y) + (p1.y - c0.y));
  return r;
}
// D1 without the 1/(60 h) factor (deriv.f90:12-18): (v3-v-3) - 9(v2-v-2) + 45(v1-v-1).
template <typename T>
__device__ __forceinline__ c_t<T> d1raw(c_t<T> m3, c_t<T> m2, c_t<T> m1, c_t<T> p1, c_t<T> p2,
                                        c_t<T> p3) {
  c_t<T> r;
  r.x = (p3.x - m3.x) - (T)9 * (p2.x - m2.x) + (T)45 * (p1.x - m1.x);
  r.y = (p3.y - m3.y) - (T)9 * (p2.y - m2.y) + (T)45 * (p1.y - m1.y);
  return r;
}

// Everything a cell needs after its stencil lines are assembled: the rhs of
// get_rhs (finite_diff.f90:23-132) and the stage update (run.f90:46-54).
// lap: Laplacian (scaled), fr: frame term (already multiplied by i*omega),
// c: psi at the cell (scaled), pot: potential, wold: w before the stage.
template <typename T, int KIND>
__device__ __forceinline__ void cell_update(c_t<T> c, c_t<T> lap, c_t<T> fr, T pot, c_t<T> wold,
                                            const StageArgs<T>& a, c_t<T>& wnew, c_t<T>& pnew) {
  T a2 = c.x * c.x + c.y * c.y;
  T rho = (T)1 - a2 - pot;
  c_t<T> rhs;
  rhs.x = lap.x + fr.x + rho * c.x;
  rhs.y = lap.y + fr.y + rho * c.y;
  c_t<T> cr;
  cr.x = a.c_re * rhs.x - a.c_im * rhs.y;
  cr.y = a.c_re * rhs.y + a.c_im * rhs.x;
  if (KIND == ST_EU) {
    pnew.x = c.x + cr.x;
    pnew.y = c.y + cr.y;
    wnew = cr;
  } else {
    if (KIND == ST_S1) {
      wnew = cr;
    } else {
      wnew.x = a.A * wold.x + cr.x;
      wnew.y = a.A * wold.y + cr.y;
    }
    pnew.x = c.x + a.B * wnew.x;
    pnew.y = c.y + a.B * wnew.y;
  }
}

// Neumaier-compensated FP64 accumulator.
struct Acc {
  double s, c;
  __device__ __forceinline__ void init() { s = 0.0; c = 0.0; }
  __device__ __forceinline__ void add(double v) {
    double t = s + v;
    if (fabs(s) >= fabs(v)) c += (s - t) + v; else c += (v - t) + s;
    s = t;
  }
  __device__ __forceinline__ double val() const { return s + c; }
};

}  // namespace tb
