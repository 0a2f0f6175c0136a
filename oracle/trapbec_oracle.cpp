// trapbec_oracle.cpp -- CPU restatement of TrapBEC's time-stepping hot path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the checker: tests, the smoke check
// and the CPU-baseline leg of the benchmark call it to produce the answers the
// CUDA path must reproduce.  Nothing in the shipped library links, loads or
// calls it.
//
// Parity status: the reference is Fortran 90 + MPI and no Fortran compiler or
// MPI exists in the build or GPU images, so the reference binary cannot be run
// and the reference ships no golden vectors.  The reference's own source is
// run instead, by the Fortran-subset interpreter oracle/fortran_subset.py
// (gfortran -O3 x86-64 semantics, no FP contraction): the golden vectors it
// produced (tests/golden/refsrc_cases.*, generator
// tests/golden/make_refsrc_fixtures.py) are reproduced by this restatement
// bit for bit for the time stepping in FP64 and FP32, on 1 rank and a 2 x 2
// process grid (tests/test_refsrc_golden.py).  Known-answer tests derived
// from mathematics (stencil exactness on polynomials, convergence order, the
// RK3 amplification polynomial, the Lz eigenvalue, norm conservation, the
// harmonic-oscillator ground state) check it as well.
//
// It follows the reference statement by statement, in the same evaluation
// order, with T = float for the shipped single-precision build and
// T = double for the -fdefault-real-8 build:
//   coordinates        initial.f90:26,34-42
//   ghost fill         ghost.f90:27-192 (local fills + the face exchange of
//                      an nprocx x nprocy process grid, done in-process)
//   stencils           deriv.f90:12-25
//   get_rhs            finite_diff.f90:8-136
//   RK3 / imag Euler   run.f90:19-57
//   Psi_info/Psi_norm  diagnostic.f90:7-25
//   initial states     initial.f90:58-157,202-870
// and adds the FP64 energy / chemical potential and the RK3 imaginary-time
// relaxation with renormalisation, which the reference does not have.
// Complex arithmetic is written out in real arithmetic so the operation order
// is explicit; operations gfortran lowers component-wise (complex * real,
// complex / real) are component-wise here too.  Build with -ffp-contract=off.

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#include <limits>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/trapbec.h"

namespace {

template <typename T> struct C {  // complex value, explicit arithmetic
  T re, im;
};
template <typename T> inline C<T> cadd(C<T> a, C<T> b) { return {a.re + b.re, a.im + b.im}; }
template <typename T> inline C<T> csub(C<T> a, C<T> b) { return {a.re - b.re, a.im - b.im}; }
template <typename T> inline C<T> cscale(T s, C<T> a) { return {s * a.re, s * a.im}; }
template <typename T> inline C<T> cdivr(C<T> a, T d) { return {a.re / d, a.im / d}; }
template <typename T> inline C<T> cmul(C<T> a, C<T> b) {
  return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
template <typename T> inline T cabs_(C<T> a) { return std::hypot(a.re, a.im); }

// ---------------------------------------------------------------- RNG ----
// Seeded replacement for the clock-seeded Fortran RNG (mpi_var.f90:183-209,
// statistics.f90:29-35).  splitmix64: host draws are a sequence, per-cell
// draws are a keyed hash of (seed, global cell index), so results do not
// depend on the decomposition.
inline uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
  return z ^ (z >> 31);
}
struct Rng {
  uint64_t s;
  double next() {  // U[0,1)
    s += 0x9e3779b97f4a7c15ULL;
    return (double)(mix64(s) >> 11) * (1.0 / 9007199254740992.0);
  }
};
inline double cell_uniform(uint64_t seed, uint64_t idx, uint64_t stream) {
  uint64_t h = mix64(seed ^ mix64(idx * 2ULL + stream + 0x632be59bd9b4e019ULL));
  return (double)(h >> 11) * (1.0 / 9007199254740992.0);
}

// --------------------------------------------------------- one "rank" ----
template <typename T> struct Rank {
  int cx, cy;                 // coords(1), coords(2)
  int nmx, nmy, nmz;          // nmeshx, nmeshy, nmeshz
  int left, right, top, bot;  // neighbour ranks, -1 = MPI_PROC_NULL
  std::vector<T> xx, yy, zz;  // 1-based storage: index 0 unused
  std::vector<C<T>> psi;      // (-2:nmz+3, -2:nmy+3, -2:nmx+3)
  std::vector<C<T>> rhs, w;   // (1:nmz, 1:nmy, 1:nmx)
  std::vector<C<T>> lo;       // (1:nmz, 1:nmy, 1:nmx): remainders of the compensated RK3 (new)
  std::vector<T> trap;        // (1:nmz, 1:nmy, 1:nmx)
  size_t gz, gy;              // ghosted extents in z and y
  inline size_t g(int k, int j, int i) const {  // Psi(k,j,i), ghosted
    return ((size_t)(i + 2) * gy + (size_t)(j + 2)) * gz + (size_t)(k + 2);
  }
  inline size_t in(int k, int j, int i) const {  // interior arrays, 1-based
    return ((size_t)(i - 1) * nmy + (size_t)(j - 1)) * nmz + (size_t)(k - 1);
  }
};

template <typename T> struct Oracle {
  trapbec_params p;
  int px, py;
  T Lx, Ly, Lz, hx, hy, hz;
  C<T> dt;      // current complex dt (run.f90:42 multiplies it once)
  T t;          // simulation time
  T pi;
  T eps;        // epsilon(0.)
  std::vector<Rank<T>> ranks;
  double norm_target = -1.0;
  bool norm_user = false;   // set by orc_set_norm_target; otherwise derived from each new state
  double e_prev = std::numeric_limits<double>::quiet_NaN();
  int imag_stop = 0;          // stop test: 0 relative |dE|/|E| <= tol; 1 absolute |dE| * escale < tol;
                              // 2 absolute per unit norm |dE| / N0 * escale < tol
  double imag_escale = 0.0;
  double intpsi2_old = 1.0;

  explicit Oracle(const trapbec_params& pp) : p(pp) {
    px = p.nprocx > 0 ? p.nprocx : 1;
    py = p.nprocy > 0 ? p.nprocy : 1;
    Lx = (T)p.lx; Ly = (T)p.ly; Lz = (T)p.lz;
    hx = Lx / (T)p.nx; hy = Ly / (T)p.ny; hz = Lz / (T)p.nz;   // initial.f90:26
    dt = {(T)p.dt_re, (T)p.dt_im};
    t = 0;
    pi = (T)3.14159265359;                                         // cdata.f90:13
    eps = std::numeric_limits<T>::epsilon();
    int nmx = p.nx / px, nmy = p.ny / py, nmz = p.nz;              // mpi_var.f90:156
    bool per = p.boundaries == TRAPBEC_BC_PERIODIC;
    ranks.resize((size_t)px * py);
    for (int r = 0; r < px * py; ++r) {
      Rank<T>& R = ranks[r];
      R.cx = r / py; R.cy = r % py;   // MPI_Cart_create row-major ordering
      R.nmx = nmx; R.nmy = nmy; R.nmz = nmz;
      auto rk = [&](int cx, int cy) -> int {
        if (per) { cx = (cx + px) % px; cy = (cy + py) % py; }
        if (cx < 0 || cx >= px || cy < 0 || cy >= py) return -1;
        return cx * py + cy;
      };
      R.left = rk(R.cx - 1, R.cy); R.right = rk(R.cx + 1, R.cy);
      R.top = rk(R.cx, R.cy - 1); R.bot = rk(R.cx, R.cy + 1);
      R.gz = (size_t)nmz + 6; R.gy = (size_t)nmy + 6;
      R.psi.assign(R.gz * R.gy * ((size_t)nmx + 6), C<T>{0, 0});
      R.rhs.assign((size_t)nmx * nmy * nmz, C<T>{0, 0});
      R.w.assign((size_t)nmx * nmy * nmz, C<T>{0, 0});
      R.lo.assign((size_t)nmx * nmy * nmz, C<T>{0, 0});
      R.trap.assign((size_t)nmx * nmy * nmz, (T)0);
      R.xx.assign(nmx + 1, 0); R.yy.assign(nmy + 1, 0); R.zz.assign(nmz + 1, 0);
      // initial.f90:34-42
      for (int k = 1; k <= nmz; ++k)
        R.zz[k] = (T)(2 * k - 1) / ((T)2 * (T)nmz) * Lz - Lz / (T)2;
      for (int j = 1; j <= nmy; ++j)
        R.yy[j] = (T)(2 * j - 1) / ((T)2 * (T)nmy) * Ly / (T)py + (T)R.cy * Ly / (T)py - Ly / (T)2;
      for (int i = 1; i <= nmx; ++i)
        R.xx[i] = (T)(2 * i - 1) / ((T)2 * (T)nmx) * Lx / (T)px + (T)R.cx * Lx / (T)px - Lx / (T)2;
    }
    if (p.potential == TRAPBEC_POT_MOBIUS) init_mobius_trap();
  }

  // initial.f90:159-198: mesh_init's Trap of the 'mobius' potential (a later
  // set_trap replaces it).  The strip table mobius(200,200,3), the per-cell
  // sum over it clamped at 3 after every term, the maximum over all ranks
  // (MPI_REDUCE MAX + BCAST) and Trap = theta - Trap.
  void init_mobius_trap() {
    const int N = 200;
    const T pi = (T)3.14159265359;   // cdata.f90:13
    std::vector<T> m1((size_t)N * N), m2((size_t)N * N), m3((size_t)N * N);
    for (int i = 1; i <= N; ++i)
      for (int j = 1; j <= N; ++j) {
        const T r = (T)(i - 1) * (T)2 / (T)200 - (T)1;
        const T theta = (T)(j - 1) * (T)2 * pi / (T)200;
        const size_t q = (size_t)(i - 1) + (size_t)(j - 1) * N;   // mobius(i,j,:)
        m1[q] = ((T)25 + (T)5 * r * std::cos(theta / (T)2)) * std::cos(theta);
        m2[q] = ((T)25 + (T)5 * r * std::cos(theta / (T)2)) * std::sin(theta);
        m3[q] = (T)5 * r * std::sin(theta / (T)2);
      }
    T theta = 0;
    bool first = true;
    for (auto& R : ranks) {
      T rmax = 0;
      bool rfirst = true;
#pragma omp parallel for schedule(static)
      for (int i = 1; i <= R.nmx; ++i)
        for (int j = 1; j <= R.nmy; ++j)
          for (int k = 1; k <= R.nmz; ++k) {
            T acc = 0;
            for (int ii1 = 1; ii1 <= N; ++ii1)
              for (int ii2 = 1; ii2 <= N; ++ii2) {
                const size_t q = (size_t)(ii1 - 1) + (size_t)(ii2 - 1) * N;
                const T dx = R.xx[i] - m1[q], dy = R.yy[j] - m2[q], dz = R.zz[k] - m3[q];
                T e = -((T)1.5 * (dx * dx));
                e = e - (T)1.5 * (dy * dy);
                e = e - (T)1.5 * (dz * dz);
                acc = acc + std::exp(e);
                if (acc > (T)3) acc = (T)3;
              }
            R.trap[R.in(k, j, i)] = acc;
          }
      for (int i = 1; i <= R.nmx; ++i)   // r=maxval(Trap)
        for (int j = 1; j <= R.nmy; ++j)
          for (int k = 1; k <= R.nmz; ++k) {
            const T v = R.trap[R.in(k, j, i)];
            if (rfirst || v > rmax) rmax = v;
            rfirst = false;
          }
      if (first || rmax > theta) theta = rmax;
      first = false;
    }
    for (auto& R : ranks)
      for (int i = 1; i <= R.nmx; ++i)
        for (int j = 1; j <= R.nmy; ++j)
          for (int k = 1; k <= R.nmz; ++k) R.trap[R.in(k, j, i)] = theta - R.trap[R.in(k, j, i)];
  }

  // global interior index (z fastest) <-> (rank, local)
  size_t gidx(int K, int J, int I) const {  // 0-based global
    return ((size_t)I * p.ny + J) * p.nz + K;
  }

  // ---------------------------------------------------------- ghost.f90 --
  void ghost_comm() {
    // Face exchange of the process grid, then the boundary fills where a
    // side has no neighbour.  x faces first, then y faces, then z
    // (ghost.f90:29-94, 96-160, 163-191).  Corners are never read.
    for (auto& R : ranks) {
      int nmx = R.nmx, nmy = R.nmy, nmz = R.nmz;
      // ghost planes from the right neighbour (its first planes 1..3)
      if (R.right >= 0) {
        Rank<T>& N = ranks[R.right];
        for (int m = 1; m <= 3; ++m)
          for (int j = 1; j <= nmy; ++j)
            for (int k = 1; k <= nmz; ++k) R.psi[R.g(k, j, nmx + m)] = N.psi[N.g(k, j, m)];
      } else {
        for (int m = 1; m <= 3; ++m)
          for (int j = 1; j <= nmy; ++j)
            for (int k = 1; k <= nmz; ++k)
              R.psi[R.g(k, j, nmx + m)] = p.boundaries == TRAPBEC_BC_SOLID
                                              ? R.psi[R.g(k, j, nmx - m)] : C<T>{0, 0};
      }
      if (R.left >= 0) {
        Rank<T>& N = ranks[R.left];
        for (int m = 0; m <= 2; ++m)
          for (int j = 1; j <= nmy; ++j)
            for (int k = 1; k <= nmz; ++k) R.psi[R.g(k, j, -m)] = N.psi[N.g(k, j, N.nmx - m)];
      } else {
        for (int m = 0; m <= 2; ++m)
          for (int j = 1; j <= nmy; ++j)
            for (int k = 1; k <= nmz; ++k)
              R.psi[R.g(k, j, -m)] = p.boundaries == TRAPBEC_BC_SOLID
                                         ? R.psi[R.g(k, j, 2 + m)] : C<T>{0, 0};
      }
    }
    for (auto& R : ranks) {
      int nmx = R.nmx, nmy = R.nmy, nmz = R.nmz;
      if (R.bot >= 0) {
        Rank<T>& N = ranks[R.bot];
        for (int i = 1; i <= nmx; ++i)
          for (int m = 1; m <= 3; ++m)
            for (int k = 1; k <= nmz; ++k) R.psi[R.g(k, nmy + m, i)] = N.psi[N.g(k, m, i)];
      } else {
        for (int i = 1; i <= nmx; ++i)
          for (int m = 1; m <= 3; ++m)
            for (int k = 1; k <= nmz; ++k)
              R.psi[R.g(k, nmy + m, i)] = p.boundaries == TRAPBEC_BC_SOLID
                                              ? R.psi[R.g(k, nmy - m, i)] : C<T>{0, 0};
      }
      if (R.top >= 0) {
        Rank<T>& N = ranks[R.top];
        for (int i = 1; i <= nmx; ++i)
          for (int m = 0; m <= 2; ++m)
            for (int k = 1; k <= nmz; ++k) R.psi[R.g(k, -m, i)] = N.psi[N.g(k, N.nmy - m, i)];
      } else {
        for (int i = 1; i <= nmx; ++i)
          for (int m = 0; m <= 2; ++m)
            for (int k = 1; k <= nmz; ++k)
              R.psi[R.g(k, -m, i)] = p.boundaries == TRAPBEC_BC_SOLID
                                         ? R.psi[R.g(k, 2 + m, i)] : C<T>{0, 0};
      }
    }
    for (auto& R : ranks) {
      int nmx = R.nmx, nmy = R.nmy, nmz = R.nmz;
      bool zper = p.periodicz || p.boundaries == TRAPBEC_BC_PERIODIC;
      for (int i = 1; i <= nmx; ++i)
        for (int j = 1; j <= nmy; ++j)
          for (int m = 1; m <= 3; ++m) {
            C<T> hi, lo;
            if (zper) {
              hi = R.psi[R.g(m, j, i)];
              lo = R.psi[R.g(nmz + 1 - m, j, i)];
            } else if (p.boundaries == TRAPBEC_BC_SOLID) {
              hi = R.psi[R.g(nmz - m, j, i)];
              lo = R.psi[R.g(1 + m, j, i)];
            } else {
              hi = lo = C<T>{0, 0};
            }
            R.psi[R.g(nmz + m, j, i)] = hi;
            R.psi[R.g(1 - m, j, i)] = lo;
          }
    }
  }

  // ---------------------------------------------------------- deriv.f90 --
  static inline C<T> second_deriv_ref(const C<T>* v, ptrdiff_t s, T h) {  // deriv.f90:19-25
    C<T> a = cscale((T)2, v[-3 * s]);
    a = csub(a, cscale((T)27, v[-2 * s]));
    a = cadd(a, cscale((T)270, v[-1 * s]));
    a = csub(a, cscale((T)490, v[0]));
    a = cadd(a, cscale((T)270, v[1 * s]));
    a = csub(a, cscale((T)27, v[2 * s]));
    a = cadd(a, cscale((T)2, v[3 * s]));
    return cdivr(a, (T)180 * (h * h));
  }
  // The same D2 in difference form, 2((v-3 - c) + (v3 - c)) - 27(...) + 270(...),
  // the stencil of the compensated real-time form (new, no counterpart in the
  // reference): equal in exact arithmetic, smaller rounding for a resolved field.
  static inline C<T> second_deriv_diff(const C<T>* v, ptrdiff_t s, T h) {
    const C<T> c = v[0];
    C<T> a = cscale((T)2, cadd(csub(v[-3 * s], c), csub(v[3 * s], c)));
    a = csub(a, cscale((T)27, cadd(csub(v[-2 * s], c), csub(v[2 * s], c))));
    a = cadd(a, cscale((T)270, cadd(csub(v[-1 * s], c), csub(v[1 * s], c))));
    return cdivr(a, (T)180 * (h * h));
  }
  static inline C<T> first_deriv(const C<T>* v, ptrdiff_t s, T h) {  // deriv.f90:12-18
    C<T> a = {-v[-3 * s].re, -v[-3 * s].im};
    a = cadd(a, cscale((T)9, v[-2 * s]));
    a = csub(a, cscale((T)45, v[-1 * s]));
    a = cadd(a, cscale((T)45, v[1 * s]));
    a = csub(a, cscale((T)9, v[2 * s]));
    a = cadd(a, v[3 * s]);
    return cdivr(a, (T)60 * h);
  }

  // ------------------------------------------------ potential (per cell) --
  T potential(const Rank<T>& R, int k, int j, int i) const {  // finite_diff.f90:29-124
    const T x = R.xx[i], y = R.yy[j], z = R.zz[k];
    T pot = 0, r, r1, r2;
    switch (p.potential) {
      case TRAPBEC_POT_ZERO: break;
      case TRAPBEC_POT_HARMONIC: {
        T a = x / Lx, b = y / Ly, c = z / Lz;
        pot = (T)p.harm_wx * (a * a) + (T)p.harm_wy * (b * b) + (T)p.harm_wz * (c * c);
      } break;
      case TRAPBEC_POT_HARMONIC_RING: {
        T a = x / Lx, b = y / Lx;
        r = std::sqrt(a * a + b * b);
        T d = r - (T)0.3;
        pot = (T)p.harm_wx * (d * d);
        if (std::fabs(r - (T)0.3) < (T)0.01) pot = std::max((T)0, (T)5 - (T)0.1 * t);
      } break;
      case TRAPBEC_POT_HARMONIC_RING2: {
        T pw = 6;
        r1 = std::pow(std::fabs(std::pow((T)0.25, pw) - (T)0.15 * std::pow(x / Lx, pw) -
                                (T)4 * std::pow(y / Ly - (T)0.2, pw)), (T)1 / pw);
        r2 = std::pow(std::fabs(std::pow((T)0.25, pw) - (T)0.15 * std::pow(x / Lx, pw) -
                                (T)4 * std::pow(y / Ly + (T)0.2, pw)), (T)1 / pw);
        r1 = (r1 < (T)0.2495) ? (T)0 : (T)5;
        r2 = (r2 < (T)0.2495) ? (T)0 : (T)5;
        pot = r1 * r2;
        if (pot < (T)0) pot = 0;
        if (std::fabs(y / Ly) < (T)0.01 && pot < (T)0.01) pot = std::max((T)0, (T)5 - (T)0.1 * t);
      } break;
      case TRAPBEC_POT_BARRIER:
        pot = 0;
        if (std::fabs(y / Ly) > (T)0.3) pot = 5;
        if (std::fabs(y / Ly) < (T)0.01) pot = std::max((T)0, (T)5 - (T)0.1 * t);
        break;
      case TRAPBEC_POT_BOX_TRAP:
        pot = 10;
        r = std::sqrt(x * x + y * y);
        if (r < Lx / (T)3 && std::fabs(z) < Lz / (T)2.5) pot = 0;
        pot = pot + (T)5 * std::sin((T)0.1 * t) * z / Lz;
        break;
      case TRAPBEC_POT_CHANNEL:
        pot = 0;
        if (std::fabs(y) > (T)0.75 * Ly / (T)2 || std::fabs(z) > (T)0.75 * Lz / (T)2) pot = 5;
        for (int l1 = -1; l1 <= 1; ++l1)
          if (std::fabs(x) < Lx / (T)p.nx && std::fabs(y - (T)l1 * Ly / (T)5) < Ly / (T)p.ny) pot = (T)7.5;
        for (int l1 = -1; l1 <= 1; ++l1)
          if (std::fabs(x) < Lx / (T)p.nx && std::fabs(z - (T)l1 * Lz / (T)5) < Ly / (T)p.ny) pot = (T)7.5;
        break;
      case TRAPBEC_POT_QUARTIC: {
        T a = x / Lx, b = y / Ly;
        r = std::sqrt(a * a + b * b);
        T r2_ = r * r, r4 = r2_ * r2_;
        pot = (T)p.harm_wx * (r4 * r4);
      } break;
      case TRAPBEC_POT_SPHERE: {
        T theta = std::atan2(y, x);
        T a = x / Lx, b = y / Ly, c = z / Lz;
        r1 = std::sqrt(a * a + b * b + c * c);
        T phi = std::acos((z / Lz) / r1);
        pot = (r1 < (T)0.2 + (T)0.01 * std::sin((T)20 * phi) + (T)0.01 * std::cos((T)30 * theta + (T)0.03))
                  ? (T)10 : (T)0;
      } break;
      case TRAPBEC_POT_MOBIUS:
        pot = R.trap[R.in(k, j, i)];
        if (std::fabs(y) < (T)1 && std::fabs(x - (T)25) < (T)1) pot = pot + 10;
        break;
      case TRAPBEC_POT_ARRAY:
        pot = R.trap[R.in(k, j, i)];
        break;
    }
    if (p.lbeam) {  // finite_diff.f90:118-123, las_freq = 0
      T las_freq = 0;
      T las_x = (T)70 * std::cos(las_freq * t) * ((T)1 - std::sin(las_freq * t));
      T las_y = (T)30 * std::sin(las_freq * t) * std::cos(las_freq * t);
      T a = (x - las_x) / (T)p.wbeam, b = (y - las_y) / (T)p.wbeam;
      pot = pot + (T)20 * std::exp(-(a * a) - (b * b));
    }
    if (t > (T)p.potential_off) pot = 0;  // finite_diff.f90:124
    return pot;
  }

  // Rotation / advective term of get_rhs (finite_diff.f90:126-131), or zero.
  inline C<T> frame_term(const Rank<T>& R, const C<T>* c, ptrdiff_t sx, ptrdiff_t sy,
                         int j, int i, bool* active) const {
    *active = false;
    if (std::fabs((T)p.advective_vx) > eps) {
      *active = true;
      C<T> d = first_deriv(c, sx, hx);
      T s = (T)2 * (T)p.advective_vx;   // (2*eye*vx) = (0, 2vx)
      return {-s * d.im, s * d.re};
    } else if (std::fabs((T)p.omega_z) > eps && t < (T)p.t_spindown) {
      *active = true;
      C<T> dy = first_deriv(c, sy, hy), dx = first_deriv(c, sx, hx);
      C<T> zc = csub(cscale(R.xx[i], dy), cscale(R.yy[j], dx));
      T om = (T)p.omega_z;              // (omega_z*eye) = (0, omega)
      return {-om * zc.im, om * zc.re};
    }
    return {0, 0};
  }

  // --------------------------------------------------- finite_diff.f90 --
  bool diff_lap = false;   // get_rhs takes the difference-form D2 (compensated form)
  void get_rhs() {
    ghost_comm();
    const bool two = p.two_dim != 0;
    auto second_deriv = diff_lap ? &Oracle::second_deriv_diff : &Oracle::second_deriv_ref;
    for (auto& R : ranks) {
      const ptrdiff_t sx = (ptrdiff_t)(R.gz * R.gy), sy = (ptrdiff_t)R.gz;
#pragma omp parallel for schedule(static)
      for (int i = 1; i <= R.nmx; ++i)
        for (int j = 1; j <= R.nmy; ++j)
          for (int k = 1; k <= R.nmz; ++k) {
            const C<T>* c = &R.psi[R.g(k, j, i)];
            C<T> rhs = second_deriv(c, sx, hx);
            rhs = cadd(rhs, second_deriv(c, sy, hy));
            if (!two) rhs = cadd(rhs, second_deriv(c, 1, hz));
            T pot = potential(R, k, j, i);
            bool act;
            C<T> fr = frame_term(R, c, sx, sy, j, i, &act);
            if (act) rhs = cadd(rhs, fr);
            T rho = (T)1 - cabs_(cmul(*c, *c)) - pot;   // abs(Psi**2)
            rhs = cadd(rhs, cscale(rho, *c));
            R.rhs[R.in(k, j, i)] = rhs;
          }
    }
  }

  // ------------------------------------------------------------ run.f90 --
  template <typename F> void for_interior(F f) {
    for (auto& R : ranks) {
#pragma omp parallel for schedule(static)
      for (int i = 1; i <= R.nmx; ++i)
        for (int j = 1; j <= R.nmy; ++j)
          for (int k = 1; k <= R.nmz; ++k) f(R, k, j, i);
    }
  }

  void apply_damping() {  // run.f90:42, dt=dt*(1.-gamma*eye)
    C<T> f = {(T)1, -(T)p.gamma};
    dt = cmul(dt, f);
  }

  void rk3_step() {  // run.f90:44-55
    // eye*0.5*dt: (0, 0.5) * dt
    const C<T> cf = {-(T)0.5 * dt.im, (T)0.5 * dt.re};
    get_rhs();
    for_interior([&](Rank<T>& R, int k, int j, int i) {
      size_t q = R.in(k, j, i);
      C<T> w = cmul(cf, R.rhs[q]);
      R.w[q] = w;
      C<T>& ps = R.psi[R.g(k, j, i)];
      ps = cadd(ps, cdivr(w, (T)3));
    });
    get_rhs();
    const T a2 = (T)(-2.) / (T)3.;
    for_interior([&](Rank<T>& R, int k, int j, int i) {
      size_t q = R.in(k, j, i);
      C<T> w = cadd(cscale(a2, R.w[q]), cmul(cf, R.rhs[q]));
      R.w[q] = w;
      C<T>& ps = R.psi[R.g(k, j, i)];
      ps = cadd(ps, w);
    });
    get_rhs();
    for_interior([&](Rank<T>& R, int k, int j, int i) {
      size_t q = R.in(k, j, i);
      C<T> w = cadd(C<T>{-R.w[q].re, -R.w[q].im}, cmul(cf, R.rhs[q]));
      R.w[q] = w;
      C<T>& ps = R.psi[R.g(k, j, i)];
      ps = cadd(ps, cscale((T)0.5, w));
    });
    t = t + dt.re;  // run.f90:55, t real
  }

  // The same RK3 with a compensated state (new, no counterpart in the
  // reference): each stage's psi update psi + (B w) is carried out as an
  // exact two-term sum (Knuth's TwoSum) of psi and B w + lo, where lo keeps
  // the rounding remainder of the previous update, so increments below half
  // an ulp of psi are kept in lo instead of being lost.  get_rhs reads psi
  // alone.  With T = double the remainders are ~1e-16 relative.
  static void two_sum(T a, T b, T& s, T& e) {
    s = a + b;
    const T bb = s - a;
    e = (a - (s - bb)) + (b - bb);
  }
  void comp_update(Rank<T>& R, int k, int j, int i, C<T> inc_plain) {
    C<T>& ps = R.psi[R.g(k, j, i)];
    C<T>& l = R.lo[R.in(k, j, i)];
    const C<T> inc = cadd(inc_plain, l);
    C<T> sum, rem;
    two_sum(ps.re, inc.re, sum.re, rem.re);
    two_sum(ps.im, inc.im, sum.im, rem.im);
    ps = sum;
    l = rem;
  }
  void rk3_step_comp() {
    const C<T> cf = {-(T)0.5 * dt.im, (T)0.5 * dt.re};
    struct DiffScope {   // the compensated form's get_rhs takes the difference-form D2
      bool& f;
      explicit DiffScope(bool& g) : f(g) { f = true; }
      ~DiffScope() { f = false; }
    } scope(diff_lap);
    get_rhs();
    for_interior([&](Rank<T>& R, int k, int j, int i) {
      size_t q = R.in(k, j, i);
      C<T> w = cmul(cf, R.rhs[q]);
      R.w[q] = w;
      comp_update(R, k, j, i, cdivr(w, (T)3));
    });
    get_rhs();
    const T a2 = (T)(-2.) / (T)3.;
    for_interior([&](Rank<T>& R, int k, int j, int i) {
      size_t q = R.in(k, j, i);
      C<T> w = cadd(cscale(a2, R.w[q]), cmul(cf, R.rhs[q]));
      R.w[q] = w;
      comp_update(R, k, j, i, w);
    });
    get_rhs();
    for_interior([&](Rank<T>& R, int k, int j, int i) {
      size_t q = R.in(k, j, i);
      C<T> w = cadd(C<T>{-R.w[q].re, -R.w[q].im}, cmul(cf, R.rhs[q]));
      R.w[q] = w;
      comp_update(R, k, j, i, cscale((T)0.5, w));
    });
    t = t + dt.re;
  }

  void imag_euler_step() {  // run.f90:21-23
    const C<T> cf = {dt.re * (T)0.5, dt.im * (T)0.5};
    get_rhs();
    for_interior([&](Rank<T>& R, int k, int j, int i) {
      C<T>& ps = R.psi[R.g(k, j, i)];
      ps = cadd(ps, cmul(cf, R.rhs[R.in(k, j, i)]));
    });
  }

  // Reference Psi_norm: sum(abs(Psi)**2) in T per rank, then rank-order sum.
  T psi_norm_ref() {
    T tot = 0;
    for (auto& R : ranks) {
      T s = 0;
      for (int i = 1; i <= R.nmx; ++i)
        for (int j = 1; j <= R.nmy; ++j)
          for (int k = 1; k <= R.nmz; ++k) {
            T a = cabs_(R.psi[R.g(k, j, i)]);
            s = s + a * a;
          }
      tot = tot + s;
    }
    return tot;
  }

  // ------------------------------------------------ FP64 diagnostics (new) --
  struct Acc {  // Neumaier-compensated FP64 sum
    double s = 0, c = 0;
    void add(double v) {
      double tt = s + v;
      if (std::fabs(s) >= std::fabs(v)) c += (s - tt) + v; else c += (v - tt) + s;
      s = tt;
    }
    double val() const { return s + c; }
  };

  void diag(trapbec_diag_out* o) {
    ghost_comm();
    const bool two = p.two_dim != 0;
    Acc n, K, P, Q, Rr, sa;
    double mx = -1, mn = std::numeric_limits<double>::infinity();
    int nonfinite = 0;
    for (auto& R : ranks) {
      const ptrdiff_t sx = (ptrdiff_t)(R.gz * R.gy), sy = (ptrdiff_t)R.gz;
      for (int i = 1; i <= R.nmx; ++i)
        for (int j = 1; j <= R.nmy; ++j)
          for (int k = 1; k <= R.nmz; ++k) {
            const C<T>* c = &R.psi[R.g(k, j, i)];
            C<T> lap = second_deriv_ref(c, sx, hx);
            lap = cadd(lap, second_deriv_ref(c, sy, hy));
            if (!two) lap = cadd(lap, second_deriv_ref(c, 1, hz));
            bool act;
            C<T> fr = frame_term(R, c, sx, sy, j, i, &act);
            double re = c->re, im = c->im;
            double a2 = re * re + im * im;
            if (!std::isfinite(a2)) nonfinite = 1;
            double pot = potential(R, k, j, i);
            n.add(a2);
            K.add(re * (double)lap.re + im * (double)lap.im);
            P.add(pot * a2);
            Q.add(a2 * a2);
            Rr.add(re * (double)fr.re + im * (double)fr.im);
            double a = std::sqrt(a2);
            sa.add(a);
            mx = std::max(mx, a); mn = std::min(mn, a);
          }
    }
    double dV = (double)hx * (double)hy * (p.two_dim ? 1.0 : (double)hz);
    o->intpsi2 = n.val();
    o->maxpsi = mx; o->minpsi = mn;
    o->meanpsi = sa.val() / ((double)p.nx * p.ny * p.nz);
    o->norm = dV * n.val();
    o->kinetic = K.val(); o->potential = P.val(); o->interaction = Q.val(); o->rotation = Rr.val();
    o->energy = dV * (-0.5 * K.val() + 0.5 * P.val() + 0.25 * Q.val() - 0.5 * Rr.val());
    o->mu = (-0.5 * K.val() + 0.5 * P.val() + 0.5 * Q.val() - 0.5 * Rr.val()) / n.val();
    o->nonfinite = nonfinite;
    o->reserved = 0;
  }

  // ---------------------------- imaginary-time RK3 with renormalisation (new) --
  // d psi / d tau = rhs / 2 (the real-time operator i*0.5*dt replaced by the
  // real 0.5*dtau), same 2N-storage coefficients as run.f90:46-54, then
  // psi <- psi * sqrt(N0/N) in FP64, then E in FP64.
  int imag_rk3(int nsteps, double tol, int* steps_done, double* rel_de) {
    const T cf = (T)0.5 * dt.re;
    trapbec_diag_out d;
    if (!(norm_target > 0)) { diag(&d); norm_target = d.norm; }
    diag(&d);            // energy of the incoming state: the first test is after step 1
    e_prev = d.energy;
    int s = 0;
    double rel = std::numeric_limits<double>::infinity();
    const T a2 = (T)(-2.) / (T)3.;
    for (s = 1; s <= nsteps; ++s) {
      get_rhs();
      for_interior([&](Rank<T>& R, int k, int j, int i) {
        size_t q = R.in(k, j, i);
        C<T> w = cscale(cf, R.rhs[q]);
        R.w[q] = w;
        C<T>& ps = R.psi[R.g(k, j, i)];
        ps = cadd(ps, cdivr(w, (T)3));
      });
      get_rhs();
      for_interior([&](Rank<T>& R, int k, int j, int i) {
        size_t q = R.in(k, j, i);
        C<T> w = cadd(cscale(a2, R.w[q]), cscale(cf, R.rhs[q]));
        R.w[q] = w;
        C<T>& ps = R.psi[R.g(k, j, i)];
        ps = cadd(ps, w);
      });
      get_rhs();
      for_interior([&](Rank<T>& R, int k, int j, int i) {
        size_t q = R.in(k, j, i);
        C<T> w = cadd(C<T>{-R.w[q].re, -R.w[q].im}, cscale(cf, R.rhs[q]));
        R.w[q] = w;
        C<T>& ps = R.psi[R.g(k, j, i)];
        ps = cadd(ps, cscale((T)0.5, w));
      });
      // renormalise (FP64 norm, scale rounded to T)
      Acc n;
      for (auto& R : ranks)
        for (int i = 1; i <= R.nmx; ++i)
          for (int j = 1; j <= R.nmy; ++j)
            for (int k = 1; k <= R.nmz; ++k) {
              const C<T>& c = R.psi[R.g(k, j, i)];
              n.add((double)c.re * c.re + (double)c.im * c.im);
            }
      double dV = (double)hx * (double)hy * (p.two_dim ? 1.0 : (double)hz);
      double N = dV * n.val();
      if (!(N > 0) || !std::isfinite(N)) { *steps_done = s; *rel_de = NAN; return TRAPBEC_ERR_NONFINITE; }
      const T sc = (T)std::sqrt(norm_target / N);
      for_interior([&](Rank<T>& R, int k, int j, int i) {
        C<T>& ps = R.psi[R.g(k, j, i)];
        ps = cscale(sc, ps);
      });
      diag(&d);
      const double dE = std::fabs(d.energy - e_prev);
      rel = imag_stop == 0 ? dE / std::fabs(d.energy) : (imag_stop == 2 ? dE / norm_target : dE) * imag_escale;
      e_prev = d.energy;
      if (imag_stop == 0 ? rel <= tol : rel < tol) break;
    }
    if (s > nsteps) s = nsteps;
    *steps_done = s;
    *rel_de = rel;
    return TRAPBEC_OK;
  }

  // ------------------------------------------------------ initial states --
  T ring_density(T r) const {  // initial.f90:628-635
    T c1 = (T)11 / (T)32;
    T c3 = ((T)5 - (T)32 * c1) / ((T)48 - (T)192 * c1);
    T c2 = c1 * (c3 - (T)0.25);
    T r2 = r * r;
    return std::sqrt(r2 * (c1 + c2 * r2) / ((T)1 + c3 * r2 + c2 * (r2 * r2)));
  }
  static C<T> cexpi(T th) { return {std::cos(th), std::sin(th)}; }
  T vortex_func(T r) const { return (T)1 - std::exp((T)(-0.7) * std::pow(r, (T)1.15)); }

  void set_cell(Rank<T>& R, int k, int j, int i, C<T> v) { R.psi[R.g(k, j, i)] = v; }
  C<T>& cell(Rank<T>& R, int k, int j, int i) { return R.psi[R.g(k, j, i)]; }

  T tf_dense(const Rank<T>& R, int k, int j, int i) const {  // initial.f90:644
    T a = R.xx[i] / Lx, b = R.yy[j] / Ly, c = R.zz[k] / Lz;
    return (T)1 - (T)p.harm_wx * (a * a) - (T)p.harm_wy * (b * b) - (T)p.harm_wz * (c * c);
  }

  int init_state(const char* name, const trapbec_init_args* a) {
    std::string nm(name);
    Rng rng{a ? a->seed : 0};
    auto runif = [&](T lo, T hi) { T u = (T)rng.next(); return lo + u * (hi - lo); };
    const bool helper = nm == "add_noise" || nm == "add_ring" || nm == "add_dipole" || nm == "phase_imprint" ||
                        nm == "add_pcurrent";
    if (!helper)
      for (auto& R : ranks) std::fill(R.psi.begin(), R.psi.end(), C<T>{0, 0});
    const T ring_rad = (T)p.ring_rad;
    // psi *= func(r) e^{i dir theta} for a straight vortex in plane pl (0: x-y, 1: x-z, 2: y-z)
    auto vortex_mul = [&](T p1, T p2, T dir, int pl) {
      for_interior([&](Rank<T>& R, int k, int j, int i) {
        T c1 = pl == 2 ? R.yy[j] : R.xx[i], c2 = pl == 0 ? R.yy[j] : R.zz[k];
        T dx = c1 - p1, dy = c2 - p2;
        C<T> tmp = cscale(vortex_func(std::sqrt(dx * dx + dy * dy)), cexpi(dir * std::atan2(dy, dx)));
        cell(R, k, j, i) = cmul(cell(R, k, j, i), tmp);
      });
    };
    // ring_p1 * conjg(ring_p2) of a ring whose axis coordinate is x (axis 0) or
    // y (axis 1) shifted by sa, radius over the other in-plane coordinate and z - sz
    auto ringpair = [&](int axis, T sa, T sz, T rr0, bool assign) {
      for_interior([&](Rank<T>& R, int k, int j, int i) {
        T u = (axis == 0 ? R.xx[i] : R.yy[j]) - sa;
        T ww = axis == 0 ? R.yy[j] : R.xx[i];
        T zq = R.zz[k] - sz;
        T sq = std::sqrt(ww * ww + zq * zq);
        T th = std::atan2(u, sq + rr0);
        T r = std::sqrt(u * u + (sq + rr0) * (sq + rr0));
        C<T> p1 = cscale(ring_density(r), cexpi(th));
        th = std::atan2(u, sq - rr0);
        r = std::sqrt(u * u + (sq - rr0) * (sq - rr0));
        C<T> p2 = cscale(ring_density(r), cexpi(th));
        C<T> pr = cmul(p1, C<T>{p2.re, -p2.im});
        cell(R, k, j, i) = assign ? pr : cmul(cell(R, k, j, i), pr);
      });
    };
    auto tf_mul = [&]() {  // multiply_thomas_fermi, initial.f90:654-667
      for_interior([&](Rank<T>& R, int k, int j, int i) {
        T d = tf_dense(R, k, j, i);
        if (d < (T)0) d = 0;
        cell(R, k, j, i) = cscale(d, cell(R, k, j, i));
      });
    };
    const int wn = p.winding_number;
    if (nm == "constant") {
      T v = (T)1 / std::sqrt((T)2);
      for_interior([&](Rank<T>& R, int k, int j, int i) { set_cell(R, k, j, i, {v, v}); });
    } else if (nm == "thomas_fermi" || nm == "soliton") {  // initial.f90:637-652, 67-80
      for_interior([&](Rank<T>& R, int k, int j, int i) {
        T d = tf_dense(R, k, j, i);
        d = d / std::sqrt((T)2);
        if (d < (T)0) d = 0;
        set_cell(R, k, j, i, {d, d});
      });
      if (nm == "soliton") {
        for_interior([&](Rank<T>& R, int k, int j, int i) {
          T ld = cabs_(cell(R, k, j, i));
          C<T> e = R.xx[i] < (T)0 ? cexpi((T)0) : cexpi(pi);
          set_cell(R, k, j, i, cscale(ld, e));
        });
      }
    } else if (nm == "single_vortex") {  // initial.f90:109-121
      for_interior([&](Rank<T>& R, int k, int j, int i) {
        T dx = R.xx[i], dy = R.yy[j];
        T r = std::sqrt(dx * dx + dy * dy);
        T th = std::atan2(dy, dx);
        T f = vortex_func(r);
        set_cell(R, k, j, i, cscale(f, cexpi((T)wn * th)));
      });
    } else if (nm == "sausage") {  // initial.f90:122-138
      for_interior([&](Rank<T>& R, int k, int j, int i) {
        T dx = R.xx[i], dy = R.yy[j];
        T r = std::sqrt(dx * dx + dy * dy);
        T th = std::atan2(dy, dx);
        T f = std::fabs(R.zz[k]) < (T)4 ? (T)1 - std::exp((T)(-0.1) * std::pow(r, (T)1.15)) : vortex_func(r);
        set_cell(R, k, j, i, cscale(f, cexpi(th)));
      });
    } else if (nm == "crow") {  // initial.f90:90-108
      for_interior([&](Rank<T>& R, int k, int j, int i) {
        T vy = -Ly / (T)4;
        T vx1 = (T)(-4) + std::cos(pi * R.zz[k] / Lz);
        T dx = R.xx[i] - vx1, dy = R.yy[j] - vy;
        C<T> a = cscale(vortex_func(std::sqrt(dx * dx + dy * dy)), cexpi(std::atan2(dy, dx)));
        T vx2 = (T)4 - std::cos(pi * R.zz[k] / Lz);
        dx = R.xx[i] - vx2;
        C<T> b = cscale(vortex_func(std::sqrt(dx * dx + dy * dy)), cexpi(-std::atan2(dy, dx)));
        set_cell(R, k, j, i, cmul(a, b));
      });
    } else if (nm == "random_points" || nm == "leap_frog") {  // initial.f90:268-344
      for_interior([&](Rank<T>& R, int k, int j, int i) { set_cell(R, k, j, i, {(T)0.7071, (T)0.7071}); });
      int nv = nm == "random_points" ? 20 : 4;
      for (int v = 1; v <= nv; ++v) {
        T vx, vy, dir;
        if (nm == "random_points") {
          vx = runif(-Lx / (T)5, Lx / (T)5);
          vy = runif(-Ly / (T)5, Ly / (T)5);
          dir = runif((T)0.9, (T)1);
          dir = dir < (T)0.5 ? (T)(-1) : (T)1;
        } else {
          const T sh = 3, s1 = 3, s2 = 12;
          if (v == 1) { vx = -sh; vy = s1; dir = 1; }
          else if (v == 2) { vx = sh; vy = s2; dir = 1; }
          else if (v == 3) { vx = -sh; vy = -s1; dir = -1; }
          else { vx = sh; vy = -s2; dir = -1; }
        }
        for_interior([&](Rank<T>& R, int k, int j, int i) {
          T dx = R.xx[i] - vx, dy = R.yy[j] - vy;
          C<T> tmp = cscale(vortex_func(std::sqrt(dx * dx + dy * dy)), cexpi(dir * std::atan2(dy, dx)));
          cell(R, k, j, i) = cmul(cell(R, k, j, i), tmp);
        });
      }
    } else if (nm == "vortex_rings") {  // initial.f90:202-266
      for_interior([&](Rank<T>& R, int k, int j, int i) { set_cell(R, k, j, i, {(T)1, (T)0}); });
      for (int v = 1; v <= p.vor_ring_count; ++v) {
        T ax = runif(0, 0), ay = runif(0, (T)2 * pi), az = runif(0, (T)2 * pi);
        T tu = runif(-1, 1), tth = runif(0, (T)2 * pi), tr = runif(0, Lx / (T)6);
        T tx = tr * std::sqrt((T)1 - tu * tu) * std::cos(tth);
        T ty = tr * std::sqrt((T)1 - tu * tu) * std::sin(tth);
        T tz = tr * tu;
        for_interior([&](Rank<T>& R, int k, int j, int i) {
          T x = R.xx[i], y = R.yy[j], z = R.zz[k];
          T X = std::cos(ay) * std::cos(az) * x +
                (std::cos(ax) * std::sin(az) + std::sin(ax) * std::sin(ay) * std::cos(az)) * y +
                (std::sin(ax) * std::sin(az) - std::cos(ax) * std::sin(ay) * std::cos(az)) * z;
          T Y = -std::cos(ay) * std::sin(az) * x +
                (std::cos(ax) * std::cos(az) - std::sin(ax) * std::sin(ay) * std::sin(az)) * y +
                (std::sin(ax) * std::cos(ay) + std::cos(ax) * std::sin(ay) * std::sin(az)) * z;
          T Z = std::sin(ay) * x - std::sin(ax) * std::cos(ay) * y + std::cos(ax) * std::cos(ay) * z;
          T s = std::sqrt((Y - ty) * (Y - ty) + (Z - tz) * (Z - tz));
          T r = std::sqrt((X - tx) * (X - tx) + (s + ring_rad) * (s + ring_rad));
          T th = std::atan2(Z - tz, Y - ty);
          auto pade = [&](T rr) {
            T r2 = rr * rr;
            return std::sqrt(r2 * ((T)0.347 + (T)0.0286 * r2) / ((T)1 + (T)0.3333 * r2 + (T)0.0286 * (r2 * r2)));
          };
          C<T> p1 = cscale(pade(r), cexpi(th));
          r = std::sqrt((X - tx) * (X - tx) + (s - ring_rad) * (s - ring_rad));
          C<T> p2 = cscale(pade(r), cexpi(th));
          C<T> tmp = cmul(p1, C<T>{p2.re, -p2.im});
          cell(R, k, j, i) = cmul(cell(R, k, j, i), tmp);
        });
      }
    } else if (nm == "lattice") {  // initial.f90:377-420 (ramp = 0: straight lines)
      for_interior([&](Rank<T>& R, int k, int j, int i) { set_cell(R, k, j, i, {(T)1, (T)1}); });
      for (int v1 = 1; v1 <= 10; ++v1)
        for (int v2 = 1; v2 <= 10; ++v2) {
          (void)runif(0, (T)2 * pi);
          (void)runif(0, 1);
          vortex_mul((T)v1 * (Lx / (T)16) - Lx / (T)3, (T)v2 * (Ly / (T)16) - Ly / (T)3, (T)1, 0);
        }
    } else if (nm == "lattice2" || nm == "bundle") {  // initial.f90:422-539
      for_interior([&](Rank<T>& R, int k, int j, int i) {
        T d = tf_dense(R, k, j, i) / std::sqrt((T)2);
        if (d < (T)0) d = 0;
        set_cell(R, k, j, i, {d, d});
      });
      if (nm == "lattice2") {
        for (int v1 = 1; v1 <= 3; ++v1)
          for (int v2 = 1; v2 <= 3; ++v2)
            vortex_mul((T)v1 * (Lx / (T)4) - Lx / (T)2, (T)v2 * (Ly / (T)4) - Ly / (T)2, (T)1, 0);
        for (int v1 = 1; v1 <= 3; ++v1)
          for (int v2 = 1; v2 <= 3; ++v2)
            vortex_mul((T)v1 * (Lx / (T)4) + (T)10 - Lx / (T)2, (T)v2 * (Lz / (T)4) + (T)10 - Lz / (T)2, (T)1, 1);
      } else {
        for (int pl = 0; pl < 3; ++pl)
          for (int v1 = 1; v1 <= 7; ++v1) {
            T rpos = v1 == 1 ? (T)0 : (T)10;
            T tpos = v1 == 1 ? (T)0 : (T)(v1 - 2) * (T)2 * pi / (T)6;
            T c1 = rpos * std::cos(tpos), c2 = rpos * std::sin(tpos);
            if (pl == 0 || pl == 2) c1 = c1 - (T)30; else c2 = c2 - (T)30;
            vortex_mul(c1, c2, (T)1, pl);
          }
      }
    } else if (nm == "line_of_lines") {  // initial.f90:541-585
      T v = (T)1 / std::sqrt((T)2);
      for_interior([&](Rank<T>& R, int k, int j, int i) { set_cell(R, k, j, i, {v, v}); });
      ringpair(0, 0, 0, ring_rad, false);
    } else if (nm == "linked_rings") {  // initial.f90:587-626
      ringpair(0, 0, 0, ring_rad, true);
      ringpair(1, 0, ring_rad * (T)1.2, ring_rad, false);
    } else if (nm == "random_phase") {  // setup_quench, initial.f90:346-375
      for (int kk = 1; kk <= 20; ++kk) {
        T k1 = std::floor(runif(-20, 20)), k2 = std::floor(runif(-20, 20)), k3 = std::floor(runif(-20, 20));
        T a1 = runif((T)(-0.1), (T)0.1), a2 = runif((T)(-0.1), (T)0.1);
        for_interior([&](Rank<T>& R, int k, int j, int i) {
          T sarg = R.xx[i] * k1 + R.yy[j] * k2;
          if (!p.two_dim) sarg = sarg + R.zz[k] * k3;
          T ph = sarg * (T)2 * pi / Lx;
          C<T> e = cexpi(ph);
          cell(R, k, j, i) = cadd(cell(R, k, j, i), cmul(C<T>{a1, a2}, e));
        });
      }
      tf_mul();
    } else if (nm == "add_noise") {  // initial.f90:741-757, seeded per-cell uniforms
      uint64_t sd = a ? a->seed : 0;
      for_interior([&](Rank<T>& R, int k, int j, int i) {
        int I = R.cx * R.nmx + (i - 1), J = R.cy * R.nmy + (j - 1);
        uint64_t gi = ((uint64_t)I * p.ny + J) * p.nz + (k - 1);
        T e1 = (T)cell_uniform(sd, gi, 0) * (T)2 - (T)1, e2 = (T)cell_uniform(sd, gi, 1) * (T)2 - (T)1;
        cell(R, k, j, i) = cadd(cell(R, k, j, i), C<T>{(T)0.01 * e1, (T)0.01 * e2});
      });
    } else if (nm == "add_ring") {  // setup_add_ring option 1, initial.f90:759-794
      ringpair(0, (T)(-0.25) * Lx, 0, ring_rad, false);
    } else if (nm == "add_dipole") {  // initial.f90:839-870
      vortex_mul((T)(-20), (T)5, (T)1, 0);
      vortex_mul((T)(-20), (T)(-5), (T)(-1), 0);
    } else if (nm == "phase_imprint") {  // initial.f90:820-836
      for_interior([&](Rank<T>& R, int k, int j, int i) {
        T dense = cabs_(cell(R, k, j, i));
        T th = std::atan2(R.yy[j], R.xx[i]);
        set_cell(R, k, j, i, cscale(dense, cexpi((T)wn * th)));
      });
    } else if (nm == "add_pcurrent") {  // initial.f90:669-739
      const int pk = p.potential;
      for_interior([&](Rank<T>& R, int k, int j, int i) {
        T x = R.xx[i], y = R.yy[j], th = 0, m = 1;
        if (pk == TRAPBEC_POT_BARRIER) th = y < (T)0 ? x * (T)50 * pi / Lx : (T)20 * pi - x * (T)50 * pi / Lx;
        else if (pk == TRAPBEC_POT_MOBIUS) th = (T)20 * std::atan2(y, x);
        else if (pk == TRAPBEC_POT_HARMONIC_RING) {
          T a1 = x / Lx, b1 = y / Lx;
          T r = std::sqrt(a1 * a1 + b1 * b1);
          th = r < (T)0.3 ? std::atan2(y, x) : std::atan2(-y, x);
          m = 10;
        } else if (pk == TRAPBEC_POT_HARMONIC_RING2) {
          th = y < (T)0 ? std::atan2((T)0.5 * (y + Ly / (T)5), x) : std::atan2((T)0.5 * (y - Ly / (T)5), x) - pi;
          m = 20;
        } else if (pk == TRAPBEC_POT_CHANNEL) {
          th = (T)10 * (T)2 * pi * (x + (T)0.5 * Lx) / Lx;
          m = 2;
        } else {
          return;
        }
        T ld = cabs_(cell(R, k, j, i));
        set_cell(R, k, j, i, cscale(ld, cexpi(m * th)));
      });
    } else if (nm == "tf_vortex_line" || nm == "tf_vortex_ring" || nm == "tf_noise") {
      // States of the workload set (not reference init_cond cases), in the
      // reference's units, evaluated in FP64 and rounded to T:
      //   tf_vortex_line: amp*sqrt(max(0,1-sum x_a^2 r_tf2_a)) * rho/sqrt(rho^2+core2) * e^{i theta}
      //   tf_vortex_ring: TF * Pade ring of radius ring_radius in z=0 (axis z)
      //                   * e^{i noise_amp (2u-1)}
      //   tf_noise      : TF + noise_amp*(eta1 + i eta2), eta in U[-1,1]
      if (!a) return TRAPBEC_ERR_ARG;
      for_interior([&](Rank<T>& R, int k, int j, int i) {
        double x = R.xx[i], y = R.yy[j], z = R.zz[k];
        double q = 1.0 - x * x * a->r_tf2[0] - y * y * a->r_tf2[1] - z * z * a->r_tf2[2];
        double tf = a->amp * std::sqrt(q > 0 ? q : 0.0);
        int I = R.cx * R.nmx + (i - 1), J = R.cy * R.nmy + (j - 1), K = k - 1;
        uint64_t gi = ((uint64_t)I * p.ny + J) * p.nz + K;
        double re, im;
        if (nm == "tf_vortex_line") {
          double rho2 = x * x + y * y;
          double f = std::sqrt(rho2) / std::sqrt(rho2 + a->core2);
          double th = std::atan2(y, x);
          re = tf * f * std::cos(th); im = tf * f * std::sin(th);
        } else if (nm == "tf_vortex_ring") {
          double s = std::sqrt(x * x + y * y);
          double th1 = std::atan2(z, s + a->ring_radius);
          double r1 = std::sqrt(z * z + (s + a->ring_radius) * (s + a->ring_radius));
          double th2 = std::atan2(z, s - a->ring_radius);
          double r2 = std::sqrt(z * z + (s - a->ring_radius) * (s - a->ring_radius));
          auto pade = [](double r) {
            double c1 = 11.0 / 32.0, c3 = (5.0 - 32.0 * c1) / (48.0 - 192.0 * c1), c2 = c1 * (c3 - 0.25);
            double rr = r * r;
            return std::sqrt(rr * (c1 + c2 * rr) / (1.0 + c3 * rr + c2 * rr * rr));
          };
          double amp = tf * pade(r1) * pade(r2);
          double ph = th1 - th2 + a->noise_amp * (2.0 * cell_uniform(a->seed, gi, 0) - 1.0);
          re = amp * std::cos(ph); im = amp * std::sin(ph);
        } else {
          re = tf + a->noise_amp * (2.0 * cell_uniform(a->seed, gi, 0) - 1.0);
          im = a->noise_amp * (2.0 * cell_uniform(a->seed, gi, 1) - 1.0);
        }
        set_cell(R, k, j, i, {(T)re, (T)im});
      });
    } else {
      return TRAPBEC_ERR_ARG;
    }
    return TRAPBEC_OK;
  }

  // ------------------------------------------------------------ host I/O --
  void set_psi(const T* src) {  // interior, global, z fastest
    for_interior([&](Rank<T>& R, int k, int j, int i) {
      int I = R.cx * R.nmx + (i - 1), J = R.cy * R.nmy + (j - 1);
      size_t q = gidx(k - 1, J, I);
      R.psi[R.g(k, j, i)] = {src[2 * q], src[2 * q + 1]};
    });
  }
  void get_psi(T* dst) {
    for_interior([&](Rank<T>& R, int k, int j, int i) {
      int I = R.cx * R.nmx + (i - 1), J = R.cy * R.nmy + (j - 1);
      size_t q = gidx(k - 1, J, I);
      const C<T>& c = R.psi[R.g(k, j, i)];
      dst[2 * q] = c.re; dst[2 * q + 1] = c.im;
    });
  }
  void get_rhs_out(T* dst) {
    get_rhs();
    for_interior([&](Rank<T>& R, int k, int j, int i) {
      int I = R.cx * R.nmx + (i - 1), J = R.cy * R.nmy + (j - 1);
      size_t q = gidx(k - 1, J, I);
      const C<T>& c = R.rhs[R.in(k, j, i)];
      dst[2 * q] = c.re; dst[2 * q + 1] = c.im;
    });
  }
  void get_ghosted(T* dst) {  // single rank only: Psi(-2:nz+3,-2:ny+3,-2:nx+3)
    ghost_comm();
    const Rank<T>& R = ranks[0];
    for (size_t q = 0; q < R.psi.size(); ++q) { dst[2 * q] = R.psi[q].re; dst[2 * q + 1] = R.psi[q].im; }
  }
  // ---------------------------------------------------------- force.f90 --
  static T pade_density(T r) {  // force.f90:46-54
    const T c1 = (T)11 / (T)32;
    const T c3 = ((T)5 - (T)32 * c1) / ((T)48 - (T)192 * c1);
    const T c2 = c1 * (c3 - (T)0.25);
    return std::sqrt((r * r) * (c1 + c2 * (r * r)) / ((T)1 + c3 * (r * r) + c2 * (r * r * r * r)));
  }
  // force_random_points body (force.f90:33-44) at a given position and sign
  void force_vortex(T x0, T y0, T dir) {
    for_interior([&](Rank<T>& R, int k, int j, int i) {
      const T r = std::sqrt((R.xx[i] - x0) * (R.xx[i] - x0) + (R.yy[j] - y0) * (R.yy[j] - y0));
      const T theta = std::atan2(R.yy[j] - y0, R.xx[i] - x0);
      const T func = pade_density(r);
      const C<T> f = {func * std::cos(dir * theta), func * std::sin(dir * theta)};
      C<T>& ps = R.psi[R.g(k, j, i)];
      ps = cmul(ps, f);
    });
  }

  // ----------------------------------------------------- diagnostic.f90 --
  // Both diagnostics follow the ghost_comm of run.f90:64 and work per rank on
  // its ghosted array, whose edge and corner ghosts ghost_comm never writes
  // (they keep the zeros of initial.f90:27).  Output: [3][nx][ny][nz].
  static T first_deriv(const T* v, T h) {  // deriv.f90:5-11, v points at vect(0)
    return (-v[-3] + (T)9 * v[-2] - (T)45 * v[-1] + (T)45 * v[1] - (T)9 * v[2] + v[3]) / ((T)60 * h);
  }
  static T real_second_deriv(T m2, T m1, T c, T p1, T p2, T h) {  // deriv.f90:26-32
    return (-m2 + (T)16 * m1 - (T)30 * c + (T)16 * p1 - p2) / ((T)12 * (h * h));
  }
  static T low_first_deriv(T m1, T p1, T h) { return (-m1 + p1) / ((T)2 * h); }  // deriv.f90:33-39

  // get_phase (diagnostic.f90:27-48)
  void velocity(T* out) {
    ghost_comm();
    const size_t n = (size_t)p.nx * p.ny * p.nz;
    for (auto& R : ranks) {
      std::vector<T> ph(R.psi.size());
      for (size_t q = 0; q < ph.size(); ++q) ph[q] = std::atan2(R.psi[q].im, R.psi[q].re);
      std::vector<T> lx(7), ly(7);
      for (int i = 1; i <= R.nmx; ++i)
        for (int j = 1; j <= R.nmy; ++j)
          for (int k = 1; k <= R.nmz; ++k) {
            for (int m = -3; m <= 3; ++m) {
              lx[m + 3] = ph[R.g(k, j, i + m)];
              ly[m + 3] = ph[R.g(k, j + m, i)];
            }
            const size_t q = gidx(k - 1, R.cy * R.nmy + j - 1, R.cx * R.nmx + i - 1);
            out[q] = first_deriv(&lx[3], hx);
            out[n + q] = first_deriv(&ly[3], hy);
            out[2 * n + q] = first_deriv(&ph[R.g(k, j, i)], hz);   // z is contiguous
          }
    }
  }

  // get_qpressure (diagnostic.f90:50-84)
  void qpressure(T* out) {
    ghost_comm();
    const size_t n = (size_t)p.nx * p.ny * p.nz;
    for (auto& R : ranks) {
      std::vector<T> den(R.psi.size());
      for (size_t q = 0; q < den.size(); ++q) den[q] = std::hypot(R.psi[q].re, R.psi[q].im);
      const int ex = R.nmx + 2, ey = R.nmy + 2, ez = R.nmz + 2;   // laplace_rho(0:nmz+1, 0:nmy+1, 0:nmx+1)
      std::vector<T> lap((size_t)ex * ey * ez);
      auto L = [&](int k, int j, int i) -> T& { return lap[((size_t)i * ey + j) * ez + k]; };
      auto d = [&](int k, int j, int i) { return den[R.g(k, j, i)]; };
      for (int i = 0; i <= R.nmx + 1; ++i)
        for (int j = 0; j <= R.nmy + 1; ++j)
          for (int k = 0; k <= R.nmz + 1; ++k) {
            T v = real_second_deriv(d(k, j, i - 2), d(k, j, i - 1), d(k, j, i), d(k, j, i + 1), d(k, j, i + 2), hx);
            v = v + real_second_deriv(d(k, j - 2, i), d(k, j - 1, i), d(k, j, i), d(k, j + 1, i), d(k, j + 2, i), hy);
            v = v + real_second_deriv(d(k - 2, j, i), d(k - 1, j, i), d(k, j, i), d(k + 1, j, i), d(k + 2, j, i), hz);
            L(k, j, i) = v;
          }
      for (int i = 1; i <= R.nmx; ++i)
        for (int j = 1; j <= R.nmy; ++j)
          for (int k = 1; k <= R.nmz; ++k) {
            const size_t q = gidx(k - 1, R.cy * R.nmy + j - 1, R.cx * R.nmx + i - 1);
            out[q] = low_first_deriv(L(k, j, i - 1), L(k, j, i + 1), hx);
            out[n + q] = low_first_deriv(L(k, j - 1, i), L(k, j + 1, i), hy);
            out[2 * n + q] = low_first_deriv(L(k - 1, j, i), L(k + 1, j, i), hz);
          }
    }
  }

  void set_trap(const double* tr) {
    for_interior([&](Rank<T>& R, int k, int j, int i) {
      int I = R.cx * R.nmx + (i - 1), J = R.cy * R.nmy + (j - 1);
      R.trap[R.in(k, j, i)] = (T)tr[gidx(k - 1, J, I)];
    });
  }
};

struct Handle {
  int prec;
  void* o;
};

template <typename F> int dispatch(Handle* h, F f) {
  if (!h) return TRAPBEC_ERR_ARG;
  if (h->prec == TRAPBEC_FP64) return f(*static_cast<Oracle<double>*>(h->o));
  return f(*static_cast<Oracle<float>*>(h->o));
}

}  // namespace

extern "C" {

void* orc_create(const trapbec_params* p) {
  if (!p || p->nx <= 0 || p->ny <= 0 || p->nz <= 0) return nullptr;
  int px = p->nprocx > 0 ? p->nprocx : 1, py = p->nprocy > 0 ? p->nprocy : 1;
  if (p->nx % px || p->ny % py) return nullptr;  // mpi_var.f90:157-160
  Handle* h = new Handle;
  h->prec = p->precision;
  if (p->precision == TRAPBEC_FP64) h->o = new Oracle<double>(*p);
  else h->o = new Oracle<float>(*p);
  return h;
}
void orc_destroy(void* hv) {
  Handle* h = (Handle*)hv;
  if (!h) return;
  if (h->prec == TRAPBEC_FP64) delete (Oracle<double>*)h->o; else delete (Oracle<float>*)h->o;
  delete h;
}
void orc_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}
int orc_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
int orc_set_psi(void* h, const void* psi) {
  return dispatch((Handle*)h, [&](auto& o) {
    using T = std::remove_reference_t<decltype(o.t)>;
    o.set_psi((const T*)psi);
    for (auto& R : o.ranks) std::fill(R.lo.begin(), R.lo.end(), C<T>{0, 0});   // a new state: no remainder
    if (!o.norm_user) o.norm_target = -1.0;   // the next relaxation keeps the new state's norm
    return 0; });
}
int orc_get_psi(void* h, void* psi) {
  return dispatch((Handle*)h, [&](auto& o) {
    using T = std::remove_reference_t<decltype(o.t)>;
    o.get_psi((T*)psi); return 0; });
}
int orc_get_psi_ghosted(void* h, void* out) {
  return dispatch((Handle*)h, [&](auto& o) {
    using T = std::remove_reference_t<decltype(o.t)>;
    if (o.ranks.size() != 1) return (int)TRAPBEC_ERR_ARG;
    o.get_ghosted((T*)out); return 0; });
}
int orc_get_rhs(void* h, void* out) {
  return dispatch((Handle*)h, [&](auto& o) {
    using T = std::remove_reference_t<decltype(o.t)>;
    o.get_rhs_out((T*)out); return 0; });
}
int orc_force_vortex(void* h, double x0, double y0, double dir) {
  return dispatch((Handle*)h, [&](auto& o) {
    using T = std::remove_reference_t<decltype(o.t)>;
    o.force_vortex((T)x0, (T)y0, (T)dir); return 0; });
}
int orc_velocity(void* h, void* out) {
  return dispatch((Handle*)h, [&](auto& o) {
    using T = std::remove_reference_t<decltype(o.t)>;
    o.velocity((T*)out); return 0; });
}
int orc_qpressure(void* h, void* out) {
  return dispatch((Handle*)h, [&](auto& o) {
    using T = std::remove_reference_t<decltype(o.t)>;
    o.qpressure((T*)out); return 0; });
}
int orc_set_trap(void* h, const double* tr) {
  return dispatch((Handle*)h, [&](auto& o) { o.set_trap(tr); return 0; });
}
int orc_coords(void* h, double* xx, double* yy, double* zz) {  // global arrays
  return dispatch((Handle*)h, [&](auto& o) {
    for (auto& R : o.ranks) {
      for (int i = 1; i <= R.nmx; ++i) xx[R.cx * R.nmx + i - 1] = R.xx[i];
      for (int j = 1; j <= R.nmy; ++j) yy[R.cy * R.nmy + j - 1] = R.yy[j];
      for (int k = 1; k <= R.nmz; ++k) zz[k - 1] = R.zz[k];
    }
    return 0; });
}
int orc_apply_damping(void* h) {
  return dispatch((Handle*)h, [&](auto& o) { o.apply_damping(); return 0; });
}
int orc_step_rt(void* h, int nsteps, double* t) {
  return dispatch((Handle*)h, [&](auto& o) {
    using T = std::remove_reference_t<decltype(o.t)>;
    o.t = (T)*t;
    for (int s = 0; s < nsteps; ++s) o.rk3_step();
    *t = (double)o.t; return 0; });
}
int orc_step_rt_comp(void* h, int nsteps, double* t) {
  return dispatch((Handle*)h, [&](auto& o) {
    using T = std::remove_reference_t<decltype(o.t)>;
    o.t = (T)*t;
    for (int s = 0; s < nsteps; ++s) o.rk3_step_comp();
    *t = (double)o.t; return 0; });
}
int orc_step_imag_euler(void* h, int nsteps, double* ratio) {
  return dispatch((Handle*)h, [&](auto& o) {
    double r = 0;
    for (int s = 0; s < nsteps; ++s) {
      o.imag_euler_step();
      double n = (double)o.psi_norm_ref();
      r = n / o.intpsi2_old;   // run.f90:23
      o.intpsi2_old = n;
    }
    *ratio = r; return 0; });
}
int orc_step_imag_rk3(void* h, int nsteps, double tol, int* steps_done, double* rel) {
  return dispatch((Handle*)h, [&](auto& o) { return o.imag_rk3(nsteps, tol, steps_done, rel); });
}
int orc_set_imag_stop(void* h, int mode, double escale) {
  return dispatch((Handle*)h, [&](auto& o) { o.imag_stop = mode; o.imag_escale = escale; return 0; });
}
int orc_set_norm_target(void* h, double n0) {
  return dispatch((Handle*)h, [&](auto& o) { o.norm_target = n0; o.norm_user = n0 > 0; return 0; });
}
int orc_set_omega(void* h, double om) {
  return dispatch((Handle*)h, [&](auto& o) { o.p.omega_z = om; return 0; });
}
int orc_set_t(void* h, double t) {
  return dispatch((Handle*)h, [&](auto& o) {
    using T = std::remove_reference_t<decltype(o.t)>;
    o.t = (T)t; return 0; });
}
int orc_diag(void* h, trapbec_diag_out* out) {
  return dispatch((Handle*)h, [&](auto& o) { o.diag(out); return 0; });
}
double orc_psi_norm_ref(void* h) {
  Handle* hh = (Handle*)h;
  if (hh->prec == TRAPBEC_FP64) return ((Oracle<double>*)hh->o)->psi_norm_ref();
  return (double)((Oracle<float>*)hh->o)->psi_norm_ref();
}
int orc_init_state(void* h, const char* name, const trapbec_init_args* a) {
  return dispatch((Handle*)h, [&](auto& o) {
    if (!o.norm_user) o.norm_target = -1.0;
    return o.init_state(name, a); });
}
double orc_cell_uniform(uint64_t seed, uint64_t idx, uint64_t stream) {
  return cell_uniform(seed, idx, stream);
}

}  // extern "C"
