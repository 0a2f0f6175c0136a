// kernels_init.cuh -- potential fill and initial-state kernels.
//
// The reference evaluates its potential inside get_rhs, per cell per stage
// (finite_diff.f90:29-124).  Here the separable 'harmonic' trap is evaluated
// in the stage kernels from three 1D tables; every other shape (and the laser
// of finite_diff.f90:118-123) is evaluated once per step by fill_potential
// into the Trap array, which the stage kernels read.  Initial states follow
// initial.f90:58-157 and its helpers; random draws come from the host.
#pragma once
#include "common.cuh"

namespace tb {

// splitmix64 finaliser and the per-cell uniform shared with the host.
__host__ __device__ inline uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
  return z ^ (z >> 31);
}
__host__ __device__ inline double cell_uniform(uint64_t seed, uint64_t idx, uint64_t stream) {
  uint64_t h = mix64(seed ^ mix64(idx * 2ULL + stream + 0x632be59bd9b4e019ULL));
  return (double)(h >> 11) * (1.0 / 9007199254740992.0);
}

template <typename T> struct PotArgs {
  T* trap_out;            // destination (n cells)
  const T* trap_in;       // user Trap array (mobius / array), may alias nothing
  const T* xx; const T* yy; const T* zz;
  int nx, ny, nz;         // global grid (for 'channel' cell sizes)
  int kind;               // trapbec_potential
  int lbeam;
  T Lx, Ly, Lz, t;
  T harm_wx, harm_wy, harm_wz, wbeam;
};

template <typename T>
__device__ inline T pot_shape(const PotArgs<T>& a, T x, T y, T z, size_t idx) {
  T pot = 0, r, r1, r2;
  switch (a.kind) {
    case TRAPBEC_POT_ZERO: break;
    case TRAPBEC_POT_HARMONIC: {
      T p = x / a.Lx, q = y / a.Ly, s = z / a.Lz;
      pot = a.harm_wx * (p * p) + a.harm_wy * (q * q) + a.harm_wz * (s * s);
    } break;
    case TRAPBEC_POT_HARMONIC_RING: {
      T p = x / a.Lx, q = y / a.Lx;
      r = sqrt(p * p + q * q);
      T d = r - (T)0.3;
      pot = a.harm_wx * (d * d);
      if (fabs(r - (T)0.3) < (T)0.01) pot = fmax((T)0, (T)5 - (T)0.1 * a.t);
    } break;
    case TRAPBEC_POT_HARMONIC_RING2: {
      T pw = 6;
      r1 = pow(fabs(pow((T)0.25, pw) - (T)0.15 * pow(x / a.Lx, pw) - (T)4 * pow(y / a.Ly - (T)0.2, pw)), (T)1 / pw);
      r2 = pow(fabs(pow((T)0.25, pw) - (T)0.15 * pow(x / a.Lx, pw) - (T)4 * pow(y / a.Ly + (T)0.2, pw)), (T)1 / pw);
      r1 = (r1 < (T)0.2495) ? (T)0 : (T)5;
      r2 = (r2 < (T)0.2495) ? (T)0 : (T)5;
      pot = r1 * r2;
      if (pot < (T)0) pot = 0;
      if (fabs(y / a.Ly) < (T)0.01 && pot < (T)0.01) pot = fmax((T)0, (T)5 - (T)0.1 * a.t);
    } break;
    case TRAPBEC_POT_BARRIER:
      pot = 0;
      if (fabs(y / a.Ly) > (T)0.3) pot = 5;
      if (fabs(y / a.Ly) < (T)0.01) pot = fmax((T)0, (T)5 - (T)0.1 * a.t);
      break;
    case TRAPBEC_POT_BOX_TRAP:
      pot = 10;
      r = sqrt(x * x + y * y);
      if (r < a.Lx / (T)3 && fabs(z) < a.Lz / (T)2.5) pot = 0;
      pot = pot + (T)5 * sin((T)0.1 * a.t) * z / a.Lz;
      break;
    case TRAPBEC_POT_CHANNEL:
      pot = 0;
      if (fabs(y) > (T)0.75 * a.Ly / (T)2 || fabs(z) > (T)0.75 * a.Lz / (T)2) pot = 5;
      for (int l1 = -1; l1 <= 1; ++l1)
        if (fabs(x) < a.Lx / (T)a.nx && fabs(y - (T)l1 * a.Ly / (T)5) < a.Ly / (T)a.ny) pot = (T)7.5;
      for (int l1 = -1; l1 <= 1; ++l1)
        if (fabs(x) < a.Lx / (T)a.nx && fabs(z - (T)l1 * a.Lz / (T)5) < a.Ly / (T)a.ny) pot = (T)7.5;
      break;
    case TRAPBEC_POT_QUARTIC: {
      T p = x / a.Lx, q = y / a.Ly;
      r = sqrt(p * p + q * q);
      T s2 = r * r, s4 = s2 * s2;
      pot = a.harm_wx * (s4 * s4);
    } break;
    case TRAPBEC_POT_SPHERE: {
      T theta = atan2(y, x);
      T p = x / a.Lx, q = y / a.Ly, s = z / a.Lz;
      r1 = sqrt(p * p + q * q + s * s);
      T phi = acos((z / a.Lz) / r1);
      pot = (r1 < (T)0.2 + (T)0.01 * sin((T)20 * phi) + (T)0.01 * cos((T)30 * theta + (T)0.03)) ? (T)10 : (T)0;
    } break;
    case TRAPBEC_POT_MOBIUS:
      pot = a.trap_in[idx];
      if (fabs(y) < (T)1 && fabs(x - (T)25) < (T)1) pot = pot + 10;
      break;
    case TRAPBEC_POT_ARRAY:
      pot = a.trap_in[idx];
      break;
  }
  if (a.lbeam) {
    T las_freq = 0;
    T las_x = (T)70 * cos(las_freq * a.t) * ((T)1 - sin(las_freq * a.t));
    T las_y = (T)30 * sin(las_freq * a.t) * cos(las_freq * a.t);
    T p = (x - las_x) / a.wbeam, q = (y - las_y) / a.wbeam;
    pot = pot + (T)20 * exp(-(p * p) - (q * q));
  }
  return pot;
}

template <typename T>
__global__ void fill_potential_kernel(PotArgs<T> a) {
  const size_t n = (size_t)a.nx * a.ny * a.nz;
  for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += (size_t)gridDim.x * blockDim.x) {
    const int k = (int)(idx % a.nz);
    const size_t r = idx / a.nz;
    const int j = (int)(r % a.ny);
    const int i = (int)(r / a.ny);
    a.trap_out[idx] = pot_shape(a, a.xx[i], a.yy[j], a.zz[k], idx);
  }
}

// The Trap array of the 'mobius' potential, as mesh_init builds it
// (initial.f90:159-198): at every cell the sum over the 200 x 200 points of
// the strip table of exp(-1.5 dx^2 - 1.5 dy^2 - 1.5 dz^2), clamped at 3 after
// every term -- so the terms are added in the reference's order, ii1 outer,
// ii2 inner -- then Trap = max(Trap) - Trap.  The table tab[c][ii2][ii1]
// (200 x 200 per coordinate c) is formed on the host; the arithmetic rounds
// once per operation as the reference's does (no contraction to FMA).
constexpr int MOBIUS_N = 200;
template <typename T> struct RN;
template <> struct RN<float> {
  static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
  static __device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
  static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
};
template <> struct RN<double> {
  static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
  static __device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
  static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
};

template <typename T>
__global__ void mobius_trap_kernel(const T* __restrict__ tab, const T* __restrict__ xx, const T* __restrict__ yy,
                                   const T* __restrict__ zz, int nx, int ny, int nz, T* __restrict__ trap,
                                   unsigned long long* __restrict__ maxbits) {
  using R = RN<T>;
  const size_t n = (size_t)nx * ny * nz;
  const T* t1 = tab;
  const T* t2 = tab + MOBIUS_N * MOBIUS_N;
  const T* t3 = tab + 2 * MOBIUS_N * MOBIUS_N;
  const T c15 = (T)1.5, cap = (T)3;
  T mx = 0;
  for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += (size_t)gridDim.x * blockDim.x) {
    const int k = (int)(idx % nz);
    const size_t r = idx / nz;
    const int j = (int)(r % ny);
    const int i = (int)(r / ny);
    const T x = xx[i], y = yy[j], z = zz[k];
    T acc = 0;   // Trap=0. (initial.f90:171)
    for (int i1 = 0; i1 < MOBIUS_N; ++i1) {
      for (int i2 = 0; i2 < MOBIUS_N; ++i2) {
        const int q = i2 * MOBIUS_N + i1;   // mobius(ii1, ii2, c)
        const T dx = R::sub(x, __ldg(t1 + q)), dy = R::sub(y, __ldg(t2 + q)), dz = R::sub(z, __ldg(t3 + q));
        // -1.5*(dx)**2 - 1.5*(dy)**2 - 1.5*(dz)**2
        T e = -R::mul(c15, R::mul(dx, dx));
        e = R::sub(e, R::mul(c15, R::mul(dy, dy)));
        e = R::sub(e, R::mul(c15, R::mul(dz, dz)));
        acc = R::add(acc, exp(e));
        if (acc > cap) acc = cap;
      }
    }
    trap[idx] = acc;
    mx = acc > mx ? acc : mx;
  }
  // the Trap values are non-negative, so their bit patterns order as unsigned integers
  unsigned long long bits = sizeof(T) == 8 ? (unsigned long long)__double_as_longlong((double)mx)
                                           : (unsigned long long)__float_as_uint((float)mx);
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long b = __shfl_down_sync(0xffffffffu, bits, o);
    bits = b > bits ? b : bits;
  }
  if ((threadIdx.x & 31) == 0) atomicMax(maxbits, bits);
}

// Trap = theta - Trap with theta the maximum over all cells (the MPI_MAX
// reduction over the ranks of initial.f90:189-197).
template <typename T>
__global__ void mobius_invert_kernel(T* __restrict__ trap, size_t n, const unsigned long long* __restrict__ maxbits) {
  const unsigned long long b = *maxbits;
  const T theta = sizeof(T) == 8 ? (T)__longlong_as_double((long long)b) : (T)__uint_as_float((unsigned int)b);
  for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += (size_t)gridDim.x * blockDim.x)
    trap[idx] = theta - trap[idx];
}

// ---------------------------------------------------------------- states --
enum InitKind : int {
  IK_CONST = 0, IK_TF = 1, IK_SOLITON_PHASE = 2, IK_VORTEX_MUL = 3, IK_SINGLE = 4,
  IK_SAUSAGE = 5, IK_CROW = 6, IK_RING_MUL = 7, IK_TF_LINE = 8, IK_TF_RING = 9, IK_TF_NOISE = 10,
  IK_SET = 11, IK_TF_MUL = 12, IK_RINGPAIR_MUL = 13, IK_QUENCH_ADD = 14, IK_PHASE_IMPRINT = 15,
  IK_NOISE_ADD = 16, IK_PCURRENT = 17, IK_FORCE_VORTEX = 18
};

template <typename T> struct InitArgsDev {
  c_t<T>* psi;
  const T* xx; const T* yy; const T* zz;
  int nx, ny, nz;
  int kind;
  int wn;                 // winding number
  T Lx, Ly, Lz, pi;
  T harm_wx, harm_wy, harm_wz;
  T v[12];                // case parameters (reference precision)
  double d[12];           // case parameters of the FP64 workload states
  uint64_t seed;
};

template <typename T> __device__ inline T vortex_func(T r) {  // initial.f90:117
  return (T)1 - exp((T)(-0.7) * pow(r, (T)1.15));
}
// Pade vortex density, ring_density (initial.f90:628-635) = pade_density (force.f90:46-54)
template <typename T> __device__ inline T pade_density(T r) {
  const T c1 = (T)11 / (T)32;
  const T c3 = ((T)5 - (T)32 * c1) / ((T)48 - (T)192 * c1);
  const T c2 = c1 * (c3 - (T)0.25);
  const T r2 = r * r;
  return sqrt(r2 * (c1 + c2 * r2) / ((T)1 + c3 * r2 + c2 * (r2 * r2)));
}
template <typename T> __device__ inline c_t<T> cmul_(c_t<T> a, c_t<T> b) {
  return mk<T>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

template <typename T>
__global__ void init_state_kernel(InitArgsDev<T> a) {
  const size_t n = (size_t)a.nx * a.ny * a.nz;
  for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += (size_t)gridDim.x * blockDim.x) {
    const int k = (int)(idx % a.nz);
    const size_t r = idx / a.nz;
    const int j = (int)(r % a.ny);
    const int i = (int)(r / a.ny);
    const T x = a.xx[i], y = a.yy[j], z = a.zz[k];
    c_t<T>& out = a.psi[idx];
    switch (a.kind) {
      case IK_CONST: out = mk<T>(a.v[0], a.v[1]); break;
      case IK_SET: out = mk<T>(a.v[0], a.v[1]); break;
      case IK_TF: {  // initial.f90:637-652
        T p = x / a.Lx, q = y / a.Ly, s = z / a.Lz;
        T d = (T)1 - a.harm_wx * (p * p) - a.harm_wy * (q * q) - a.harm_wz * (s * s);
        d = d / sqrt((T)2);
        if (d < (T)0) d = 0;
        out = mk<T>(d, d);
      } break;
      case IK_SOLITON_PHASE: {  // initial.f90:67-80
        T ld = hypot(out.x, out.y);
        T th = x < (T)0 ? (T)0 : a.pi;
        out = mk<T>(ld * cos(th), ld * sin(th));
      } break;
      case IK_SINGLE: {  // initial.f90:109-121
        T rr = sqrt(x * x + y * y);
        T th = atan2(y, x);
        T f = vortex_func(rr);
        T ph = (T)a.wn * th;
        out = mk<T>(f * cos(ph), f * sin(ph));
      } break;
      case IK_SAUSAGE: {  // initial.f90:122-138
        T rr = sqrt(x * x + y * y);
        T th = atan2(y, x);
        T f = fabs(z) < (T)4 ? (T)1 - exp((T)(-0.1) * pow(rr, (T)1.15)) : vortex_func(rr);
        out = mk<T>(f * cos(th), f * sin(th));
      } break;
      case IK_CROW: {  // initial.f90:90-108
        T vy = -a.Ly / (T)4;
        T vx1 = (T)(-4) + cos(a.pi * z / a.Lz);
        T dx = x - vx1, dy = y - vy;
        T f = vortex_func(sqrt(dx * dx + dy * dy)), th = atan2(dy, dx);
        c_t<T> p1 = mk<T>(f * cos(th), f * sin(th));
        T vx2 = (T)4 - cos(a.pi * z / a.Lz);
        dx = x - vx2;
        f = vortex_func(sqrt(dx * dx + dy * dy));
        th = -atan2(dy, dx);
        c_t<T> p2 = mk<T>(f * cos(th), f * sin(th));
        out = cmul_<T>(p1, p2);
      } break;
      case IK_VORTEX_MUL: {  // psi *= func(r) e^{i dir theta}; v = (p1, p2, dir, plane)
        // plane 0: (x, y), 1: (x, z), 2: (y, z)  (initial.f90:109-121, 455-457, 530-531)
        const int pl = (int)a.v[3];
        const T c1 = pl == 2 ? y : x, c2 = pl == 0 ? y : z;
        T dx = c1 - a.v[0], dy = c2 - a.v[1];
        T f = vortex_func(sqrt(dx * dx + dy * dy));
        T th = a.v[2] * atan2(dy, dx);
        out = cmul_<T>(out, mk<T>(f * cos(th), f * sin(th)));
      } break;
      case IK_TF_MUL: {  // multiply_thomas_fermi, initial.f90:654-667
        T p = x / a.Lx, q = y / a.Ly, s = z / a.Lz;
        T d = (T)1 - a.harm_wx * (p * p) - a.harm_wy * (q * q) - a.harm_wz * (s * s);
        if (d < (T)0) d = 0;
        out = mk<T>(out.x * d, out.y * d);
      } break;
      case IK_RINGPAIR_MUL: {
        // Pade vortex pair of a ring (ring_density, initial.f90:628-635): axis
        // coordinate u (x if v[0] = 0, y if 1) shifted by v[1]; in-plane radius
        // sqrt(w^2 + (z - v[2])^2) with w the other of x, y; radius v[3]
        // (initial.f90:575-581, 602-622, 775-781).  v[4] = 1: assign instead of multiply.
        const T u = (a.v[0] == (T)0 ? x : y) - a.v[1];
        const T ww = a.v[0] == (T)0 ? y : x;
        const T zz2 = z - a.v[2];
        const T s = sqrt(ww * ww + zz2 * zz2);
        const T R0 = a.v[3];
        auto rd = [](T r) { return pade_density(r); };
        T th = atan2(u, s + R0);
        T r = sqrt(u * u + (s + R0) * (s + R0));
        const c_t<T> p1 = mk<T>(rd(r) * cos(th), rd(r) * sin(th));
        th = atan2(u, s - R0);
        r = sqrt(u * u + (s - R0) * (s - R0));
        const c_t<T> p2 = mk<T>(rd(r) * cos(th), -(rd(r) * sin(th)));
        const c_t<T> pr = cmul_<T>(p1, p2);
        out = a.v[4] != (T)0 ? pr : cmul_<T>(out, pr);
      } break;
      case IK_QUENCH_ADD: {  // setup_quench wave, initial.f90:362-372; v = (k1, k2, k3, ra1, ra2)
        T sarg = x * a.v[0] + y * a.v[1];
        if (!a.wn) sarg = sarg + z * a.v[2];   // wn carries two_dim here
        const T ph = sarg * (T)2 * a.pi / a.Lx;
        const c_t<T> e = mk<T>(cos(ph), sin(ph));
        out = mk<T>(out.x + (a.v[3] * e.x - a.v[4] * e.y), out.y + (a.v[3] * e.y + a.v[4] * e.x));
      } break;
      case IK_PHASE_IMPRINT: {  // initial.f90:820-836
        const T dense = hypot(out.x, out.y);
        const T th = atan2(y, x);
        const T ph = (T)a.wn * th;
        out = mk<T>(dense * cos(ph), dense * sin(ph));
      } break;
      case IK_NOISE_ADD: {  // add_noise, initial.f90:741-757, per-cell seeded uniforms
        const T e1 = (T)cell_uniform(a.seed, (uint64_t)idx, 0) * (T)2 - (T)1;
        const T e2 = (T)cell_uniform(a.seed, (uint64_t)idx, 1) * (T)2 - (T)1;
        out = mk<T>(out.x + (T)0.01 * e1, out.y + (T)0.01 * e2);
      } break;
      case IK_FORCE_VORTEX: {  // force_random_points body, force.f90:33-44; v = (x0, y0, dir)
        const T dx = x - a.v[0], dy = y - a.v[1];
        const T f = pade_density(sqrt(dx * dx + dy * dy));
        const T th = a.v[2] * atan2(dy, dx);
        out = cmul_<T>(out, mk<T>(f * cos(th), f * sin(th)));
      } break;
      case IK_PCURRENT: {  // setup_pcurrent, initial.f90:669-739; v[0] = potential kind
        const int pk = (int)a.v[0];
        T th = 0, m = 1;
        if (pk == TRAPBEC_POT_BARRIER) {
          th = y < (T)0 ? x * (T)50 * a.pi / a.Lx : (T)20 * a.pi - x * (T)50 * a.pi / a.Lx;
        } else if (pk == TRAPBEC_POT_MOBIUS) {
          th = (T)20 * atan2(y, x);
        } else if (pk == TRAPBEC_POT_HARMONIC_RING) {
          const T p = x / a.Lx, q = y / a.Lx;
          const T r = sqrt(p * p + q * q);
          th = r < (T)0.3 ? atan2(y, x) : atan2(-y, x);
          m = 10;
        } else if (pk == TRAPBEC_POT_HARMONIC_RING2) {
          th = y < (T)0 ? atan2((T)0.5 * (y + a.Ly / (T)5), x) : atan2((T)0.5 * (y - a.Ly / (T)5), x) - a.pi;
          m = 20;
        } else if (pk == TRAPBEC_POT_CHANNEL) {
          th = (T)10 * (T)2 * a.pi * (x + (T)0.5 * a.Lx) / a.Lx;
          m = 2;
        } else {
          break;
        }
        const T ld = hypot(out.x, out.y);
        const T ph = m * th;
        out = mk<T>(ld * cos(ph), ld * sin(ph));
      } break;
      case IK_RING_MUL: {  // setup_vortex_rings body, initial.f90:239-254
        const T ax = a.v[0], ay = a.v[1], az = a.v[2], tx = a.v[3], ty = a.v[4], tz = a.v[5], rr0 = a.v[6];
        T X = cos(ay) * cos(az) * x + (cos(ax) * sin(az) + sin(ax) * sin(ay) * cos(az)) * y +
              (sin(ax) * sin(az) - cos(ax) * sin(ay) * cos(az)) * z;
        T Y = -cos(ay) * sin(az) * x + (cos(ax) * cos(az) - sin(ax) * sin(ay) * sin(az)) * y +
              (sin(ax) * cos(ay) + cos(ax) * sin(ay) * sin(az)) * z;
        T Z = sin(ay) * x - sin(ax) * cos(ay) * y + cos(ax) * cos(ay) * z;
        T s = sqrt((Y - ty) * (Y - ty) + (Z - tz) * (Z - tz));
        T rr = sqrt((X - tx) * (X - tx) + (s + rr0) * (s + rr0));
        T th = atan2(Z - tz, Y - ty);
        T r2 = rr * rr;
        T pd = sqrt(r2 * ((T)0.347 + (T)0.0286 * r2) / ((T)1 + (T)0.3333 * r2 + (T)0.0286 * (r2 * r2)));
        c_t<T> p1 = mk<T>(pd * cos(th), pd * sin(th));
        rr = sqrt((X - tx) * (X - tx) + (s - rr0) * (s - rr0));
        r2 = rr * rr;
        pd = sqrt(r2 * ((T)0.347 + (T)0.0286 * r2) / ((T)1 + (T)0.3333 * r2 + (T)0.0286 * (r2 * r2)));
        c_t<T> p2 = mk<T>(pd * cos(th), -(pd * sin(th)));
        out = cmul_<T>(out, cmul_<T>(p1, p2));
      } break;
      case IK_TF_LINE:
      case IK_TF_RING:
      case IK_TF_NOISE: {  // workload states, FP64 then rounded
        const double X = x, Y = y, Z = z;
        double q = 1.0 - X * X * a.d[1] - Y * Y * a.d[2] - Z * Z * a.d[3];
        double tf = a.d[0] * sqrt(q > 0 ? q : 0.0);
        double re, im;
        if (a.kind == IK_TF_LINE) {
          double rho2 = X * X + Y * Y;
          double f = sqrt(rho2) / sqrt(rho2 + a.d[5]);
          double th = atan2(Y, X);
          re = tf * f * cos(th); im = tf * f * sin(th);
        } else if (a.kind == IK_TF_RING) {
          const double R0 = a.d[4];
          double s = sqrt(X * X + Y * Y);
          double th1 = atan2(Z, s + R0);
          double r1 = sqrt(Z * Z + (s + R0) * (s + R0));
          double th2 = atan2(Z, s - R0);
          double r2 = sqrt(Z * Z + (s - R0) * (s - R0));
          const double c1 = 11.0 / 32.0, c3 = (5.0 - 32.0 * c1) / (48.0 - 192.0 * c1), c2 = c1 * (c3 - 0.25);
          double q1 = r1 * r1, q2 = r2 * r2;
          double p1 = sqrt(q1 * (c1 + c2 * q1) / (1.0 + c3 * q1 + c2 * q1 * q1));
          double p2 = sqrt(q2 * (c1 + c2 * q2) / (1.0 + c3 * q2 + c2 * q2 * q2));
          double amp = tf * p1 * p2;
          double ph = th1 - th2 + a.d[6] * (2.0 * cell_uniform(a.seed, (uint64_t)idx, 0) - 1.0);
          re = amp * cos(ph); im = amp * sin(ph);
        } else {
          re = tf + a.d[6] * (2.0 * cell_uniform(a.seed, (uint64_t)idx, 0) - 1.0);
          im = a.d[6] * (2.0 * cell_uniform(a.seed, (uint64_t)idx, 1) - 1.0);
        }
        out = mk<T>((T)re, (T)im);
      } break;
    }
  }
}

}  // namespace tb
