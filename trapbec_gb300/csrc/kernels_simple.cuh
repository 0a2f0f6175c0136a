// kernels_simple.cuh -- per-cell stage kernel, diagnostics reduction and the
// reduction finaliser.
//
// The per-cell kernel is the general path: any grid shape (including the 2D
// mode, odd sizes and grids too small to tile), every boundary type, read
// through the L1/L2 caches with the ghost cells produced by index mapping
// instead of stored ghost planes.  The tiled kernel (kernels_tiled.cuh) is the
// fast path for large 3D grids and must give the same results.
#pragma once
#include "common.cuh"

namespace tb {

constexpr int SIMPLE_THREADS = 256;

// Block-level reduction of NRED accumulators into red[q * nblk + blockIdx.x].
// Sums for q < 6, max for 6, min for 7, max for 8 (nonfinite flag).
template <int NT>
__device__ __forceinline__ void block_reduce_store(double v[NRED], double* red, int blk, int nblk) {
  __shared__ double sh[NRED][NT / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < NRED; ++q) {
    double x = v[q];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      double y = __shfl_down_sync(0xffffffffu, x, o);
      x = (q == 6 || q == 8) ? fmax(x, y) : (q == 7 ? fmin(x, y) : x + y);
    }
    if (lane == 0) sh[q][wid] = x;
  }
  __syncthreads();
  if (threadIdx.x < NRED) {
    const int q = threadIdx.x;
    double x = sh[q][0];
    for (int w = 1; w < NT / 32; ++w) {
      double y = sh[q][w];
      x = (q == 6 || q == 8) ? fmax(x, y) : (q == 7 ? fmin(x, y) : x + y);
    }
    red[(size_t)q * nblk + blk] = x;
  }
}

template <typename T>
__device__ __forceinline__ c_t<T> ld_cell(const StageArgs<T>& a, T scale, int i, int j, int k) {
  int ii = map_ghost(i, a.nx, a.bc);
  int jj = map_ghost(j, a.ny, a.bc);
  int kk = map_ghost(k, a.nz, a.zper ? TRAPBEC_BC_PERIODIC : a.bc);
  if ((ii | jj | kk) < 0) return mk<T>((T)0, (T)0);
  c_t<T> v = a.psi_in[((size_t)ii * a.ny + jj) * a.nz + kk];
  v.x *= scale;
  v.y *= scale;
  return v;
}

// KIND: StageKind, or 4 = diagnostics only (no writes, full reduction).
template <typename T, int KIND>
__global__ void __launch_bounds__(SIMPLE_THREADS) stage_simple_kernel(StageArgs<T> a) {
  T scale;
  if (stage_skip(a, &scale)) return;
  const size_t n = (size_t)a.nx * a.ny * a.nz;
  double acc[NRED];
  Acc sN, sK, sP, sQ, sR, sA;
  sN.init(); sK.init(); sP.init(); sQ.init(); sR.init(); sA.init();
  double mx = 0.0, mn = 1.0e300, nf = 0.0;
  for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n;
       idx += (size_t)gridDim.x * blockDim.x) {
    const int k = (int)(idx % a.nz);
    const size_t r = idx / a.nz;
    const int j = (int)(r % a.ny);
    const int i = (int)(r / a.ny);
    c_t<T> c = a.psi_in[idx];
    c.x *= scale;
    c.y *= scale;
    c_t<T> xm3 = ld_cell(a, scale, i - 3, j, k), xm2 = ld_cell(a, scale, i - 2, j, k), xm1 = ld_cell(a, scale, i - 1, j, k);
    c_t<T> xp1 = ld_cell(a, scale, i + 1, j, k), xp2 = ld_cell(a, scale, i + 2, j, k), xp3 = ld_cell(a, scale, i + 3, j, k);
    c_t<T> ym3 = ld_cell(a, scale, i, j - 3, k), ym2 = ld_cell(a, scale, i, j - 2, k), ym1 = ld_cell(a, scale, i, j - 1, k);
    c_t<T> yp1 = ld_cell(a, scale, i, j + 1, k), yp2 = ld_cell(a, scale, i, j + 2, k), yp3 = ld_cell(a, scale, i, j + 3, k);
    c_t<T> dx2 = d2raw<T>(xm3, xm2, xm1, c, xp1, xp2, xp3);
    c_t<T> dy2 = d2raw<T>(ym3, ym2, ym1, c, yp1, yp2, yp3);
    c_t<T> lap;
    lap.x = dx2.x * a.ix2 + dy2.x * a.iy2;
    lap.y = dx2.y * a.ix2 + dy2.y * a.iy2;
    if (!a.two_dim) {
      c_t<T> zm3 = ld_cell(a, scale, i, j, k - 3), zm2 = ld_cell(a, scale, i, j, k - 2), zm1 = ld_cell(a, scale, i, j, k - 1);
      c_t<T> zp1 = ld_cell(a, scale, i, j, k + 1), zp2 = ld_cell(a, scale, i, j, k + 2), zp3 = ld_cell(a, scale, i, j, k + 3);
      c_t<T> dz2 = d2raw<T>(zm3, zm2, zm1, c, zp1, zp2, zp3);
      lap.x += dz2.x * a.iz2;
      lap.y += dz2.y * a.iz2;
    }
    c_t<T> fr = mk<T>((T)0, (T)0);
    if (a.frame_mode == FRAME_ROT) {
      c_t<T> d1x = d1raw<T>(xm3, xm2, xm1, xp1, xp2, xp3);
      c_t<T> d1y = d1raw<T>(ym3, ym2, ym1, yp1, yp2, yp3);
      T x = a.xx[i], y = a.yy[j];
      T zr = x * (d1y.x * a.iy1) - y * (d1x.x * a.ix1);
      T zi = x * (d1y.y * a.iy1) - y * (d1x.y * a.ix1);
      fr.x = -a.omega * zi;   // (0, omega) * Z
      fr.y = a.omega * zr;
    } else if (a.frame_mode == FRAME_ADV) {
      c_t<T> d1x = d1raw<T>(xm3, xm2, xm1, xp1, xp2, xp3);
      fr.x = -a.omega * (d1x.y * a.ix1);   // (0, 2 vx) * D1x
      fr.y = a.omega * (d1x.x * a.ix1);
    }
    T pot = (T)0;
    if (a.pot_mode == POT_HARM) pot = a.px[i] + a.py[j] + a.pz[k];
    else if (a.pot_mode == POT_ARR) pot = a.trap[idx];
    if (KIND <= ST_EU) {
      c_t<T> wold = mk<T>((T)0, (T)0);
      if (KIND == ST_S2 || KIND == ST_S3) wold = a.w[idx];
      c_t<T> wnew, pnew;
      cell_update<T, KIND>(c, lap, fr, pot, wold, a, wnew, pnew);
      if (KIND == ST_S1 || KIND == ST_S2) a.w[idx] = wnew;
      a.psi_out[idx] = pnew;
      if (a.reduce == 1) {  // norm of the new state
        sN.add((double)pnew.x * pnew.x + (double)pnew.y * pnew.y);
      }
    }
    if (KIND == 4 || a.reduce == 2) {
      double re = c.x, im = c.y;
      double a2 = re * re + im * im;
      sN.add(a2);
      c_t<T> lapk = lap;   // FP32 diagnostics: the kinetic sum takes the difference form of the stencil
      if constexpr (sizeof(T) == 4 && KIND == 4) {
        c_t<T> ex = d2diff<T>(xm3, xm2, xm1, c, xp1, xp2, xp3);
        c_t<T> ey = d2diff<T>(ym3, ym2, ym1, c, yp1, yp2, yp3);
        lapk.x = ex.x * a.ix2 + ey.x * a.iy2;
        lapk.y = ex.y * a.ix2 + ey.y * a.iy2;
        if (!a.two_dim) {
          c_t<T> zm3 = ld_cell(a, scale, i, j, k - 3), zm2 = ld_cell(a, scale, i, j, k - 2), zm1 = ld_cell(a, scale, i, j, k - 1);
          c_t<T> zp1 = ld_cell(a, scale, i, j, k + 1), zp2 = ld_cell(a, scale, i, j, k + 2), zp3 = ld_cell(a, scale, i, j, k + 3);
          c_t<T> ez = d2diff<T>(zm3, zm2, zm1, c, zp1, zp2, zp3);
          lapk.x += ez.x * a.iz2;
          lapk.y += ez.y * a.iz2;
        }
      }
      sK.add(re * (double)lapk.x + im * (double)lapk.y);
      sP.add((double)pot * a2);
      sQ.add(a2 * a2);
      sR.add(re * (double)fr.x + im * (double)fr.y);
      double am = sqrt(a2);
      sA.add(am);
      mx = fmax(mx, am);
      mn = fmin(mn, am);
      if (!isfinite(a2)) nf = 1.0;
    }
  }
  if (a.red == nullptr) return;
  acc[0] = sN.val(); acc[1] = sK.val(); acc[2] = sP.val(); acc[3] = sQ.val();
  acc[4] = sR.val(); acc[5] = sA.val(); acc[6] = mx; acc[7] = mn; acc[8] = nf;
  block_reduce_store<SIMPLE_THREADS>(acc, a.red, blockIdx.x, gridDim.x);
}

// Reduce the [NRED][nblk] partials to NRED values, in a fixed order so the
// result is bitwise reproducible run to run.
constexpr int FIN_THREADS = 512;

// Combination rule of reduction slot q: sums (0-5), max (6, 8), min (7).
__device__ __forceinline__ double fin_op(int q, double z, double y) {
  return (q == 6 || q == 8) ? fmax(z, y) : (q == 7 ? fmin(z, y) : z + y);
}

// One thread's running values of the NRED quantities.  A thread combines a
// few partials (each already a CTA's compensated sum), so plain FP64 adds in
// a fixed order lose nothing measurable, while a compensated add per partial
// was most of a one-block finaliser's time on GB300, whose FP64 issue rate
// is about one lane operation per SM clock.
struct FinAcc {
  double s[6];
  double mx6, mn7, mx8;
  __device__ __forceinline__ void init() {
#pragma unroll
    for (int q = 0; q < 6; ++q) s[q] = 0.0;
    mx6 = 0.0; mn7 = 1.0e300; mx8 = 0.0;
  }
  __device__ __forceinline__ void add(const double* v) {   // v[NRED] of one partial
#pragma unroll
    for (int q = 0; q < 6; ++q) s[q] += v[q];
    mx6 = fmax(mx6, v[6]);
    mn7 = fmin(mn7, v[7]);
    mx8 = fmax(mx8, v[8]);
  }
};

// Combine the FIN_THREADS threads' values with a fixed pairwise tree (thread
// t takes t + s at every level s = 256 ... 1: shared memory down to 32, warp
// shuffles below, the same pairs either way); out[] is written by thread 0.
__device__ __forceinline__ void fin_tree(const FinAcc& a, double* out) {
  __shared__ double sh[NRED][FIN_THREADS];
  const int t = threadIdx.x;
#pragma unroll
  for (int q = 0; q < 6; ++q) sh[q][t] = a.s[q];
  sh[6][t] = a.mx6;
  sh[7][t] = a.mn7;
  sh[8][t] = a.mx8;
  __syncthreads();
  for (int s = FIN_THREADS / 2; s >= 32; s >>= 1) {
    if (t < s) {
#pragma unroll
      for (int q = 0; q < NRED; ++q) sh[q][t] = fin_op(q, sh[q][t], sh[q][t + s]);
    }
    __syncthreads();
  }
  if (t < 32) {
    double x[NRED];
#pragma unroll
    for (int q = 0; q < NRED; ++q) x[q] = sh[q][t];
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) {
#pragma unroll
      for (int q = 0; q < NRED; ++q) x[q] = fin_op(q, x[q], __shfl_down_sync(0xffffffffu, x[q], s));
    }
    if (t == 0) {
#pragma unroll
      for (int q = 0; q < NRED; ++q) out[q] = x[q];
    }
  }
  __syncthreads();
}

// Called by all FIN_THREADS threads of one block: combines the block partials
// red[q * nblk + b] (thread t takes b = t, t + FIN_THREADS, ... in order, then
// the fixed tree); out[] is written by thread 0.
__device__ __forceinline__ void finalize_partials(const double* __restrict__ red, int nblk, double* out) {
  FinAcc a;
  a.init();
  for (int b = threadIdx.x; b < nblk; b += FIN_THREADS) {
    double v[NRED];
#pragma unroll
    for (int q = 0; q < NRED; ++q) v[q] = red[(size_t)q * nblk + b];
    a.add(v);
  }
  fin_tree(a, out);
}

static __global__ void __launch_bounds__(FIN_THREADS) reduce_finalize_kernel(const double* __restrict__ red,
                                                                      int nblk, double* __restrict__ out) {
  finalize_partials(red, nblk, out);
}

// psi *= s (applies a pending renormalisation to the stored state).
template <typename T>
__global__ void scale_kernel(c_t<T>* __restrict__ psi, size_t n, T s) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    c_t<T> v = psi[i];
    v.x *= s;
    v.y *= s;
    psi[i] = v;
  }
}

// dst = src for a state array of n16 16-byte words and, when tail8, one
// trailing 8-byte word (a complex FP32 array of odd length): the device-side
// half of the overlapped host copies (queued state into psi, psi into the
// read-back snapshot).  Four independent 16-byte loads in flight per thread,
// streaming cache hints (the arrays are far larger than L2).
constexpr int COPY_THREADS = 512, COPY_UNROLL = 4;
static __global__ void __launch_bounds__(COPY_THREADS) copy_state_kernel(const uint4* __restrict__ src,
                                                                   uint4* __restrict__ dst, size_t n16, int tail8) {
  const size_t step = (size_t)gridDim.x * COPY_THREADS * COPY_UNROLL;
  for (size_t base = (size_t)blockIdx.x * COPY_THREADS * COPY_UNROLL + threadIdx.x; base < n16; base += step) {
    uint4 v[COPY_UNROLL];
#pragma unroll
    for (int u = 0; u < COPY_UNROLL; ++u) {
      const size_t j = base + (size_t)u * COPY_THREADS;
      if (j < n16) v[u] = __ldcs(src + j);
    }
#pragma unroll
    for (int u = 0; u < COPY_UNROLL; ++u) {
      const size_t j = base + (size_t)u * COPY_THREADS;
      if (j < n16) __stcs(dst + j, v[u]);
    }
  }
  if (tail8 && blockIdx.x == 0 && threadIdx.x == 0)
    *reinterpret_cast<uint2*>(dst + n16) = *reinterpret_cast<const uint2*>(src + n16);
}

}  // namespace tb
