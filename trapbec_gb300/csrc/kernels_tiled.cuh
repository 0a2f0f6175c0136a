// kernels_tiled.cuh -- TMA-staged, register-streaming fused RK3 stage kernel.
//
// One launch performs one stage of the 2N-storage RK3 (run.f90:46-54) over
// the whole grid: rhs = get_rhs(psi) (finite_diff.f90:19-132) fused with the
// w / psi updates, so psi is read once and written once per stage.
//
// Decomposition: the (y, z) plane is cut into TY x TZ tiles; a work unit is
// one tile on one x-plane.  The units (tile-major, x-minor) are split evenly
// over a persistent grid of CTAs, so each CTA streams a contiguous x-range of
// one or two tiles and the load is balanced to within one plane.
//
// Staging: each x-plane of a tile is copied with one TMA box of
// (TZ + 2*HZ) x (TY + 6) complex values (the 3-deep y/z ghost planes
// included) into an S-slot shared-memory ring; slots are guarded by
// mbarriers and refilled S planes ahead (S per stage kind: KindGeom).
// Out-of-range boxes come back zero, which is the reference's 'zero' ghost
// fill (ghost.f90:53-55); for 'solid' and periodic sides the x-plane
// coordinate is remapped before the copy and
// the y/z ghost cells of boundary tiles are patched from global memory.
// The x-direction neighbours live in a 7-deep register queue per thread
// whose rotation is resolved at compile time (the x loop is unrolled by 7).
// FP32 complex arithmetic uses Blackwell's packed f32x2 add/mul/fma.
// Every mbarrier wait is bounded: on timeout the kernel records an error
// code, lets the copies it has in flight land (a wait on each, also bounded)
// and returns.  A test hook (inject_wait) points every wait at an extra
// mbarrier that nothing arrives on, so the timeout path can be exercised
// without a fault.
#pragma once
#include <cuda.h>

#include <type_traits>

#include "common.cuh"
#include "kernels_simple.cuh"
#include "tiled_api.h"

namespace tb {

// ----------------------------------------------------- packed complex ops --
// FP32 complex values are float2 register pairs operated on with Blackwell's
// packed FFMA2/FADD2/FMUL2 (CUDA builtins); FP64 uses scalar pairs.
template <typename T> struct PK;
template <> struct PK<float> {
  using V = float2;
  static __device__ __forceinline__ V add(V a, V b) { return __fadd2_rn(a, b); }
  // a - b as one packed FMA (-1 * b is exact, so the result is the rounded difference)
  static __device__ __forceinline__ V sub(V a, V b) { return __ffma2_rn(make_float2(-1.f, -1.f), b, a); }
  static __device__ __forceinline__ V mul(V a, V b) { return __fmul2_rn(a, b); }
  static __device__ __forceinline__ V fma(V a, V b, V c) { return __ffma2_rn(a, b, c); }
};
template <> struct PK<double> {
  using V = double2;
  static __device__ __forceinline__ V add(V a, V b) { return make_double2(a.x + b.x, a.y + b.y); }
  static __device__ __forceinline__ V sub(V a, V b) { return make_double2(a.x - b.x, a.y - b.y); }
  static __device__ __forceinline__ V mul(V a, V b) { return make_double2(a.x * b.x, a.y * b.y); }
  static __device__ __forceinline__ V fma(V a, V b, V c) {
    return make_double2(::fma(a.x, b.x, c.x), ::fma(a.y, b.y, c.y));
  }
};
template <typename T> __device__ __forceinline__ c_t<T> splat(T s) { return mk<T>(s, s); }
template <typename T> __device__ __forceinline__ T neg(T v) { v.x = -v.x; v.y = -v.y; return v; }

// ------------------------------------------------------------- mbarrier --
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* b, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* b, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* b, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(b)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// Wait for the phase of `parity` to complete; false if `limit_us` microseconds pass first.
__device__ __forceinline__ bool mbar_wait_slow(uint64_t* b, uint32_t parity, uint32_t limit_us) {
  const uint64_t t0 = global_ns();
  const uint64_t lim = (uint64_t)limit_us * 1000u;
  while (!mbar_try_wait(b, parity)) {
    if (global_ns() - t0 > lim) return false;
  }
  return true;
}
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* b, uint32_t parity, uint32_t limit_us) {
  return mbar_try_wait(b, parity) || mbar_wait_slow(b, parity, limit_us);
}
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* tm, int c0, int c1, int c2, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
      ::"r"(smem_u32(dst)), "l"(tm), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// Error codes written to TiledArgs::err.
enum TiledErr : int { TERR_NONE = 0, TERR_WAIT_TIMEOUT = 1, TERR_TOO_MANY_SEGMENTS = 2 };
constexpr uint32_t WAIT_US_DEFAULT = 2000000;  // a wait for TMA data gives up after 2 s

template <typename T> struct TiledArgs {
  StageArgs<T> s;
  int ntz, nty;            // tiles along z and y
  long long units;         // ntz * nty * nx
  int* err;                // error flag (device)
  int bcz;                 // boundary type along z (periodic if zper)
  int fix_y, fix_z;        // ghost fix-up needed on y / z boundary tiles
  int chunk;               // x-chunk length of the work order
  uint32_t wait_us;        // microseconds before a wait gives up (WAIT_US_DEFAULT by default)
  int inject_wait;         // test hook: every wait waits for a phase that never completes
  // Packed coefficients, formed on the host so the kernel can take them from
  // the parameter (constant) bank instead of holding them in registers:
  // 0-2: (2,-27,270)/(180 hx^2), 3-5: y, 6-8: z, 9: -490*sum(1/(180 h^2)),
  // 10: -9, 11: 45, 12: (c_re, c_re), 13: (-c_im, c_im), 14: (A, A), 15: (B, B),
  // 16: (B1, B1) (deferred S2) or (1/B, 1/B) of the previous stage (S2P, S3P)
  c_t<T> k[17];
};

// Float-float (FP32) or Neumaier (FP64) running sums for the fused reductions.
template <typename T> struct RSum;
template <> struct RSum<float> {
  float hi, lo;
  __device__ __forceinline__ void init() { hi = 0.f; lo = 0.f; }
  __device__ __forceinline__ void add(float b) {  // TwoSum
    float s = hi + b;
    float bb = s - hi;
    float e = (hi - (s - bb)) + (b - bb);
    hi = s;
    lo += e;
  }
  __device__ __forceinline__ double val() const { return (double)hi + (double)lo; }
};
template <> struct RSum<double> {
  Acc a;
  __device__ __forceinline__ void init() { a.init(); }
  __device__ __forceinline__ void add(double b) { a.add(b); }
  __device__ __forceinline__ double val() const { return a.val(); }
};

// Float-float pairs (value = hi + lo) for the block trees of the FP32
// reductions.  GB300 issues FP64 at a small fraction of its FP32 rate (about
// one FP64 lane operation per SM clock), so a tree of nine FP64 values over a
// CTA costs ~10 us per flush when two CTAs share an SM; the same tree on
// float-float pairs is FP32 work (TwoSum, renormalised with a second TwoSum,
// ~44 significant bits) and only the CTA's final values are converted.
struct FF {
  float hi, lo;
};
__device__ __forceinline__ FF ff_add(FF a, FF b) {
  const float s = a.hi + b.hi;
  const float bb = s - a.hi;
  const float e = ((a.hi - (s - bb)) + (b.hi - bb)) + (a.lo + b.lo);
  const float h = s + e;
  const float hb = h - s;
  FF r;
  r.hi = h;
  r.lo = (s - (h - hb)) + (e - hb);
  return r;
}

// Block reduction of the fused sums into red[q * nblk + blk] (the layout and
// combination rules of block_reduce_store): FP64 threads go through
// block_reduce_store; FP32 threads reduce their float-float sums with
// shuffles and a fixed order over the warps, in FP32 arithmetic.  With FFOUT
// (FP32 only) each value is stored as a float-float pair (hi, lo) in the
// eight bytes of its double word, for a finaliser that stays in FP32.
template <int NT, bool FFOUT, typename T>
__device__ __forceinline__ void block_reduce_sums(const RSum<T> (&rs)[6], T mx, T mn, bool nf, double* red, int blk,
                                                  int nblk) {
  static_assert(!FFOUT || sizeof(T) == 4, "float-float output is for FP32 sums");
  if constexpr (sizeof(T) == 8) {
    double acc[NRED];
#pragma unroll
    for (int q = 0; q < 6; ++q) acc[q] = rs[q].val();
    acc[6] = (double)mx; acc[7] = (double)mn; acc[8] = nf ? 1.0 : 0.0;
    block_reduce_store<NT>(acc, red, blk, nblk);
  } else {
    constexpr int NW = NT / 32;
    __shared__ FF shf[6][NW];
    __shared__ float shm[3][NW];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    FF v[6];
#pragma unroll
    for (int q = 0; q < 6; ++q) { v[q].hi = rs[q].hi; v[q].lo = rs[q].lo; }
    float fmx = mx, fmn = mn, fnf = nf ? 1.f : 0.f;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
      for (int q = 0; q < 6; ++q) {
        FF y;
        y.hi = __shfl_down_sync(0xffffffffu, v[q].hi, o);
        y.lo = __shfl_down_sync(0xffffffffu, v[q].lo, o);
        v[q] = ff_add(v[q], y);
      }
      fmx = fmaxf(fmx, __shfl_down_sync(0xffffffffu, fmx, o));
      fmn = fminf(fmn, __shfl_down_sync(0xffffffffu, fmn, o));
      fnf = fmaxf(fnf, __shfl_down_sync(0xffffffffu, fnf, o));
    }
    if (lane == 0) {
#pragma unroll
      for (int q = 0; q < 6; ++q) shf[q][wid] = v[q];
      shm[0][wid] = fmx; shm[1][wid] = fmn; shm[2][wid] = fnf;
    }
    __syncthreads();
    if (threadIdx.x < NRED) {
      const int q = threadIdx.x;
      FF x;
      if (q < 6) {
        x = shf[q][0];
        for (int w = 1; w < NW; ++w) x = ff_add(x, shf[q][w]);
      } else {
        x.hi = shm[q - 6][0];
        x.lo = 0.f;
        for (int w = 1; w < NW; ++w) x.hi = (q == 7) ? fminf(x.hi, shm[1][w]) : fmaxf(x.hi, shm[q - 6][w]);
      }
      if constexpr (FFOUT)
        reinterpret_cast<float2*>(red)[(size_t)q * nblk + blk] = make_float2(x.hi, x.lo);
      else
        red[(size_t)q * nblk + blk] = (double)x.hi + (double)x.lo;
    }
  }
}

template <typename T> constexpr int halo_z() { return sizeof(T) == 4 ? 4 : 3; }

template <typename T, int TZ, int TY, int R, int NSLOT = 8, int MINB = 0> struct TileGeom {
  static constexpr int HZ = halo_z<T>();
  static constexpr int TZP = TZ + 2 * HZ;           // row pitch (complex)
  static constexpr int ROWS = TY + 6;
  static constexpr int SLOT_ELEMS = ROWS * TZP;
  static constexpr int SLOT_BYTES = SLOT_ELEMS * (int)sizeof(c_t<T>);   // one psi TMA box
  static constexpr int W_OFF = (SLOT_BYTES + 127) / 128 * 128;           // w tile after the psi box
  static constexpr int W_BYTES = TZ * TY * (int)sizeof(c_t<T>);          // one w TMA box (no ghosts)
  static constexpr int SLOT_STRIDE = (W_OFF + W_BYTES + 127) / 128 * 128; // 128-B aligned slots
  static constexpr int SLOT_STRIDE_ELEMS = SLOT_STRIDE / (int)sizeof(c_t<T>);
  static constexpr int W_OFF_ELEMS = W_OFF / (int)sizeof(c_t<T>);
  static constexpr int NT = TZ * (TY / R);
  static constexpr int S = NSLOT;                   // ring slots
  static constexpr int SMEM = S * SLOT_STRIDE + (S + 1) * 8;
  // CTAs per SM the register allocation is sized for
  static constexpr int MIN_BLOCKS = MINB > 0 ? MINB : ((sizeof(T) == 4 && NT < 512) ? 2 : 1);
};

// Ring of one stage kind, in the shared memory of the shape (G::SMEM) so all
// kinds keep the same CTAs per SM.  Stages 2 and 3 use the shape's slots (psi
// box + w tile).  Kinds that read no w (stage 1, Euler, diagnostics) keep the
// psi box only and as many slots as fit (up to 12): a deeper prefetch.  The
// deferred S2 holds a ghosted w1 box beside the psi box (at least 6 slots).
// S2P and S3P load the previous psi tile where the other stages load w.
template <typename T, class G, int KIND> struct KindGeom {
  static constexpr bool DEFER = (KIND == ST_S2D);
  static constexpr bool NO_W = (KIND == ST_S1 || KIND == ST_S1W || KIND == ST_S1P || KIND == ST_EU || KIND == ST_DIAG);
  static constexpr int W_BYTES = DEFER ? G::SLOT_BYTES : (NO_W ? 0 : G::W_BYTES);
  static constexpr int SLOT_STRIDE =
      DEFER ? (G::W_OFF + G::SLOT_BYTES + 127) / 128 * 128 : (NO_W ? G::W_OFF : G::SLOT_STRIDE);
  static constexpr int SLOT_STRIDE_ELEMS = SLOT_STRIDE / (int)sizeof(c_t<T>);
  static constexpr int FIT_D = (G::S * G::SLOT_STRIDE) / SLOT_STRIDE;
  static constexpr int FIT = (G::SMEM - 8) / (SLOT_STRIDE + 8);
  static constexpr int S = DEFER ? (FIT_D < 6 ? 6 : (FIT_D > G::S ? G::S : FIT_D))
                                 : (NO_W ? (FIT > 12 ? 12 : FIT) : G::S);
  static constexpr int SMEM = S * SLOT_STRIDE + (S + 1) * 8;
  static_assert(DEFER || SMEM <= G::SMEM, "a kind's ring fits the shape's shared memory");
};

// Work description of a batched launch: the concatenated units of all active
// instances, each instance's arguments and tensor maps in a device table.
template <typename T> struct InstDesc {
  CUtensorMap tm[2];       // the two psi buffers
  CUtensorMap tmw;         // w
  TiledArgs<T> ta[2][3];   // [step parity][stage S1, S2, S3]
  const void* buf0;        // psi buffer described by tm[0]
};
struct BatchArgs {
  const void* desc;        // InstDesc<T>[ninst]
  const long long* ustart; // unit prefix sums over the active list, nact + 1 entries
  const int* act;          // active instance ids
  int nact;
  double* part;            // fused-reduction partials, [gridDim][smax][NRED]
  int* part_tag;           // instance of each partial slot, -1 = unused
  int smax;                // partial slots per CTA
  int par;                 // step parity of this launch (selects TiledArgs)
};

// Variants (VAR):
// VAR_PLAIN: the real-time / get_rhs fast path -- no fused reductions, no load
//   factor, harmonic or no potential, rotation or no frame term (the rotation
//   algebra runs with omega = 0 when the frame is off).
// VAR_IMAG: the imaginary-time RK3 stages -- the same compile-time physics,
//   plus the load factor, the converged-loop skip and the reductions fixed by
//   the stage (stage 1 the energy set of the incoming state, stage 3 the norm
//   of the new state, stage 2 none).  Same states, energies and norms as the
//   general variant; the |psi| statistics of Psi_info (partials 5-7), which
//   only diagnostics read, are left at their initial values.
// VAR_GEN: everything else, with run-time switches (array potential,
//   advective frame, diagnostics, any reduction).
// VAR_COMP: the plain variant with a compensated FP32 state.  The stage
//   update psi' = psi + B w (run.f90:48,51,54) is formed as a TwoSum of psi
//   and B w + lo, where lo (a second complex array, read and rewritten at the
//   centre cell only) holds the rounding remainder of the previous update:
//   psi' + lo' equals psi + lo + B w exactly, so increments smaller than half
//   an ulp of psi accumulate in lo instead of being lost.  The stencil reads
//   psi alone, as the reference's get_rhs reads its FP32 Psi.
// BATCH: the units of many independent grids in one launch (batched
// imaginary-time solves); arguments are read per segment from the table.
enum StageVar : int { VAR_GEN = 0, VAR_PLAIN = 1, VAR_IMAG = 2, VAR_COMP = 5 };

template <typename T, int TZ, int TY, int R, int NSLOT, int MINB, int KIND, int VAR, bool BATCH>
__global__ void __launch_bounds__(TileGeom<T, TZ, TY, R, NSLOT, MINB>::NT, TileGeom<T, TZ, TY, R, NSLOT, MINB>::MIN_BLOCKS)
stage_tiled_kernel(const __grid_constant__ CUtensorMap tm0, const __grid_constant__ CUtensorMap tmw0,
                   const __grid_constant__ TiledArgs<T> ta0, const __grid_constant__ BatchArgs ba) {
  using G = TileGeom<T, TZ, TY, R, NSLOT, MINB>;
  using K = KindGeom<T, G, KIND>;
  using P = PK<T>;
  using V = c_t<T>;
  constexpr int HZ = G::HZ, TZP = G::TZP, S = K::S, NT = G::NT;
  // the psi-difference stages S2P / S3P read the previous psi tile in the w slot
  constexpr bool PDIFF = (KIND == ST_S1P || KIND == ST_S2P || KIND == ST_S3P);
  constexpr bool READS_W = (KIND == ST_S2 || KIND == ST_S3 || KIND == ST_S2D || KIND == ST_S2P || KIND == ST_S3P);
  constexpr bool COMP = (VAR == VAR_COMP);   // a plain variant whose update carries the remainder
  constexpr bool PLAIN = (VAR == VAR_PLAIN) || COMP, IMAG = (VAR == VAR_IMAG), GEN = (VAR == VAR_GEN);
  static_assert(!COMP || (!BATCH && (KIND == ST_S1 || KIND == ST_S2 || KIND == ST_S3)),
                "the compensated state is for the real-time RK3 stages");
  constexpr bool ANALYTIC = PLAIN || IMAG;   // harmonic / no potential, rotation / no frame
  static_assert(!K::DEFER || PLAIN, "the deferred stage has a plain variant only");
  static_assert(!PDIFF || (VAR == VAR_PLAIN && !BATCH), "the psi-difference stages have a plain variant only");
  static_assert(!IMAG || KIND == ST_S1 || KIND == ST_S2 || KIND == ST_S3, "imaginary-time variant: RK3 stages only");
  // the queue preload waits for planes xa-3 .. xa+2, all issued before it
  static_assert(S >= 6, "the ring needs at least 6 slots");

  extern __shared__ __align__(128) unsigned char smem_raw[];
  // batched launches: the current grid's arguments, staged from the device table
  __shared__ typename std::conditional<BATCH, TiledArgs<T>, char>::type targs_s;
  V* ring = reinterpret_cast<V*>(smem_raw);
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem_raw + S * K::SLOT_STRIDE);   // S slots + 1 never-completed

  const int tid = threadIdx.x;
  const int lz = tid % TZ;
  const int yg = tid / TZ;

  if (!BATCH) {  // a converged single-instance loop does nothing
    T sc;
    if (!PLAIN && stage_skip(ta0.s, &sc)) return;
  }

  if (tid == 0) {
    for (int s = 0; s <= S; ++s) mbar_init(&bars[s], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();

  RSum<T> rs[6];   // norm, kinetic, potential, quartic, rotation, sum |psi|
  RSum<T>&rN = rs[0], &rK = rs[1], &rP = rs[2], &rQ = rs[3], &rR = rs[4], &rA = rs[5];
  rN.init(); rK.init(); rP.init(); rQ.init(); rR.init(); rA.init();
  // max/min |psi| in the state precision (FP64 operations are slow on GB300)
  T mx = (T)0, mn = (T)3.0e38;
  bool nf = false;
  int nseg = 0;        // partial slots used (batched launches)
  int cur_inst = -1;   // grid whose sums the accumulators hold (batched launches)
  bool cur_red = false;  // this launch reduces (stage kinds with fused sums)
  int* cur_err = nullptr;
  // Store the accumulators as one partial slot tagged with its grid, then reset.
  auto flush = [&](int* errp) {
    if (nseg < ba.smax) {
      const int slot = blockIdx.x * ba.smax + nseg;
      block_reduce_sums<NT, BATCH && sizeof(T) == 4>(rs, mx, mn, nf, ba.part + (size_t)slot * NRED, 0, 1);
      if (tid == 0) ba.part_tag[slot] = cur_inst;
    } else if (tid == 0) {
      atomicExch(errp, (int)TERR_TOO_MANY_SEGMENTS);
    }
    ++nseg;
    rN.init(); rK.init(); rP.init(); rQ.init(); rR.init(); rA.init();
    mx = (T)0; mn = (T)3.0e38; nf = false;
    __syncthreads();
  };

  const long long total = BATCH ? ba.ustart[ba.nact] : ta0.units;
  // Strided order (single grids, chunk < 0): segments of -chunk x-planes in
  // (x-chunk, z-tile, y-tile) order, dealt round-robin over the CTAs, so the
  // CTAs stream neighbouring tiles over the same x-range at the same time and
  // the ghost rows two tiles share are read from DRAM once, then from L2.  On
  // a grid of more tiles than CTAs the contiguous order below streams a tile's
  // neighbours at other times, and their shared rows come from DRAM twice.
  const bool strided = !BATCH && ta0.chunk < 0;
  const long long nsegs =   // strided: segments of the whole grid
      strided ? (long long)((ta0.s.nx - ta0.chunk - 1) / (-ta0.chunk)) * ta0.ntz * ta0.nty : 0;
  const long long G0 = strided ? (long long)blockIdx.x : (long long)blockIdx.x * total / gridDim.x;
  const long long G1 = strided ? nsegs : (long long)(blockIdx.x + 1) * total / gridDim.x;
  uint32_t seq = 0;       // load sequence number of the first plane of a segment
  uint32_t seq_issue = 0; // next sequence number to issue (thread 0)
  bool failed = false;

  for (long long g0 = G0; g0 < G1;) {
    // ---- which grid this segment belongs to -------------------------------
    const TiledArgs<T>* tap = &ta0;
    const CUtensorMap* tmp = &tm0;
    const CUtensorMap* tmwp = &tmw0;
    long long ubase = 0, uend = G1;
    int inst = 0;
    if (BATCH) {
      int k = 0;
      while (k + 1 < ba.nact && ba.ustart[k + 1] <= g0) ++k;
      inst = ba.act[k];
      const InstDesc<T>* d = static_cast<const InstDesc<T>*>(ba.desc) + inst;
      tap = &d->ta[ba.par][KIND == ST_S2 ? 1 : (KIND == ST_S3 ? 2 : 0)];
      tmp = ((const void*)tap->s.psi_in == d->buf0) ? &d->tm[0] : &d->tm[1];
      tmwp = &d->tmw;
      ubase = ba.ustart[k];
      uend = ba.ustart[k + 1] < G1 ? ba.ustart[k + 1] : G1;
      if constexpr (BATCH) {
        // read the arguments from shared memory: they are reloaded after each
        // barrier instead of holding ~40 registers for the whole segment.  The
        // barrier before the copy keeps it from overwriting the previous
        // segment's copy while slower threads still read it: a segment of a
        // converged grid is skipped right after its arguments are read, with
        // no barrier of its own.
        __syncthreads();
        const int* src = reinterpret_cast<const int*>(tap);
        int* dst = reinterpret_cast<int*>(&targs_s);
        for (int e = tid; e < (int)(sizeof(TiledArgs<T>) / 4); e += NT) dst[e] = src[e];
        __syncthreads();
        tap = &targs_s;
      }
    }
    const TiledArgs<T>& ta = *tap;
    const StageArgs<T>& a = ta.s;
    const long long u0 = g0 - ubase;                 // unit within this grid
    if (BATCH && !PLAIN && inst != cur_inst) {       // new grid: hand over the previous grid's sums
      if (cur_inst >= 0 && cur_red) flush(cur_err);
      cur_inst = inst;
      cur_red = IMAG ? (KIND == ST_S1 || KIND == ST_S3) : (a.reduce != 0 || KIND == ST_DIAG);
      cur_err = ta.err;
    }
    T scale = (T)1;
    bool skip = false;
    if (BATCH) skip = stage_skip(a, &scale);
    else if (!PLAIN) stage_skip(a, &scale);
    const int nx = a.nx, ny = a.ny, nz = a.nz;
    const int L = ta.chunk;

    const V vscale = splat<T>(scale);
    const T oms = (ANALYTIC && a.frame_mode == FRAME_NONE) ? (T)0 : a.omega * scale;
    const bool rot = ANALYTIC || a.frame_mode == FRAME_ROT;
    const bool harm = a.pot_mode == POT_HARM;

    auto plane_src = [&](int p) -> int {  // x coordinate the TMA reads for plane p
      if (p >= 0 && p < nx) return p;
      if (a.bc == TRAPBEC_BC_ZERO) return p;  // out of range -> zero fill
      return map_ghost(p, nx, a.bc);
    };

    // Work units are ordered (z-tile, x-chunk, y-tile, x); with the default
    // chunk = nx this is tile-major order and each CTA streams a contiguous
    // x-range of one or two tiles.
    int tzi, tyi, xa, xb;
    if (strided) {   // g0 is the segment index
      const int Ls = -L;
      const long long per_x = (long long)ta.ntz * ta.nty;
      const int xc = (int)(g0 / per_x);
      const long long rem = g0 - (long long)xc * per_x;
      tzi = (int)(rem / ta.nty);
      tyi = (int)(rem - (long long)tzi * ta.nty);
      xa = xc * Ls;
      xb = min(xa + Ls, nx);
      g0 += gridDim.x;
    } else {
      const long long per_tz = (long long)ta.nty * nx;
      tzi = (int)(u0 / per_tz);
      const long long rr0 = u0 - (long long)tzi * per_tz;
      const int xc = (int)(rr0 / ((long long)ta.nty * L));
      const long long rr1 = rr0 - (long long)xc * ta.nty * L;
      const int Lc = min(L, nx - xc * L);
      tyi = (int)(rr1 / Lc);
      xa = xc * L + (int)(rr1 - (long long)tyi * Lc);
      xb = xc * L + Lc;
      if (g0 + (xb - xa) > uend) xb = xa + (int)(uend - g0);
      g0 += xb - xa;
    }
    if (skip) continue;   // converged grid in a batch: nothing to do, nothing loaded

    const int z0 = tzi * TZ;
    const int y0 = tyi * TY;
    const int gz = z0 + lz;
    const bool zok = gz < nz;
    const bool bnd_y = ta.fix_y && (y0 == 0 || y0 + TY >= ny);
    const bool bnd_z = ta.fix_z && (z0 == 0 || z0 + TZ >= nz);
    // the x loop runs in groups of 7 planes (compile-time queue rotation);
    // planes past xb in the last group are computed but not stored
    const int nit = (xb - xa + 6) / 7;
    const int xe = xa + 7 * nit;   // end of the computed range
    const int plast = xe + 2;      // last plane loaded for this segment
    const uint32_t base = seq;     // sequence number of plane xa - 3
    const int c0 = (int)(sizeof(T) == 4 ? (z0 - HZ) : 2 * (z0 - HZ));
    const int cw = (int)(sizeof(T) == 4 ? z0 : 2 * z0);

    // per-thread constants of this tile
    T pyv[R];
    V myv1[R];   // (-y/(60 hx), -y/(60 hx)) for the rotation term
    bool yok[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int gy = y0 + yg * R + r;
      yok[r] = gy < ny;
      pyv[r] = (yok[r] && harm) ? a.py[gy] : (T)0;
      myv1[r] = splat<T>(yok[r] ? -a.yy[gy] * a.ix1 : (T)0);
    }
    const T pzv = (zok && harm) ? a.pz[gz] : (T)0;

    // One ring slot = the psi box of plane p and, for stages that read w,
    // the w tile of plane p (only planes this segment stores); the deferred
    // S2 loads the ghosted w1 box of every plane instead.
    auto issue = [&](int p) {
      const uint32_t sq = seq_issue++;
      const int sl = sq % S;
      const bool with_w = K::DEFER || (READS_W && p >= xa && p < xb);
      V* dst = ring + (size_t)sl * K::SLOT_STRIDE_ELEMS;
      fence_proxy_async();
      mbar_expect_tx(&bars[sl], G::SLOT_BYTES + (with_w ? K::W_BYTES : 0));
      tma_load_3d(dst, tmp, c0, y0 - 3, plane_src(p), &bars[sl]);
      if (K::DEFER) tma_load_3d(dst + G::W_OFF_ELEMS, tmwp, c0, y0 - 3, plane_src(p), &bars[sl]);
      else if (with_w) tma_load_3d(dst + G::W_OFF_ELEMS, tmwp, cw, y0, p, &bars[sl]);
    };
    if (tid == 0) {
      seq_issue = base;
      for (int p = xa - 3; p <= plast && p < xa - 3 + S; ++p) issue(p);
    }

    auto wait_plane = [&](uint32_t sq) {
      const int sl = ta.inject_wait ? S : (int)(sq % S);
      const uint32_t par = ta.inject_wait ? 0u : (sq / S) & 1u;
      if (!mbar_wait_bounded(&bars[sl], par, ta.wait_us)) {
        failed = true;
        atomicExch(ta.err, (int)TERR_WAIT_TIMEOUT);
      }
    };

    // Patch the y/z ghost cells of a boundary tile's slot from global memory
    // (solid mirror or periodic wrap; zero where map_ghost says so).
    auto fixup = [&](uint32_t sq, int p) {
      V* sl = ring + (size_t)(sq % S) * K::SLOT_STRIDE_ELEMS;
      const int xp = plane_src(p);
      if (xp < 0 || xp >= nx) return;  // zero plane
      const size_t plane = (size_t)xp * ny;
      if (bnd_y) {
        for (int e = tid; e < 6 * TZ; e += NT) {
          const int rr = e / TZ, cz = e % TZ;
          const int ry = rr < 3 ? rr - 3 : TY + rr - 3;
          const int gy = y0 + ry, gzz = z0 + cz;
          if ((gy >= 0 && gy < ny) || gzz >= nz) continue;
          const int my = map_ghost(gy, ny, a.bc);
          V v = mk<T>((T)0, (T)0);
          if (my >= 0) v = a.psi_in[(plane + my) * nz + gzz];
          sl[(ry + 3) * TZP + cz + HZ] = v;
        }
      }
      if (bnd_z) {
        for (int e = tid; e < 6 * TY; e += NT) {
          const int ry = e / 6, m = e % 6;
          const int cz = m < 3 ? m - 3 : TZ + m - 3;
          const int gy = y0 + ry, gzz = z0 + cz;
          if ((gzz >= 0 && gzz < nz) || gy >= ny) continue;
          const int mz = map_ghost(gzz, nz, ta.bcz);
          V v = mk<T>((T)0, (T)0);
          if (mz >= 0) v = a.psi_in[(plane + gy) * nz + mz];
          sl[(ry + 3) * TZP + cz + HZ] = v;
        }
      }
    };

    // register queue: at plane x, q[(x - xa + j) % 7][r] holds plane x - 3 + j
    V q[7][R];
    const int qoff = (yg * R + 3) * TZP + lz + HZ;   // first cell of this thread in a slot

    // Deferred S2: psi1 = psi0 + B1*w1 (the FMA stage 1 would have stored)
    // into the psi box of slot sq (plane p): this thread's own centre cells,
    // returned in v[], and, for a plane that will be a centre plane, its share
    // of the y and z ghost cells.  Ghost cells of boundary tiles come from
    // global psi0 and w1 as in fixup().  Every cell is formed by one thread
    // and read by others only after the __syncthreads() that ends the plane.
    auto prepare = [&](uint32_t sq, int p, bool ghosts, V* v) {
      V* sl = ring + (size_t)(sq % S) * K::SLOT_STRIDE_ELEMS;
      const V* swb = sl + G::W_OFF_ELEMS;
      const V kb = ta.k[16];
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const int cell = qoff + r * TZP;
        v[r] = P::fma(kb, swb[cell], sl[cell]);
        sl[cell] = v[r];
      }
      if (!ghosts) return;
      const int xp = plane_src(p);
      const bool zplane = xp < 0 || xp >= nx;   // zero plane: both boxes came back zero
      const size_t plane = (size_t)(zplane ? 0 : xp) * ny;
      for (int e = tid; e < 6 * TZ; e += NT) {
        const int rr = e / TZ, cz = e % TZ;
        const int ry = rr < 3 ? rr - 3 : TY + rr - 3;
        const int cell = (ry + 3) * TZP + cz + HZ;
        const int gy = y0 + ry, gzz = z0 + cz;
        V val;
        if (bnd_y && !zplane && !(gy >= 0 && gy < ny) && gzz < nz) {
          const int my = map_ghost(gy, ny, a.bc);
          val = mk<T>((T)0, (T)0);
          if (my >= 0) {
            const size_t gi = (plane + my) * nz + gzz;
            val = P::fma(kb, a.w_in[gi], a.psi_in[gi]);
          }
        } else {
          val = P::fma(kb, swb[cell], sl[cell]);
        }
        sl[cell] = val;
      }
      for (int e = tid; e < 6 * TY; e += NT) {
        const int ry = e / 6, m = e % 6;
        const int cz = m < 3 ? m - 3 : TZ + m - 3;
        const int cell = (ry + 3) * TZP + cz + HZ;
        const int gy = y0 + ry, gzz = z0 + cz;
        V val;
        if (bnd_z && !zplane && !(gzz >= 0 && gzz < nz) && gy < ny) {
          const int mz = map_ghost(gzz, nz, ta.bcz);
          val = mk<T>((T)0, (T)0);
          if (mz >= 0) {
            const size_t gi = (plane + gy) * nz + mz;
            val = P::fma(kb, a.w_in[gi], a.psi_in[gi]);
          }
        } else {
          val = P::fma(kb, swb[cell], sl[cell]);
        }
        sl[cell] = val;
      }
    };
#pragma unroll
    for (int j = 0; j < 6; ++j) {
      const uint32_t sq = base + j;
      wait_plane(sq);
      if (K::DEFER) {
        V v[R];
        prepare(sq, xa - 3 + j, j >= 3, v);
#pragma unroll
        for (int r = 0; r < R; ++r) q[j][r] = v[r];
      } else {
        if (j >= 3 && (bnd_y || bnd_z)) fixup(sq, xa - 3 + j);
        const V* sl = ring + (size_t)(sq % S) * K::SLOT_STRIDE_ELEMS;
#pragma unroll
        for (int r = 0; r < R; ++r) q[j][r] = sl[qoff + r * TZP];
      }
    }
    // generic-proxy writes of prepare() before the ring's next TMA writes
    if (K::DEFER) fence_proxy_async();
    __syncthreads();
    // a slot is refilled only after its previous copy was waited for: once a
    // wait of the issuing thread gave up, nothing more is issued
    if (tid == 0 && !failed) {
      for (int j = 0; j < 3; ++j) {
        const int p = xa - 3 + j + S;
        if (p > plast) break;
        issue(p);
      }
    }

    const size_t plane_stride = (size_t)ny * nz;
    size_t rowbase = ((size_t)xa * ny + (y0 + yg * R)) * nz + gz;
    // compensated state: the remainders of the next plane, loaded one plane
    // ahead (streaming: each is read once) so that a plane's compute hides
    // their latency
    [[maybe_unused]] V lo_nx[COMP ? R : 1];
    if constexpr (COMP) {
#pragma unroll
      for (int r = 0; r < R; ++r)
        lo_nx[r] = (xa < xb && zok && yok[r]) ? __ldcs(a.lo + rowbase + (size_t)r * nz) : mk<T>((T)0, (T)0);
    }
    // x / (60 hy) and the x part of the trap, loaded one plane ahead
    T xnext = a.xx[xa] * a.iy1;
    T pnext = harm ? a.px[xa] : (T)0;

    auto body = [&](auto offc, int x) {
      constexpr int OFF = decltype(offc)::value;
      const bool store = x < xb;
      const uint32_t sqx = base + (uint32_t)(x - xa) + 3;   // plane x
      const uint32_t sq3 = sqx + 3;                          // plane x + 3
      T tv[R];
#pragma unroll
      for (int r = 0; r < R; ++r) {
        tv[r] = (T)0;
        if (GEN && a.pot_mode == POT_ARR && store && zok && yok[r]) tv[r] = a.trap[rowbase + (size_t)r * nz];
      }
      // compensated state: this plane's remainders (loaded during the previous
      // plane), used by the update at the end of the plane; the next plane's
      // are requested now
      [[maybe_unused]] V lov[COMP ? R : 1];
      if constexpr (COMP) {
        const bool nstore = x + 1 < xb;
#pragma unroll
        for (int r = 0; r < R; ++r) {
          lov[r] = lo_nx[r];
          lo_nx[r] = (nstore && zok && yok[r]) ? __ldcs(a.lo + rowbase + plane_stride + (size_t)r * nz)
                                               : mk<T>((T)0, (T)0);
        }
      }
      const V xv1 = splat<T>(xnext);
      const T pxv = pnext;
      {
        const int xn = x + 1 < nx ? x + 1 : nx - 1;
        xnext = a.xx[xn] * a.iy1;
        pnext = harm ? a.px[xn] : (T)0;
      }
      wait_plane(sq3);
      if (K::DEFER) {
        V v[R];
        prepare(sq3, x + 3, true, v);
        fence_proxy_async();
#pragma unroll
        for (int r = 0; r < R; ++r) q[(OFF + 6) % 7][r] = v[r];
      } else {
        if (bnd_y || bnd_z) fixup(sq3, x + 3);
        const V* sl3 = ring + (size_t)(sq3 % S) * K::SLOT_STRIDE_ELEMS;
#pragma unroll
        for (int r = 0; r < R; ++r) q[(OFF + 6) % 7][r] = sl3[qoff + r * TZP];
      }
      const V* slx = ring + (size_t)(sqx % S) * K::SLOT_STRIDE_ELEMS;
      const V* col = slx + qoff;
      // y column: 3 ghost rows above, R centres (from the queue), 3 below
      V yc[R + 6];
#pragma unroll
      for (int j = 0; j < 3; ++j) yc[j] = col[(j - 3) * TZP];
#pragma unroll
      for (int r = 0; r < R; ++r) yc[r + 3] = q[(OFF + 3) % 7][r];
#pragma unroll
      for (int j = 0; j < 3; ++j) yc[R + 3 + j] = col[(R + j) * TZP];
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const V craw = q[(OFF + 3) % 7][r];
        const V xm3 = q[(OFF + 0) % 7][r], xm2 = q[(OFF + 1) % 7][r], xm1 = q[(OFF + 2) % 7][r];
        const V xp1 = q[(OFF + 4) % 7][r], xp2 = q[(OFF + 5) % 7][r], xp3 = q[(OFF + 6) % 7][r];
        const V ym3 = yc[r], ym2 = yc[r + 1], ym1 = yc[r + 2];
        const V yp1 = yc[r + 4], yp2 = yc[r + 5], yp3 = yc[r + 6];
        const V* zr = col + r * TZP;
        // The stencil in difference form, sum_j k_j ((v_-j - c) + (v_+j - c)):
        // equal to the centre-weighted form in exact arithmetic, but
        // neighbouring values of a resolved field differ by little, so the
        // differences are exact or nearly so and the rounding scales with the
        // Laplacian itself instead of with the partial sums (490/180 h^-2 |psi|
        // per axis cancelling to |lap psi|).
        auto lap_diff = [&]() {
          V d = P::mul(ta.k[0], P::add(P::sub(xm3, craw), P::sub(xp3, craw)));
          d = P::fma(ta.k[1], P::add(P::sub(xm2, craw), P::sub(xp2, craw)), d);
          d = P::fma(ta.k[2], P::add(P::sub(xm1, craw), P::sub(xp1, craw)), d);
          d = P::fma(ta.k[3], P::add(P::sub(ym3, craw), P::sub(yp3, craw)), d);
          d = P::fma(ta.k[4], P::add(P::sub(ym2, craw), P::sub(yp2, craw)), d);
          d = P::fma(ta.k[5], P::add(P::sub(ym1, craw), P::sub(yp1, craw)), d);
          d = P::fma(ta.k[6], P::add(P::sub(zr[-3], craw), P::sub(zr[3], craw)), d);
          d = P::fma(ta.k[7], P::add(P::sub(zr[-2], craw), P::sub(zr[2], craw)), d);
          d = P::fma(ta.k[8], P::add(P::sub(zr[-1], craw), P::sub(zr[1], craw)), d);
          return d;
        };
        V lap;
        if constexpr (COMP) {
          // the compensated form also takes the more accurate stencil: its
          // point is FP32 results close to FP64 ones
          lap = lap_diff();
        } else {
          // the reference's form (deriv.f90:19-25): the centre term and the
          // symmetric pairs, accumulated with FMAs
          lap = P::mul(ta.k[9], craw);
          lap = P::fma(ta.k[0], P::add(xm3, xp3), lap);
          lap = P::fma(ta.k[1], P::add(xm2, xp2), lap);
          lap = P::fma(ta.k[2], P::add(xm1, xp1), lap);
          lap = P::fma(ta.k[3], P::add(ym3, yp3), lap);
          lap = P::fma(ta.k[4], P::add(ym2, yp2), lap);
          lap = P::fma(ta.k[5], P::add(ym1, yp1), lap);
          lap = P::fma(ta.k[6], P::add(zr[-3], zr[3]), lap);
          lap = P::fma(ta.k[7], P::add(zr[-2], zr[2]), lap);
          lap = P::fma(ta.k[8], P::add(zr[-1], zr[1]), lap);
        }
        V fr = mk<T>((T)0, (T)0);
        if (ANALYTIC || a.frame_mode != FRAME_NONE) {
          // D1 without 1/(60h): (v3 - v-3) - 9 (v2 - v-2) + 45 (v1 - v-1)
          V dx = P::sub(xp3, xm3);
          dx = P::fma(ta.k[10], P::sub(xp2, xm2), dx);
          dx = P::fma(ta.k[11], P::sub(xp1, xm1), dx);
          V zc;
          if (rot) {
            V dy = P::sub(yp3, ym3);
            dy = P::fma(ta.k[10], P::sub(yp2, ym2), dy);
            dy = P::fma(ta.k[11], P::sub(yp1, ym1), dy);
            // Z = x D1y - y D1x with the 1/(60h) factors folded into x and y
            zc = P::fma(myv1[r], dx, P::mul(xv1, dy));
          } else {
            zc = P::mul(splat<T>(a.ix1), dx);
          }
          // (0, omega) * Z = (-omega Z.im, omega Z.re), on the renormalised state
          fr = P::mul(mk<T>(zc.y, zc.x), mk<T>(-oms, oms));
        }
        V c = craw;
        if (!PLAIN) {   // everything above is linear in psi: apply the load factor once
          c = P::mul(vscale, craw);
          lap = P::mul(vscale, lap);
        }
        // FP32 energy sums (diagnostics and the imaginary-time loop's energy of
        // stage 1) take the kinetic term from the difference form, which
        // carries the FP32 rounding of the Laplacian itself instead of the
        // ~1e4x larger rounding of the centre-weighted sum; the update keeps
        // the reference's form.  With the centre-weighted sum the energy of a
        // converged FP32 state scatters by a few 1e-10 relative from step to
        // step, which is what an |dE| stop test sees.
        V lapd = lap;
        if constexpr ((KIND == ST_DIAG || (IMAG && KIND == ST_S1)) && sizeof(T) == 4 && !COMP) {
          lapd = lap_diff();
          if (!PLAIN) lapd = P::mul(vscale, lapd);
        }
        T pot = pxv + pyv[r] + pzv;
        if (GEN && a.pot_mode == POT_ARR) pot = tv[r];
        const T a2 = c.x * c.x + c.y * c.y;
        const T rho = (T)1 - a2 - pot;
        const V rhs = P::fma(splat<T>(rho), c, P::add(lap, fr));
        // w = A w + c_f * rhs ; psi' = psi + B w  (run.f90:47-54)
        const V cr = P::fma(ta.k[13], mk<T>(rhs.y, rhs.x), P::mul(ta.k[12], rhs));
        V wn, pn;
        if (KIND == ST_EU) {
          pn = P::add(c, cr);
          wn = cr;
        } else {
          const V wv = K::DEFER ? slx[G::W_OFF_ELEMS + qoff + r * TZP]
                       : READS_W ? slx[G::W_OFF_ELEMS + (yg * R + r) * TZ + lz] : mk<T>((T)0, (T)0);
          if constexpr (KIND == ST_S2P || KIND == ST_S3P) {
            // the previous stage's w from the two psi values: (psi - psi_prev) / B_prev
            wn = P::fma(ta.k[14], P::mul(ta.k[16], P::sub(craw, wv)), cr);
          } else {
            wn = (KIND == ST_S1 || KIND == ST_S1W || KIND == ST_S1P) ? cr : P::fma(ta.k[14], wv, cr);
          }
          pn = P::fma(ta.k[15], wn, c);
        }
        V lon = mk<T>((T)0, (T)0);
        if constexpr (COMP) {
          // TwoSum of psi and the increment B w + lo: pn + lon == c + inc exactly
          const V inc = P::fma(ta.k[15], wn, lov[r]);
          const V sum = P::add(c, inc);
          const V bb = P::sub(sum, c);
          lon = P::add(P::sub(c, P::sub(sum, bb)), P::sub(inc, bb));
          pn = sum;
        }
        if (store && zok && yok[r]) {
          const size_t idx = rowbase + (size_t)r * nz;
          if (KIND == ST_S1 || KIND == ST_S2 || KIND == ST_S1W || KIND == ST_S2D) a.w[idx] = wn;
          if (KIND != ST_DIAG && KIND != ST_S1W) a.psi_out[idx] = pn;
          if constexpr (COMP) __stcs(a.lo + idx, lon);
          if (!PLAIN) {
            if (GEN ? a.reduce == 1 : KIND == ST_S3) rN.add(pn.x * pn.x + pn.y * pn.y);
            if (GEN ? (KIND == ST_DIAG || a.reduce == 2) : KIND == ST_S1) {
              rN.add(a2);
              rK.add(c.x * lapd.x + c.y * lapd.y);
              rP.add(pot * a2);
              rQ.add(a2 * a2);
              rR.add(c.x * fr.x + c.y * fr.y);
              if (GEN) {   // |psi| statistics of Psi_info: diagnostics only, not the imaginary-time loop
                const T am = sqrt(a2);
                rA.add(am);
                mx = fmax(mx, am);
                mn = fmin(mn, am);
              }
              nf |= !isfinite(a2);
            }
          }
        }
      }
      __syncthreads();
      if (tid == 0 && !failed && x + S <= plast) issue(x + S);
      rowbase += plane_stride;
    };

    if constexpr (IMAG && BATCH) {
      // The batched imaginary-time stages (energy and norm sums, per-segment
      // arguments) are long; seven unrolled copies of them overflow the
      // instruction cache (no_instruction was the top stall of a small
      // batch's stage 1) and spilled registers, so they run one copy and shift
      // the x queue by register moves (4 x 128^3: 274 -> 260 us per step;
      // the single-grid loop at 512^3 was 2% faster unrolled).
#pragma unroll 1
      for (int x = xa; x < xe; ++x) {
        body(std::integral_constant<int, 0>{}, x);
#pragma unroll
        for (int j = 0; j < 6; ++j)
#pragma unroll
          for (int r = 0; r < R; ++r) q[j][r] = q[j + 1][r];
      }
    } else {
      for (int x = xa; x < xe; x += 7) {
        body(std::integral_constant<int, 0>{}, x);
        body(std::integral_constant<int, 1>{}, x + 1);
        body(std::integral_constant<int, 2>{}, x + 2);
        body(std::integral_constant<int, 3>{}, x + 3);
        body(std::integral_constant<int, 4>{}, x + 4);
        body(std::integral_constant<int, 5>{}, x + 5);
        body(std::integral_constant<int, 6>{}, x + 6);
      }
    }
    seq = base + (uint32_t)(xe - xa) + 6;
    failed = __syncthreads_or(failed) != 0;
    if (failed) break;
  }

  if (failed && tid == 0) {
    // let every copy this CTA issued land before its shared memory is released:
    // the last S sequence numbers cover all slots; completed phases return at once
    const uint32_t first = seq_issue > (uint32_t)S ? seq_issue - (uint32_t)S : 0u;
    for (uint32_t sq = first; sq < seq_issue; ++sq) (void)mbar_wait_bounded(&bars[sq % S], (sq / S) & 1u, WAIT_US_DEFAULT);
  }

  if (BATCH && !PLAIN && cur_inst >= 0 && cur_red) flush(cur_err);
  if (!BATCH && (GEN || (IMAG && KIND != ST_S2)) && ta0.s.red != nullptr)
    block_reduce_sums<NT, false>(rs, mx, mn, nf, ta0.s.red, blockIdx.x, gridDim.x);
}

}  // namespace tb
