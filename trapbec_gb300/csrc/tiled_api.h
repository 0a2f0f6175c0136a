// tiled_api.h -- host-side interface of the tiled stage kernel (plan + launch).
#pragma once
#include <cuda.h>

#include "common.cuh"

namespace tb {

// Launch plan of the tiled kernel for one grid: tile shape, persistent grid
// size, the two TMA descriptors (one per psi buffer) and the boundary fix-up
// switches.
struct TiledPlan {
  int valid = 0;
  int shape = -1;        // index into the shape table of the precision
  int tz = 0, ty = 0, r = 0;
  int grid = 0, smem = 0, nt = 0;
  int ntz = 0, nty = 0;
  long long units = 0;
  int fix_y = 0, fix_z = 0, bcz = 0;
  int chunk = 0;         // x-chunk length of the work order (nx: tile-major; < 0: the strided order)
  int chunk_s1 = 0;      // work order of the stage-1 kinds when it differs (0: chunk)
  const void* psi_base[2] = {nullptr, nullptr};
  const void* w_base[2] = {nullptr, nullptr};   // w, second w buffer (deferred form)
  CUtensorMap tm[2];
  CUtensorMap tmw;       // w (read by stages 2 and 3)
  CUtensorMap tmw1;      // second w buffer, interior tiles (S3 of the deferred form)
  CUtensorMap tmwg;      // w with the ghost frame (deferred S2 reads w1 like psi)
  CUtensorMap tmpi[2];   // the two psi buffers as interior tiles (psi-difference S2P / S3P)
  int defer_ok = 0;      // the deferred real-time form can run (FP32, second w buffer)
  int comp_ok = 0;       // the compensated-state real-time stages are built for this shape
  int pdiff_ok = 0;      // the psi-difference real-time stages can run
  int* err = nullptr;    // device error flag (owned by the context)
  uint32_t wait_us = 2000000;   // microseconds before a wait gives up
  int inject_wait = 0;   // test hook: waits aim at a phase that never completes
};

// Tile shapes instantiated per precision: {TZ, TY, R, ring slots, CTAs/SM}
// (R = rows per thread; CTAs/SM 0 = chosen from the thread count).
struct Shape { int tz, ty, r, slots, minb; };
constexpr Shape SHAPES_F32[] = {{128, 8, 2, 8, 0}, {64, 8, 2, 8, 0}, {64, 16, 2, 8, 0}, {64, 8, 2, 6, 3},
                                {64, 32, 4, 6, 0}};
constexpr Shape SHAPES_F64[] = {{32, 8, 2, 8, 0}, {64, 8, 2, 8, 0}};
constexpr int NSHAPES_F32 = 5, NSHAPES_F64 = 2;
// Default shape of the plain real-time stages: (64 x 32) with 4 rows per thread
// has the fewest ghost rows per box (6 of 38) that fit the shared memory; its
// general variants (reductions) spill, so they keep shape 0.
constexpr int RT_SHAPE_F32 = 4, RT_SHAPE_F64 = 0;
template <typename T> inline int tiled_rt_shape() { return sizeof(T) == 4 ? RT_SHAPE_F32 : RT_SHAPE_F64; }

template <typename T> inline int tiled_nshapes() { return sizeof(T) == 4 ? NSHAPES_F32 : NSHAPES_F64; }
template <typename T> inline Shape tiled_shape(int i) { return sizeof(T) == 4 ? SHAPES_F32[i] : SHAPES_F64[i]; }

// Build a plan for shape index `shape` (0 = default); w2 (may be null) is the
// second w buffer of the deferred real-time form.  Returns 0 when the
// tiled kernel can run this grid with this shape, nonzero otherwise (the
// caller then uses the per-cell kernel).  Defined in tiled_f32.cu / tiled_f64.cu.
template <typename T>
int plan_tiled(const trapbec_params& p, void* const psi[2], void* w, void* w2, int nsm, int shape, int* err_flag,
               TiledPlan* plan);

// Stage arguments the plain variant of the kernel covers: no reductions, no
// load factor, harmonic or no potential, rotation or no frame term, not
// driven by the imaginary-time control block.
template <typename T> inline bool tiled_plain(const StageArgs<T>& a) {
  return a.red == nullptr && a.reduce == 0 && a.ctrl == nullptr && a.scale == (T)1 && a.pot_mode != POT_ARR &&
         a.frame_mode != FRAME_ADV;
}

// Stage arguments the imaginary-time variant covers: an RK3 stage of the
// on-device imaginary-time loop (control block set) with harmonic or no
// potential, rotation or no frame term, and the reduction that stage makes
// in that loop (stage 1 the energy set, stage 2 none, stage 3 the norm).
template <typename T> inline bool tiled_imag(const StageArgs<T>& a, int kind) {
  return a.ctrl != nullptr && a.pot_mode != POT_ARR && a.frame_mode != FRAME_ADV &&
         ((kind == ST_S1 && a.reduce == 2) || (kind == ST_S2 && a.reduce == 0) || (kind == ST_S3 && a.reduce == 1));
}

// Launch one stage.  kind: StageKind.  a.psi_in must be one of the two psi
// buffers of the plan.  *nblk_out receives the grid size (reduction partials).
template <typename T>
int launch_tiled(const TiledPlan& plan, int kind, const StageArgs<T>& a, cudaStream_t st, int red_cap, int* nblk_out);

}  // namespace tb
