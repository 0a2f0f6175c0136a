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
  int chunk = 0;         // x-chunk length of the work order (nx: tile-major)
  const void* psi_base[2] = {nullptr, nullptr};
  CUtensorMap tm[2];
  CUtensorMap tmw;       // w (read by stages 2 and 3)
  int* err = nullptr;    // device error flag (owned by the context)
  uint32_t wait_us = 2000000;   // microseconds before a wait gives up
  int inject_wait = 0;   // test hook: waits aim at a phase that never completes
};

// Tile shapes instantiated per precision: {TZ, TY, R, ring slots, CTAs/SM}
// (R = rows per thread; CTAs/SM 0 = chosen from the thread count).
struct Shape { int tz, ty, r, slots, minb; };
constexpr Shape SHAPES_F32[] = {{128, 8, 2, 8, 0}, {64, 8, 2, 8, 0}, {64, 16, 2, 8, 0}, {64, 8, 2, 6, 3}};
constexpr Shape SHAPES_F64[] = {{32, 8, 2, 8, 0}, {64, 8, 2, 8, 0}};
constexpr int NSHAPES_F32 = 4, NSHAPES_F64 = 2;

template <typename T> inline int tiled_nshapes() { return sizeof(T) == 4 ? NSHAPES_F32 : NSHAPES_F64; }
template <typename T> inline Shape tiled_shape(int i) { return sizeof(T) == 4 ? SHAPES_F32[i] : SHAPES_F64[i]; }

// Build a plan for shape index `shape` (0 = default).  Returns 0 when the
// tiled kernel can run this grid with this shape, nonzero otherwise (the
// caller then uses the per-cell kernel).  Defined in tiled_f32.cu / tiled_f64.cu.
template <typename T>
int plan_tiled(const trapbec_params& p, void* const psi[2], void* w, int nsm, int shape, int* err_flag,
               TiledPlan* plan);

// Launch one stage.  kind: StageKind.  a.psi_in must be one of the two psi
// buffers of the plan.  *nblk_out receives the grid size (reduction partials).
template <typename T>
int launch_tiled(const TiledPlan& plan, int kind, const StageArgs<T>& a, cudaStream_t st, int red_cap, int* nblk_out);

}  // namespace tb
