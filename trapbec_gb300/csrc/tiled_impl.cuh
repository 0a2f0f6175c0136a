// tiled_impl.cuh -- plan and launch of the tiled stage kernel, instantiated
// per precision by tiled_f32.cu and tiled_f64.cu.
#pragma once
#include <cudaTypedefs.h>

#include <cstring>
#include <utility>

#include "kernels_tiled.cuh"

namespace tb {

inline PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (PFN_cuTensorMapEncodeTiled_v12000)f;
  }
  return fn;
}

// Packed stencil/update coefficients of TiledArgs::k from the StageArgs.
template <typename T> inline void fill_coeffs(TiledArgs<T>& ta) {
  auto pr = [](T v) { return mk<T>(v, v); };
  const StageArgs<T>& a = ta.s;
  const T ix2 = a.ix2, iy2 = a.iy2, iz2 = a.iz2;
  ta.k[0] = pr((T)2 * ix2); ta.k[1] = pr((T)(-27) * ix2); ta.k[2] = pr((T)270 * ix2);
  ta.k[3] = pr((T)2 * iy2); ta.k[4] = pr((T)(-27) * iy2); ta.k[5] = pr((T)270 * iy2);
  ta.k[6] = pr((T)2 * iz2); ta.k[7] = pr((T)(-27) * iz2); ta.k[8] = pr((T)270 * iz2);
  ta.k[9] = pr((T)(-490) * (ix2 + iy2 + (a.two_dim ? (T)0 : iz2)));
  ta.k[10] = pr((T)(-9)); ta.k[11] = pr((T)45);
  ta.k[12] = pr(a.c_re); ta.k[13] = mk<T>(-a.c_im, a.c_im);
  ta.k[14] = pr(a.A); ta.k[15] = pr(a.B);
  ta.k[16] = pr(a.B1);
}

// One TMA descriptor over an (nx, ny, nz) complex array: a box with the
// 3-deep ghost frame (ghosted) or an interior tile.
template <typename T, int TZ, int TY, int R, int NS, int MB>
int encode_box(const trapbec_params& p, void* base, bool ghosted, CUtensorMap* map) {
  using G = TileGeom<T, TZ, TY, R, NS, MB>;
  auto enc = tensor_map_encoder();
  if (!enc) return 2;
  cuuint64_t dims[3], strides[2];
  cuuint32_t box[3], es[3] = {1, 1, 1};
  // FP32: one 8-byte element = one complex float; FP64: a complex double is two doubles
  dims[0] = sizeof(T) == 4 ? (cuuint64_t)p.nz : (cuuint64_t)p.nz * 2;
  const int bz = ghosted ? G::TZP : TZ;
  box[0] = sizeof(T) == 4 ? bz : 2 * bz;
  dims[1] = (cuuint64_t)p.ny;
  dims[2] = (cuuint64_t)p.nx;
  strides[0] = (cuuint64_t)p.nz * sizeof(c_t<T>);
  strides[1] = (cuuint64_t)p.ny * p.nz * sizeof(c_t<T>);
  box[1] = ghosted ? G::ROWS : TY;
  box[2] = 1;
  CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, base, dims, strides, box, es,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? 0 : 3;
}

// TMA descriptors of one grid: the two psi buffers (boxes with the 3-deep
// ghost frame) and w (interior tiles).
template <typename T, int TZ, int TY, int R, int NS, int MB>
int encode_maps(const trapbec_params& p, void* const psi[2], void* w, CUtensorMap* tm, CUtensorMap* tmw) {
  for (int b = 0; b < 2; ++b)
    if (int rc = encode_box<T, TZ, TY, R, NS, MB>(p, psi[b], true, &tm[b])) return rc;
  return encode_box<T, TZ, TY, R, NS, MB>(p, w, false, tmw);
}

template <typename T, int TZ, int TY, int R, int NS, int MB>
int plan_shape(const trapbec_params& p, void* const psi[2], void* w, void* w2, int nsm, int* err_flag,
               TiledPlan* plan) {
  using G = TileGeom<T, TZ, TY, R, NS, MB>;
  if (p.two_dim || p.nx < 4 || p.ny < 4 || p.nz < 8) return 1;
  if (sizeof(T) == 4 && (p.nz % 2)) return 1;  // TMA strides must be multiples of 16 bytes
  const int bcz = (p.periodicz || p.boundaries == TRAPBEC_BC_PERIODIC) ? TRAPBEC_BC_PERIODIC : p.boundaries;
  const int fix_y = p.boundaries != TRAPBEC_BC_ZERO;
  const int fix_z = bcz != TRAPBEC_BC_ZERO;
  // ghost fix-ups address the tile edges: partial tiles only with zero ghosts
  if (fix_y && (p.ny % TY)) return 1;
  if (fix_z && (p.nz % TZ)) return 1;
  TiledPlan q;
  if (int rc = encode_maps<T, TZ, TY, R, NS, MB>(p, psi, w, q.tm, &q.tmw)) return rc;
  q.psi_base[0] = psi[0];
  q.psi_base[1] = psi[1];
  q.w_base[0] = w;
  q.w_base[1] = nullptr;
  auto k1 = stage_tiled_kernel<T, TZ, TY, R, NS, MB, ST_S1, false, false>;
  auto k2 = stage_tiled_kernel<T, TZ, TY, R, NS, MB, ST_S2, false, false>;
  auto k3 = stage_tiled_kernel<T, TZ, TY, R, NS, MB, ST_S3, false, false>;
  auto k4 = stage_tiled_kernel<T, TZ, TY, R, NS, MB, ST_EU, false, false>;
  auto k5 = stage_tiled_kernel<T, TZ, TY, R, NS, MB, ST_DIAG, false, false>;
  auto k6 = stage_tiled_kernel<T, TZ, TY, R, NS, MB, ST_S1, true, false>;
  auto k7 = stage_tiled_kernel<T, TZ, TY, R, NS, MB, ST_S2, true, false>;
  auto k8 = stage_tiled_kernel<T, TZ, TY, R, NS, MB, ST_S3, true, false>;
  auto k9 = stage_tiled_kernel<T, TZ, TY, R, NS, MB, ST_S1, VAR_IMAG, false>;
  auto k10 = stage_tiled_kernel<T, TZ, TY, R, NS, MB, ST_S2, VAR_IMAG, false>;
  auto k11 = stage_tiled_kernel<T, TZ, TY, R, NS, MB, ST_S3, VAR_IMAG, false>;
  const int sm_s1 = KindGeom<T, G, ST_S1>::SMEM, sm_eu = KindGeom<T, G, ST_EU>::SMEM;
  const int sm_dg = KindGeom<T, G, ST_DIAG>::SMEM;
  const std::pair<const void*, int> ks[] = {{(const void*)k1, sm_s1}, {(const void*)k2, G::SMEM},
                                            {(const void*)k3, G::SMEM}, {(const void*)k4, sm_eu},
                                            {(const void*)k5, sm_dg}, {(const void*)k6, sm_s1},
                                            {(const void*)k7, G::SMEM}, {(const void*)k8, G::SMEM},
                                            {(const void*)k9, sm_s1}, {(const void*)k10, G::SMEM},
                                            {(const void*)k11, G::SMEM}};
  for (const auto& k : ks)
    if (cudaFuncSetAttribute(k.first, cudaFuncAttributeMaxDynamicSharedMemorySize, k.second) != cudaSuccess) return 4;
  // the compensated-state real-time stages (FP32, two rows per thread: the
  // remainders take registers that four-row tiles do not have)
  if constexpr (sizeof(T) == 4 && R <= 2) {
    auto kc1 = stage_tiled_kernel<T, TZ, TY, R, NS, MB, ST_S1, VAR_COMP, false>;
    auto kc2 = stage_tiled_kernel<T, TZ, TY, R, NS, MB, ST_S2, VAR_COMP, false>;
    auto kc3 = stage_tiled_kernel<T, TZ, TY, R, NS, MB, ST_S3, VAR_COMP, false>;
    if (cudaFuncSetAttribute(kc1, cudaFuncAttributeMaxDynamicSharedMemorySize, sm_s1) != cudaSuccess ||
        cudaFuncSetAttribute(kc2, cudaFuncAttributeMaxDynamicSharedMemorySize, G::SMEM) != cudaSuccess ||
        cudaFuncSetAttribute(kc3, cudaFuncAttributeMaxDynamicSharedMemorySize, G::SMEM) != cudaSuccess)
      return 4;
  }
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k2, G::NT, G::SMEM) != cudaSuccess || nb < 1) return 5;
  // the psi-difference real-time form: no w array; S2P / S3P load the
  // previous psi array's interior tiles where S2 / S3 load w
  {
    auto kp1 = stage_tiled_kernel<T, TZ, TY, R, NS, MB, ST_S1P, VAR_PLAIN, false>;
    auto kp2 = stage_tiled_kernel<T, TZ, TY, R, NS, MB, ST_S2P, VAR_PLAIN, false>;
    auto kp3 = stage_tiled_kernel<T, TZ, TY, R, NS, MB, ST_S3P, VAR_PLAIN, false>;
    int nbp = 0;
    q.pdiff_ok = encode_box<T, TZ, TY, R, NS, MB>(p, psi[0], false, &q.tmpi[0]) == 0 &&
                 encode_box<T, TZ, TY, R, NS, MB>(p, psi[1], false, &q.tmpi[1]) == 0 &&
                 cudaFuncSetAttribute(kp1, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      KindGeom<T, G, ST_S1P>::SMEM) == cudaSuccess &&
                 cudaFuncSetAttribute(kp2, cudaFuncAttributeMaxDynamicSharedMemorySize, G::SMEM) == cudaSuccess &&
                 cudaFuncSetAttribute(kp3, cudaFuncAttributeMaxDynamicSharedMemorySize, G::SMEM) == cudaSuccess &&
                 cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nbp, kp2, G::NT, G::SMEM) == cudaSuccess &&
                 nbp >= nb;
    cudaGetLastError();   // a refused attribute only disables this form
  }
  // the deferred real-time form (FP32): S1 stores w1 only, S2 forms psi1 from
  // ghosted boxes of psi0 and w1 and writes w2 to the second w buffer
  q.defer_ok = 0;
  if constexpr (sizeof(T) == 4) {
    if (w2) {
      auto kw = stage_tiled_kernel<T, TZ, TY, R, NS, MB, ST_S1W, true, false>;
      auto kd = stage_tiled_kernel<T, TZ, TY, R, NS, MB, ST_S2D, true, false>;
      constexpr int SMEM_D = KindGeom<T, G, ST_S2D>::SMEM;
      int nbd = 0;
      if (encode_box<T, TZ, TY, R, NS, MB>(p, w, true, &q.tmwg) == 0 &&
          encode_box<T, TZ, TY, R, NS, MB>(p, w2, false, &q.tmw1) == 0 &&
          cudaFuncSetAttribute(kw, cudaFuncAttributeMaxDynamicSharedMemorySize, KindGeom<T, G, ST_S1W>::SMEM) ==
              cudaSuccess &&
          cudaFuncSetAttribute(kd, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_D) == cudaSuccess &&
          cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nbd, kd, G::NT, SMEM_D) == cudaSuccess && nbd >= nb) {
        q.w_base[1] = w2;
        q.defer_ok = 1;
      }
    }
  }
  cudaGetLastError();   // a refused attribute only disables the deferred form
  q.ntz = (p.nz + TZ - 1) / TZ;
  q.nty = (p.ny + TY - 1) / TY;
  q.units = (long long)q.ntz * q.nty * p.nx;
  long long g = (long long)nb * nsm;
  q.grid = (int)(g < q.units ? g : q.units);
  q.smem = G::SMEM;
  q.nt = G::NT;
  q.tz = TZ; q.ty = TY; q.r = R;
  q.comp_ok = (sizeof(T) == 4 && R <= 2) ? 1 : 0;
  q.fix_y = fix_y; q.fix_z = fix_z; q.bcz = bcz;
  q.chunk = p.nx;   // tile-major order until set_chunk chooses otherwise
  q.err = err_flag;
  q.valid = 1;
  *plan = q;
  return 0;
}

template <typename T, int TZ, int TY, int R, int NS, int MB>
int launch_shape(const TiledPlan& plan, int kind, const StageArgs<T>& a, cudaStream_t st, int red_cap, int* nblk) {
  using G = TileGeom<T, TZ, TY, R, NS, MB>;
  TiledArgs<T> ta;
  ta.s = a;
  ta.ntz = plan.ntz;
  ta.nty = plan.nty;
  ta.units = plan.units;
  ta.err = plan.err;
  ta.bcz = plan.bcz;
  ta.fix_y = plan.fix_y;
  ta.fix_z = plan.fix_z;
  const bool stage1 = kind == ST_S1 || kind == ST_S1P || kind == ST_S1W;
  ta.chunk = (stage1 && plan.chunk_s1 != 0) ? plan.chunk_s1 : plan.chunk;
  ta.wait_us = plan.wait_us;
  ta.inject_wait = plan.inject_wait;
  fill_coeffs<T>(ta);
  const CUtensorMap* tm = nullptr;
  if ((const void*)a.psi_in == plan.psi_base[0]) tm = &plan.tm[0];
  else if ((const void*)a.psi_in == plan.psi_base[1]) tm = &plan.tm[1];
  if (!tm) return 6;
  // w tiles come from whichever w buffer a.w is
  const CUtensorMap* tmw = &plan.tmw;
  if (plan.defer_ok && (const void*)a.w == plan.w_base[1]) tmw = &plan.tmw1;
  int grid = plan.grid;
  if (a.red && grid > red_cap) grid = red_cap;
  const bool plain = tiled_plain(a);
  if (kind == ST_S1P || kind == ST_S2P || kind == ST_S3P) {
    if (!plain || !plan.pdiff_ok) return 12;
    if (kind == ST_S1P) {
      stage_tiled_kernel<T, TZ, TY, R, NS, MB, ST_S1P, VAR_PLAIN, false>
          <<<grid, G::NT, KindGeom<T, G, ST_S1P>::SMEM, st>>>(*tm, *tmw, ta, BatchArgs{});
    } else {
      // the previous psi array (a.w_in) is read as interior tiles and receives psi_out
      const CUtensorMap* tmp = nullptr;
      if ((const void*)a.w_in == plan.psi_base[0]) tmp = &plan.tmpi[0];
      else if ((const void*)a.w_in == plan.psi_base[1]) tmp = &plan.tmpi[1];
      if (!tmp || (const void*)a.psi_out != (const void*)a.w_in || a.w_in == a.psi_in) return 12;
      ta.k[16] = mk<T>(a.rB, a.rB);
      if (kind == ST_S2P)
        stage_tiled_kernel<T, TZ, TY, R, NS, MB, ST_S2P, VAR_PLAIN, false><<<grid, G::NT, G::SMEM, st>>>(*tm, *tmp, ta, BatchArgs{});
      else
        stage_tiled_kernel<T, TZ, TY, R, NS, MB, ST_S3P, VAR_PLAIN, false><<<grid, G::NT, G::SMEM, st>>>(*tm, *tmp, ta, BatchArgs{});
    }
    if (nblk) *nblk = grid;
    return cudaGetLastError() == cudaSuccess ? 0 : 8;
  }
  if (kind == ST_S1W || kind == ST_S2D) {
    if constexpr (sizeof(T) == 4) {
      if (!plain || !plan.defer_ok) return 9;
      if (kind == ST_S1W) {
        stage_tiled_kernel<T, TZ, TY, R, NS, MB, ST_S1W, true, false><<<grid, G::NT, KindGeom<T, G, ST_S1W>::SMEM, st>>>(*tm, *tmw, ta, BatchArgs{});
      } else {
        // w1 (ghosted boxes) in, w2 out
        if ((const void*)a.w_in != plan.w_base[0] || (const void*)a.w != plan.w_base[1]) return 10;
        stage_tiled_kernel<T, TZ, TY, R, NS, MB, ST_S2D, true, false>
            <<<grid, G::NT, KindGeom<T, G, ST_S2D>::SMEM, st>>>(*tm, plan.tmwg, ta, BatchArgs{});
      }
      if (nblk) *nblk = grid;
      return cudaGetLastError() == cudaSuccess ? 0 : 8;
    } else {
      return 9;
    }
  }
  if (a.lo != nullptr) {   // compensated-state real-time stages
    if constexpr (sizeof(T) == 4 && R <= 2) {
      if (!plain) return 11;
      if (kind == ST_S1) stage_tiled_kernel<T, TZ, TY, R, NS, MB, ST_S1, VAR_COMP, false><<<grid, G::NT, KindGeom<T, G, ST_S1>::SMEM, st>>>(*tm, *tmw, ta, BatchArgs{});
      else if (kind == ST_S2) stage_tiled_kernel<T, TZ, TY, R, NS, MB, ST_S2, VAR_COMP, false><<<grid, G::NT, G::SMEM, st>>>(*tm, *tmw, ta, BatchArgs{});
      else if (kind == ST_S3) stage_tiled_kernel<T, TZ, TY, R, NS, MB, ST_S3, VAR_COMP, false><<<grid, G::NT, G::SMEM, st>>>(*tm, *tmw, ta, BatchArgs{});
      else return 11;
      if (nblk) *nblk = grid;
      return cudaGetLastError() == cudaSuccess ? 0 : 8;
    } else {
      return 11;
    }
  }
  if (tiled_imag(a, kind)) {
    if (kind == ST_S1) stage_tiled_kernel<T, TZ, TY, R, NS, MB, ST_S1, VAR_IMAG, false><<<grid, G::NT, KindGeom<T, G, ST_S1>::SMEM, st>>>(*tm, *tmw, ta, BatchArgs{});
    else if (kind == ST_S2) stage_tiled_kernel<T, TZ, TY, R, NS, MB, ST_S2, VAR_IMAG, false><<<grid, G::NT, KindGeom<T, G, ST_S2>::SMEM, st>>>(*tm, *tmw, ta, BatchArgs{});
    else stage_tiled_kernel<T, TZ, TY, R, NS, MB, ST_S3, VAR_IMAG, false><<<grid, G::NT, KindGeom<T, G, ST_S3>::SMEM, st>>>(*tm, *tmw, ta, BatchArgs{});
  } else if (plain && kind == ST_S1) {
    stage_tiled_kernel<T, TZ, TY, R, NS, MB, ST_S1, true, false><<<grid, G::NT, KindGeom<T, G, ST_S1>::SMEM, st>>>(*tm, *tmw, ta, BatchArgs{});
  } else if (plain && kind == ST_S2) {
    stage_tiled_kernel<T, TZ, TY, R, NS, MB, ST_S2, true, false><<<grid, G::NT, KindGeom<T, G, ST_S2>::SMEM, st>>>(*tm, *tmw, ta, BatchArgs{});
  } else if (plain && kind == ST_S3) {
    stage_tiled_kernel<T, TZ, TY, R, NS, MB, ST_S3, true, false><<<grid, G::NT, KindGeom<T, G, ST_S3>::SMEM, st>>>(*tm, *tmw, ta, BatchArgs{});
  } else {
    switch (kind) {
      case ST_S1: stage_tiled_kernel<T, TZ, TY, R, NS, MB, ST_S1, false, false><<<grid, G::NT, KindGeom<T, G, ST_S1>::SMEM, st>>>(*tm, *tmw, ta, BatchArgs{}); break;
      case ST_S2: stage_tiled_kernel<T, TZ, TY, R, NS, MB, ST_S2, false, false><<<grid, G::NT, KindGeom<T, G, ST_S2>::SMEM, st>>>(*tm, *tmw, ta, BatchArgs{}); break;
      case ST_S3: stage_tiled_kernel<T, TZ, TY, R, NS, MB, ST_S3, false, false><<<grid, G::NT, KindGeom<T, G, ST_S3>::SMEM, st>>>(*tm, *tmw, ta, BatchArgs{}); break;
      case ST_EU: stage_tiled_kernel<T, TZ, TY, R, NS, MB, ST_EU, false, false><<<grid, G::NT, KindGeom<T, G, ST_EU>::SMEM, st>>>(*tm, *tmw, ta, BatchArgs{}); break;
      case ST_DIAG: stage_tiled_kernel<T, TZ, TY, R, NS, MB, ST_DIAG, false, false><<<grid, G::NT, KindGeom<T, G, ST_DIAG>::SMEM, st>>>(*tm, *tmw, ta, BatchArgs{}); break;
      default: return 7;
    }
  }
  if (nblk) *nblk = grid;
  return cudaGetLastError() == cudaSuccess ? 0 : 8;
}

}  // namespace tb
