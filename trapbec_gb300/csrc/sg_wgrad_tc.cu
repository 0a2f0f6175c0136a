// sg_wgrad_tc.cu -- weight gradients of the surrogate's 3x3x3 convolutions
// on the 5th-generation tensor cores (tcgen05.mma, accumulator in TMEM).
//
//   dW[tap][co][ci] = sum over voxels v of dZ[v][co] * X[v + tap][ci]
//
// is a GEMM whose reduction (K) runs over voxels, so both operands are
// MN-major in channels-last memory.  Per 1 x 16 x 8 brick of voxels (K = 128,
// ordered w-column by w-column, 16 h values each):
//  - A = dZ of the brick, M = output channels.  One TMA box per 8-channel
//    chunk lands as [w][h][8 ch]: 8 consecutive h of one column are one
//    MN-major core matrix (128 contiguous bytes), the next 8 h are 128 bytes
//    on (K-group stride), the next 8 channels one chunk (2 KB) on.
//  - B = the input halo (3 x 18 x 10 voxels) of two 8-channel chunks,
//    N = (kw, chunk, kd, 8 channels).  One TMA box per brick, through a
//    tensor map of one sample whose dimensions are ordered (8 channels, h, d,
//    chunk, w), lands as [w][chunk][d][h][8 ch]: for a fixed kh the 18
//    (kw, chunk, kd) groups of a column are 18 core matrices 288 bytes apart
//    (d stride = 18 h rows, chunk stride = 3 d planes, w stride = 2 chunks),
//    so ONE descriptor covers all nine taps of both chunks: N = 144 per MMA,
//    and kh is a start-address shift.
// So a brick costs 8 columns x 3 kh = 24 MMAs of M x 144 x 16 into three
// accumulator blocks (432 TMEM columns) that stay in TMEM for the CTA's
// whole brick range; the epilogue reads them out once.  M is 64 for up to 64
// output channels (the rows beyond Cout read other shared memory of the
// stage and are discarded) and 128 for 128.  A pass covers two input-channel
// chunks (16 channels); the grid's y dimension takes the other passes.
//
// Warp roles: warp 0 issues the TMA loads into a ring of stages, warp 1 the
// MMAs (one thread), warps 2-5 the bias gradient (sum of dZ per channel, from
// the staged tiles, pass 0 only) and, at the end, the TMEM read-out.  Per-CTA
// partials go to scratch and are summed in a fixed order by a reduction
// kernel, so gradients are bitwise reproducible.  Every wait is bounded in
// time; TMEM is always released.
#include <cstring>

#include "../../include/trapbec_surrogate.h"
#include "sg_tc_common.cuh"

namespace sg {
namespace wtc {

using namespace tcc;

constexpr int BH = 16, BW = 8;                  // brick: 16 h x 8 w voxels (one d plane)
constexpr int XD = 3, XH = BH + 2, XW = BW + 2;
constexpr int XBOX = 2 * XD * XH * XW * 16;     // 17280 bytes: the halo of two 8-channel chunks
constexpr int XBOX_PAD = 17408;                 // 128-byte multiple
constexpr int ZCHUNK = BH * BW * 16;            // 2048 bytes: one 8-channel chunk of dZ
constexpr int NTHR = 192;
constexpr int NG = 18;                          // (kw, chunk, kd) groups of one MMA
constexpr int NMMA = NG * 8;                    // N = 144
constexpr int MAXB = 8;                         // samples per launch (one halo tensor map each)

__device__ int g_timeout = 0;

template <int CIN, int COUT> struct Cfg {
  static constexpr int KCO = COUT / 8;
  static constexpr int M = COUT > 64 ? 128 : 64;
  static constexpr int ACC_COLS = 3 * NMMA;     // blocks kh = 0..2: 432 of 512 columns
  static constexpr int Z_BYTES = KCO * ZCHUNK;
  static constexpr int STAGE = Z_BYTES + XBOX_PAD;
  static constexpr int TAIL = 1024;
  static constexpr int NS = (4 * STAGE + TAIL + 1024 <= 220 * 1024) ? 4 : 3;
  static constexpr int BAR_OFF = NS * STAGE + TAIL;
  static constexpr int RED_OFF = BAR_OFF + 256;
  static constexpr int SMEM = RED_OFF + 128 * 4;
  static_assert(CIN % 16 == 0 && COUT % 16 == 0 && COUT <= 128, "channels");
  static_assert(ACC_COLS <= 512, "TMEM columns");
  // the A operand of M = 64 reads 8 chunks of 2 KB from a stage's dZ tile on
  static_assert(M == 128 || STAGE >= 8 * ZCHUNK, "spare A rows stay inside the stage");
};

struct Args {
  float* part;     // [gridDim.x][27][COUT][CIN]
  float* part_b;   // [gridDim.x][COUT] or null
  int B, D, H, W;
};

// the halo tensor maps, one per sample
struct XMaps {
  CUtensorMap m[MAXB];
};

template <int CIN, int COUT>
__global__ void __launch_bounds__(NTHR, 1)
    conv3_wgrad_tc_kernel(const __grid_constant__ XMaps tmx, const __grid_constant__ CUtensorMap tmz, Args a) {
  using C = Cfg<CIN, COUT>;
  constexpr int NS = C::NS;
  extern __shared__ __align__(1024) unsigned char smem[];
  const uint32_t s0 = smem_u32(smem);
  const uint32_t full0 = s0 + C::BAR_OFF, empty0 = full0 + 8 * NS, done = empty0 + 8 * NS;
  uint32_t* taddr_s = (uint32_t*)(smem + C::BAR_OFF + 8 * (2 * NS + 1));
  float* red = (float*)(smem + C::RED_OFF);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int pass = blockIdx.y;
  const bool do_bias = pass == 0 && a.part_b != nullptr;

  const int nbw = (a.W + BW - 1) / BW, nbh = (a.H + BH - 1) / BH;
  const long long nbr = (long long)a.B * a.D * nbh * nbw;
  const long long b0 = nbr * blockIdx.x / gridDim.x, b1 = nbr * (blockIdx.x + 1) / gridDim.x;
  const int nmine = (int)(b1 - b0);   // >= 1: the grid never exceeds the brick count

  if (tid == 0) {
    for (int s = 0; s < NS; ++s) { bar_init(full0 + 8 * s, 1); bar_init(empty0 + 8 * s, 1 + 4); }
    bar_init(done, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(taddr_s)),
                 "r"(512));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t taddr = *taddr_s;
  bool ok = true;

  if (warp == 0) {
    // ---- TMA producer ---------------------------------------------------------------
    if (lane == 0) {
      for (int j = 0; j < nmine && ok; ++j) {
        const int s = j % NS;
        if (j >= NS) ok = bar_wait(empty0 + 8 * s, (uint32_t)((j / NS - 1) & 1));
        if (!ok) break;
        long long r = b0 + j;
        const int bw = (int)(r % nbw); r /= nbw;
        const int bh = (int)(r % nbh); r /= nbh;
        const int d = (int)(r % a.D), b = (int)(r / a.D);
        const uint32_t st = s0 + s * C::STAGE;
        bar_expect_tx(full0 + 8 * s, (uint32_t)(C::Z_BYTES + XBOX));
        for (int kc = 0; kc < C::KCO; ++kc)
          tma_load_5d(st + kc * ZCHUNK, &tmz, kc * 8, bh * BH, bw * BW, d, b, full0 + 8 * s);
        tma_load_5d(st + C::Z_BYTES, &tmx.m[b], 0, bh * BH - 1, d - 1, 2 * pass, bw * BW - 1, full0 + 8 * s);
      }
      // let the last loads land before the CTA can end
      for (int j = nmine - NS > 0 ? nmine - NS : 0; j < nmine; ++j)
        (void)bar_wait(full0 + 8 * (j % NS), (uint32_t)((j / NS) & 1));
    }
  } else if (warp == 1) {
    // ---- MMA issuer -------------------------------------------------------------------
    if (lane == 0) {
      constexpr uint32_t IDESC = idesc_bf16(C::M, NMMA, 1, 1);
      for (int j = 0; j < nmine && ok; ++j) {
        const int s = j % NS;
        ok = bar_wait(full0 + 8 * s, (uint32_t)((j / NS) & 1));
        if (!ok) break;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t st = s0 + s * C::STAGE;
        // A: dZ column w; K groups (8 h rows) 128 bytes apart, M groups (8 channels) one chunk apart
        const uint64_t ad0 = sdesc(st, 128, ZCHUNK);
        // B: halo rows; K groups 128 bytes apart, N groups (kw, chunk, kd) 18 h rows = one d step apart
        const uint64_t bd0 = sdesc(st + C::Z_BYTES, 128, XH * 16);
#pragma unroll
        for (int w = 0; w < BW; ++w) {
          const uint64_t ad = ad0 + (uint64_t)(w * BH);   // start address in 16-byte units
#pragma unroll
          for (int kh = 0; kh < 3; ++kh) {
            const uint64_t bd = bd0 + (uint64_t)(w * 2 * XD * XH + kh);
            const uint32_t acc = (j | w) ? 1u : 0u;
            mma_bf16_ss(taddr + (uint32_t)(kh * NMMA), ad, bd, IDESC, acc);
          }
        }
        mma_commit(empty0 + 8 * s);   // the stage is free once these MMAs are done
      }
      if (ok) mma_commit(done);
    }
  } else {
    // ---- bias gradient, stage release, and the final read-out: warps 2..5 ----------------
    const int et = tid - 64;                     // 0..127
    constexpr int G = 128 / COUT;                // voxel groups per channel
    const int co = et % COUT, grp = et / COUT;
    float bsum = 0.f;
    for (int j = 0; j < nmine && ok; ++j) {
      const int s = j % NS;
      ok = bar_wait(full0 + 8 * s, (uint32_t)((j / NS) & 1));
      if (!__all_sync(0xffffffffu, ok)) { ok = false; break; }
      if (do_bias) {
        const bf16* z = (const bf16*)(smem + s * C::STAGE + (co >> 3) * ZCHUNK) + (co & 7);
        constexpr int NV = 128 / G;
        for (int v = grp * NV; v < (grp + 1) * NV; ++v) bsum += __bfloat162float(z[v * 8]);
      }
      __syncwarp();
      if (lane == 0) bar_arrive(empty0 + 8 * s);
    }
    if (do_bias) {
      red[et] = bsum;
      asm volatile("bar.sync 1, 128;" ::: "memory");
      if (et < COUT) {
        float t = 0.f;
        for (int g = 0; g < G; ++g) t += red[g * COUT + et];
        a.part_b[(size_t)blockIdx.x * COUT + et] = t;
      }
    }
    // accumulator read-out: this warp's TMEM lane quarter
    const int q = warp & 3;
    if (ok) ok = bar_wait(done, 0);
    if (__all_sync(0xffffffffu, ok)) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      // the accumulator row (output channel) in this thread's lane: M = 128
      // keeps row r in lane r, M = 64 rows 16q..16q+15 in lanes 32q..32q+15
      int row = -1;
      if (C::M == 128) row = q * 32 + lane;
      else if (lane < 16) row = q * 16 + lane;
      const bool mine = row >= 0 && row < COUT;
      float* out = a.part + (size_t)blockIdx.x * 27 * COUT * CIN;
#pragma unroll 1
      for (int kh = 0; kh < 3; ++kh) {
#pragma unroll 1
        for (int g = 0; g < NG; ++g) {
          uint32_t r[8];
          tmem_ld8(taddr + ((uint32_t)(q * 32) << 16) + (uint32_t)(kh * NMMA + g * 8), r);
          tmem_wait_ld();
          if (mine) {
            const int kw = g / 6, c = (g / 3) & 1, kd = g % 3;
            const int tap = (kd * 3 + kh) * 3 + kw;
            float4* o = (float4*)(out + ((size_t)tap * COUT + row) * CIN + (2 * pass + c) * 8);
            o[0] = make_float4(__uint_as_float(r[0]), __uint_as_float(r[1]), __uint_as_float(r[2]),
                               __uint_as_float(r[3]));
            o[1] = make_float4(__uint_as_float(r[4]), __uint_as_float(r[5]), __uint_as_float(r[6]),
                               __uint_as_float(r[7]));
          }
        }
      }
    } else {
      ok = false;
    }
  }
  if (!ok) atomicExch(&g_timeout, 1);
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 1) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(512));
}

// out[i] = sum of the CTAs' partials in CTA order, for the weights (i < nw)
// and then the biases (nb more, from part_b); the loads of sixteen CTAs are
// issued together (one memory latency per sixteen, same summation order),
// and 64-thread blocks spread the outputs over more SMs
__global__ void reduce_parts_kernel(const float* part, const float* part_b, int nchunk, size_t nw, size_t nb,
                                    float* out_w, float* out_b) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < nw + nb; i += (size_t)gridDim.x * blockDim.x) {
    const bool w = i < nw;
    const float* p = w ? part + i : part_b + (i - nw);
    const size_t n = w ? nw : nb;
    float s = 0.f;
    int c = 0;
    for (; c + 16 <= nchunk; c += 16) {
      float v[16];
#pragma unroll
      for (int j = 0; j < 16; ++j) v[j] = p[(size_t)(c + j) * n];
#pragma unroll
      for (int j = 0; j < 16; ++j) s += v[j];
    }
    for (; c < nchunk; ++c) s += p[(size_t)c * n];
    if (w) out_w[i] = s;
    else out_b[i - nw] = s;
  }
}

inline int sm_count() {
  static int nsm = 0;
  if (!nsm) {
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    nsm = v > 0 ? v : 1;
  }
  return nsm;
}

// CTAs along x (brick ranges) for cin/16 passes: about one CTA per SM in all,
// never more than the brick count
inline int nchunks(int cin, int B, int D, int H, int W) {
  const long long nbr = (long long)B * D * ((H + BH - 1) / BH) * ((W + BW - 1) / BW);
  const int passes = cin / 16;
  const long long want = (sm_count() + passes - 1) / passes;
  return (int)(nbr < want ? nbr : want);
}

template <int CIN, int COUT>
int launch(const bf16* x, const bf16* dz, int B, int D, int H, int W, float* dw, float* db, float* scratch,
           cudaStream_t st) {
  using C = Cfg<CIN, COUT>;
  // at least half an SM's shared memory, so that one CTA holds an SM and its
  // 512 TMEM columns (a second CTA on the SM would wait in tcgen05.alloc)
  constexpr int SMEM = C::SMEM > 116 * 1024 ? C::SMEM : 116 * 1024;
  static bool attr = false;
  if (!attr) {
    if (cudaFuncSetAttribute(conv3_wgrad_tc_kernel<CIN, COUT>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM) !=
        cudaSuccess)
      return TBSG_ERR_CUDA;
    attr = true;
  }
  auto enc = encoder();
  if (!enc) return TBSG_ERR_CUDA;
  XMaps tmx;
  CUtensorMap tmz;
  std::memset(&tmx, 0, sizeof(tmx));
  for (int b = 0; b < B; ++b) {
    // sample b of X [B][D][H][W][CIN] seen as (8 channels, h, d, chunk, w): a box of two chunks lands
    // [w][chunk][d][h][8 ch]
    const bf16* xb = x + (size_t)b * D * H * W * CIN;
    cuuint64_t dims[5] = {8, (cuuint64_t)H, (cuuint64_t)D, (cuuint64_t)(CIN / 8), (cuuint64_t)W};
    cuuint64_t strides[4] = {(cuuint64_t)W * CIN * 2, (cuuint64_t)H * W * CIN * 2, 16, (cuuint64_t)CIN * 2};
    cuuint32_t box[5] = {8, (cuuint32_t)XH, (cuuint32_t)XD, 2, (cuuint32_t)XW};
    cuuint32_t es[5] = {1, 1, 1, 1, 1};
    if (enc(&tmx.m[b], CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, (void*)xb, dims, strides, box, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return TBSG_ERR_ARG;
  }
  {  // dZ [B][D][H][W][COUT] seen as (c, h, w, d, b): boxes land [w][h][8 ch]
    cuuint64_t dims[5] = {(cuuint64_t)COUT, (cuuint64_t)H, (cuuint64_t)W, (cuuint64_t)D, (cuuint64_t)B};
    cuuint64_t strides[4] = {(cuuint64_t)W * COUT * 2, (cuuint64_t)COUT * 2, (cuuint64_t)H * W * COUT * 2,
                             (cuuint64_t)D * H * W * COUT * 2};
    cuuint32_t box[5] = {8, (cuuint32_t)BH, (cuuint32_t)BW, 1, 1};
    cuuint32_t es[5] = {1, 1, 1, 1, 1};
    if (enc(&tmz, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, (void*)dz, dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
            CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) !=
        CUDA_SUCCESS)
      return TBSG_ERR_ARG;
  }
  const int nch = nchunks(CIN, B, D, H, W);
  Args a;
  a.part = scratch;
  a.part_b = db ? scratch + (size_t)nch * 27 * COUT * CIN : nullptr;
  a.B = B; a.D = D; a.H = H; a.W = W;
  conv3_wgrad_tc_kernel<CIN, COUT><<<dim3(nch, CIN / 16, 1), NTHR, SMEM, st>>>(tmx, tmz, a);
  const size_t nw = (size_t)27 * COUT * CIN, nb = db ? (size_t)COUT : 0;
  reduce_parts_kernel<<<(int)((nw + nb + 63) / 64), 64, 0, st>>>(a.part, a.part_b, nch, nw, nb, dw, db);
  return cudaGetLastError() == cudaSuccess ? TBSG_OK : TBSG_ERR_CUDA;
}

}  // namespace wtc

size_t wgrad_tc_scratch_bytes(int cin, int cout, int batch, int D, int H, int W) {
  const int nch = wtc::nchunks(cin, batch, D, H, W);
  return ((size_t)nch * 27 * cout * cin + (size_t)nch * cout) * sizeof(float);
}

// tcgen05 weight gradients; TBSG_ERR_SHAPE for pairs not built here
int wgrad_tc(const void* x, int cin, const void* dz, int cout, int batch, int D, int H, int W, float* dw, float* db,
             void* scratch, cudaStream_t st) {
  if ((uintptr_t)x % 16 || (uintptr_t)dz % 16 || (uintptr_t)scratch % 16) return TBSG_ERR_SHAPE;
  if (batch > wtc::MAXB) return TBSG_ERR_SHAPE;   // the mma.sync kernel takes larger batches
  const bf16* xb = (const bf16*)x;
  const bf16* zb = (const bf16*)dz;
  float* s = (float*)scratch;
#define SG_WTC(I, O) \
  if (cin == I && cout == O) return wtc::launch<I, O>(xb, zb, batch, D, H, W, dw, db, s, st);
  SG_WTC(16, 16) SG_WTC(16, 32) SG_WTC(32, 16) SG_WTC(32, 32) SG_WTC(32, 64) SG_WTC(64, 32) SG_WTC(64, 64)
  SG_WTC(64, 128) SG_WTC(128, 64) SG_WTC(128, 128)
#undef SG_WTC
  return TBSG_ERR_SHAPE;
}

// whether a weight-gradient launch gave up waiting (and clear the flag)
int wgrad_tc_timed_out(int* v) {
  if (cudaMemcpyFromSymbol(v, wtc::g_timeout, sizeof(int)) != cudaSuccess) return TBSG_ERR_CUDA;
  if (*v) {
    int z = 0;
    if (cudaMemcpyToSymbol(wtc::g_timeout, &z, sizeof(int)) != cudaSuccess) return TBSG_ERR_CUDA;
  }
  return TBSG_OK;
}

}  // namespace sg
