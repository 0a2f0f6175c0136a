// sg_conv_tcs.cu -- 3x3x3 convolutions of the surrogate's 64- and 128-channel
// layers (the 32^3 and 16^3 levels, and the 64-channel side of the 64^3
// level) on the 5th-generation tensor cores, with streamed weights.
//
// Implicit GEMM per 1 x 16 x 8 output brick as in sg_conv_tc.cu: M = 128
// voxels, K = 27 taps x Cin, the brick's halo K-chunked in shared memory by
// one TMA box per 8-channel chunk, so every tap's A operand is the same
// K-major descriptor with another start address.  These layers' weights
// (27 x Cin x Cout BF16: 110-884 KB) do not fit in shared memory next to the
// halo, so they stream: one TMA box per (tap, 8-channel chunk) lands the
// tap's [N][8] slice of the CTA's output channels (N = 64, or 32 for 32
// outputs) in a ring of weight stages, K-major with the chunk as the K core
// matrix.  A unit of work is (brick, block of N output channels), so the
// 128-channel layers of the coarse levels, which have few bricks, spread
// over twice as many CTAs.
//
// Warp roles as in the resident-weight kernel: warp 0 issues the TMA loads
// (halo ring and weight ring), warp 1 the MMAs (one thread; 27 x Cin/16 per
// unit into one of two TMEM accumulators), warps 2-5 drain an accumulator
// 16 columns at a time with tcgen05.ld and run the fused bias + skip +
// leaky-ReLU (or FP32 input-gradient) epilogue.  Every wait is bounded in
// time; TMEM is always released.
#include "../../include/trapbec_surrogate.h"
#include "sg_tc_common.cuh"

namespace sg {
namespace tcs {

using namespace tcc;

constexpr int BH = 16, BW = 8;
constexpr int XD = 3, XH = BH + 2;
constexpr int NTHR = 192;
constexpr int SMEM_BUDGET = 225 * 1024;

__device__ int g_timeout = 0;

// BPU bricks per unit, adjacent along w, share every weight slice (the
// weights are streamed once per unit, so two bricks halve the weight bytes
// per output voxel); their halo is one box of width 8 BPU + 2.  A halo
// stage holds GC channel chunks of the unit; the K loop runs over NG = KC/GC
// such groups, each with its 27 weight slices.
template <int CIN, int COUT, int BPU> struct Cfg {
  static constexpr int KC = CIN / 8;
  static constexpr int N = COUT >= 64 ? 64 : COUT;          // output channels of one unit
  static constexpr int NSPLIT = COUT / N;
  static constexpr int XW = BW * BPU + 2;
  static constexpr int XV = XD * XH * XW;                   // halo voxels of the unit
  static constexpr int CHB = (XV * 16 + 127) / 128 * 128;   // one chunk of the halo, 128-byte multiple
  static constexpr int GC = (BPU == 1 || KC <= 4) ? KC : 4; // chunks per halo stage
  static constexpr int NG = KC / GC;
  static constexpr int HALO = GC * CHB;
  static constexpr int WSLICE = GC * N * 16;                // one (tap, group)'s weights of one unit
  static constexpr int NSH = (2 * HALO + 4 * WSLICE + 1024 <= SMEM_BUDGET) ? 2 : 1;
  static constexpr int NSW_FIT = (SMEM_BUDGET - NSH * HALO - 1024) / WSLICE;
  static constexpr int NSW = NSW_FIT > 32 ? 32 : NSW_FIT;   // as deep as fits: the slices come from L2
  static constexpr int W_OFF = NSH * HALO;
  static constexpr int BAR_OFF = W_OFF + NSW * WSLICE;
  // hfull/hempty[NSH], wfull/wempty[NSW], afull/aempty[2], then the TMEM address
  static constexpr int NBAR = 2 * NSH + 2 * NSW + 4;
  static constexpr int SMEM = BAR_OFF + (NBAR * 8 + 4 + 127) / 128 * 128;
  static constexpr int ACC = BPU * N;                       // columns of one accumulator set
  static constexpr uint32_t TMEM_COLS = 2 * ACC < 32 ? 32 : 2 * ACC;
  static_assert(NSW >= 2, "weight ring");
  static_assert(SMEM <= SMEM_BUDGET, "shared memory of one CTA");
  static_assert(COUT % N == 0 && N % 16 == 0 && KC % GC == 0 && GC % 2 == 0, "blocks");
  static_assert(TMEM_COLS <= 512, "TMEM columns");
};

struct Args {
  const bf16* x;       // [B][D][H][W][CIN]
  const bf16* w;       // [27][COUT][CIN]
  const float* bias;
  const bf16* skip;
  bf16* y;
  float* yf;
  int B, D, H, W;
  int act;
  float slope;
  int mode;            // 0: BF16 epilogue, 1: FP32 +=, 2: FP32 =, 3: y = BF16(v act'(yact)), dskip += that
  const bf16* yact;
  float* dskip;
};

template <int CIN, int COUT, int BPU>
__global__ void __launch_bounds__(NTHR, 1)
    conv3_tcs_kernel(const __grid_constant__ CUtensorMap tmx, const __grid_constant__ CUtensorMap tmw, Args a) {
  using C = Cfg<CIN, COUT, BPU>;
  constexpr int NSH = C::NSH, NSW = C::NSW, N = C::N, NG = C::NG, GC = C::GC;
  extern __shared__ __align__(1024) unsigned char smem[];
  const uint32_t s0 = smem_u32(smem);
  const uint32_t ws0 = s0 + C::W_OFF;
  const uint32_t hfull0 = s0 + C::BAR_OFF, hempty0 = hfull0 + 8 * NSH;
  const uint32_t wfull0 = hempty0 + 8 * NSH, wempty0 = wfull0 + 8 * NSW;
  const uint32_t afull0 = wempty0 + 8 * NSW, aempty0 = afull0 + 16;
  uint32_t* taddr_s = (uint32_t*)(smem + C::BAR_OFF + 8 * C::NBAR);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  if (tid == 0) {
    for (int s = 0; s < NSH; ++s) { bar_init(hfull0 + 8 * s, 1); bar_init(hempty0 + 8 * s, 1); }
    for (int s = 0; s < NSW; ++s) { bar_init(wfull0 + 8 * s, 1); bar_init(wempty0 + 8 * s, 1); }
    for (int k = 0; k < 2; ++k) { bar_init(afull0 + 8 * k, 1); bar_init(aempty0 + 8 * k, 4); }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(taddr_s)),
                 "r"(C::TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t taddr = *taddr_s;

  const int nbu = (a.W + BW * BPU - 1) / (BW * BPU), nbh = (a.H + BH - 1) / BH;   // units along w, bricks along h
  const long long nunits = (long long)a.B * a.D * nbh * nbu * C::NSPLIT;
  const int nmine = blockIdx.x < nunits ? (int)((nunits - 1 - blockIdx.x) / gridDim.x + 1) : 0;
  bool ok = true;

  if (warp == 0) {
    // ---- TMA producer: per channel group of a unit, its halo, then its 27 weight slices --------
    if (lane == 0) {
      int hj = 0, wi = 0;   // halo loads and weight slices issued
      for (int j = 0; j < nmine && ok; ++j) {
        unsigned u = blockIdx.x + (unsigned)j * gridDim.x;
        const int split = (int)(u % (unsigned)C::NSPLIT); u /= (unsigned)C::NSPLIT;
        const int bu = (int)(u % (unsigned)nbu); u /= (unsigned)nbu;
        const int bh = (int)(u % (unsigned)nbh); u /= (unsigned)nbh;
        const int d = (int)(u % (unsigned)a.D), b = (int)(u / (unsigned)a.D);
        for (int g = 0; g < NG && ok; ++g) {
          const int hi = j * NG + g, hs = hi % NSH;
          if (hi >= NSH) ok = bar_wait(hempty0 + 8 * hs, (uint32_t)((hi / NSH - 1) & 1));
          if (!ok) break;
          bar_expect_tx(hfull0 + 8 * hs, (uint32_t)(GC * C::XV * 16));
          for (int kc = 0; kc < GC; ++kc)
            tma_load_5d(s0 + hs * C::HALO + kc * C::CHB, &tmx, (g * GC + kc) * 8, bu * BW * BPU - 1, bh * BH - 1,
                        d - 1, b, hfull0 + 8 * hs);
          ++hj;
          for (int t = 0; t < 27 && ok; ++t) {
            const int gi = hi * 27 + t, s = gi % NSW;
            if (gi >= NSW) ok = bar_wait(wempty0 + 8 * s, (uint32_t)((gi / NSW - 1) & 1));
            if (!ok) break;
            bar_expect_tx(wfull0 + 8 * s, (uint32_t)C::WSLICE);
            for (int kc = 0; kc < GC; ++kc)
              tma_load_3d(ws0 + s * C::WSLICE + kc * N * 16, &tmw, (g * GC + kc) * 8, split * N, t, wfull0 + 8 * s);
            ++wi;
          }
        }
      }
      // let the last loads issued land before the CTA can end
      for (int j = hj - NSH > 0 ? hj - NSH : 0; j < hj; ++j)
        (void)bar_wait(hfull0 + 8 * (j % NSH), (uint32_t)((j / NSH) & 1));
      for (int gi = wi - NSW > 0 ? wi - NSW : 0; gi < wi; ++gi)
        (void)bar_wait(wfull0 + 8 * (gi % NSW), (uint32_t)((gi / NSW) & 1));
    }
  } else if (warp == 1) {
    // ---- MMA issuer ----------------------------------------------------------------
    if (lane == 0) {
      constexpr uint32_t IDESC = idesc_bf16(128, N);
      for (int j = 0; j < nmine && ok; ++j) {
        const int k = j & 1;
        if (j >= 2) ok = bar_wait(aempty0 + 8 * k, (uint32_t)((j / 2 - 1) & 1));
        if (!ok) break;
        const uint32_t tacc = taddr + (uint32_t)(k * C::ACC);
        for (int g = 0; g < NG && ok; ++g) {
          const int hi = j * NG + g, hs = hi % NSH;
          ok = bar_wait(hfull0 + 8 * hs, (uint32_t)((hi / NSH) & 1));
          if (!ok) break;
          // A: brick rows (h) XW voxels apart, chunks CHB apart; brick b starts 8 voxels on
          const uint64_t ad0 = sdesc(s0 + hs * C::HALO, C::CHB, C::XW * 16);
          for (int t = 0; t < 27 && ok; ++t) {
            const int gi = hi * 27 + t, s = gi % NSW;
            ok = bar_wait(wfull0 + 8 * s, (uint32_t)((gi / NSW) & 1));
            if (!ok) break;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const int kd = t / 9, kh = (t / 3) % 3, kw = t % 3;
            const uint64_t bd0 = sdesc(ws0 + s * C::WSLICE, N * 16, 128);
#pragma unroll
            for (int q = 0; q < GC / 2; ++q) {
              const uint64_t bd = bd0 + (uint64_t)(2 * q * N);
#pragma unroll
              for (int bb = 0; bb < BPU; ++bb) {
                const uint64_t ad =
                    ad0 + (uint64_t)((2 * q) * (C::CHB / 16) + (kd * XH + kh) * C::XW + kw + bb * BW);
                mma_bf16_ss(tacc + (uint32_t)(bb * N), ad, bd, IDESC, (g | t | q) ? 1u : 0u);
              }
            }
            mma_commit(wempty0 + 8 * s);   // the weight slice is free once these MMAs are done
          }
          if (!ok) break;
          mma_commit(hempty0 + 8 * hs);   // so is the halo stage
        }
        if (!ok) break;
        mma_commit(afull0 + 8 * k);   // and the accumulators are ready
      }
    }
  } else {
    // ---- epilogue: warps 2..5, TMEM lane quarter = warp % 4 ---------------------------
    const int quarter = warp & 3;
    const int m = quarter * 32 + lane;   // brick voxel of this thread
    for (int j = 0; j < nmine && ok; ++j) {
      const int k = j & 1;
      ok = bar_wait(afull0 + 8 * k, (uint32_t)((j / 2) & 1));
      if (!__all_sync(0xffffffffu, ok)) { ok = false; break; }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      unsigned u = blockIdx.x + (unsigned)j * gridDim.x;
      const int split = (int)(u % (unsigned)C::NSPLIT); u /= (unsigned)C::NSPLIT;
      const int bu = (int)(u % (unsigned)nbu); u /= (unsigned)nbu;
      const int bh = (int)(u % (unsigned)nbh); u /= (unsigned)nbh;
      const int d = (int)(u % (unsigned)a.D), b = (int)(u / (unsigned)a.D);
      const int co0 = split * N;
#pragma unroll 1
      for (int bb = 0; bb < BPU; ++bb) {
        const int gh = bh * BH + (m >> 3), gw = (bu * BPU + bb) * BW + (m & 7);
        const bool inside = gh < a.H && gw < a.W;
        const size_t gv = inside ? (((size_t)b * a.D + d) * a.H + gh) * a.W + gw : 0;
#pragma unroll 1
        for (int c0 = 0; c0 < N; c0 += 16) {
          uint32_t r[16];
          tmem_ld16(taddr + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(k * C::ACC + bb * N + c0), r);
          tmem_wait_ld();
          if (!inside) continue;
          float v[16];
#pragma unroll
          for (int jj = 0; jj < 16; ++jj) v[jj] = __uint_as_float(r[jj]);
          const size_t o = gv * COUT + co0 + c0;
          if (a.mode == 0) {
            if (a.bias) {
#pragma unroll
              for (int jj = 0; jj < 16; ++jj) v[jj] += a.bias[co0 + c0 + jj];
            }
            if (a.skip) {
              const uint4* sp = (const uint4*)(a.skip + o);
              uint4 q0 = sp[0], q1 = sp[1];
              const bf16* e0 = (const bf16*)&q0;
              const bf16* e1 = (const bf16*)&q1;
#pragma unroll
              for (int jj = 0; jj < 8; ++jj) { v[jj] += __bfloat162float(e0[jj]); v[8 + jj] += __bfloat162float(e1[jj]); }
            }
            if (a.act) {
#pragma unroll
              for (int jj = 0; jj < 16; ++jj) v[jj] = leaky(v[jj], a.slope);
            }
            uint4 o0, o1;
            bf16* f0 = (bf16*)&o0;
            bf16* f1 = (bf16*)&o1;
#pragma unroll
            for (int jj = 0; jj < 8; ++jj) { f0[jj] = __float2bfloat16_rn(v[jj]); f1[jj] = __float2bfloat16_rn(v[8 + jj]); }
            uint4* op = (uint4*)(a.y + o);
            op[0] = o0;
            op[1] = o1;
          } else if (a.mode == 3) {
            act_grad16(v, a.yact, a.y, a.dskip, o, a.slope);
          } else {
            float4* op = (float4*)(a.yf + o);
#pragma unroll
            for (int qq = 0; qq < 4; ++qq) {
              float4 tt = make_float4(v[4 * qq], v[4 * qq + 1], v[4 * qq + 2], v[4 * qq + 3]);
              if (a.mode == 1) {
                const float4 p = op[qq];
                tt.x += p.x; tt.y += p.y; tt.z += p.z; tt.w += p.w;
              }
              op[qq] = tt;
            }
          }
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0) bar_arrive(aempty0 + 8 * k);   // the accumulators may be overwritten
    }
  }
  if (!ok) atomicExch(&g_timeout, 1);
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 1) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(C::TMEM_COLS));
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

template <int CIN, int COUT, int BPU>
int launch_bpu(const Args& a, cudaStream_t st) {
  using C = Cfg<CIN, COUT, BPU>;
  // at least half an SM's shared memory: one CTA per SM (its TMEM columns and weight stream)
  constexpr int SMEM = C::SMEM > 116 * 1024 ? C::SMEM : 116 * 1024;
  static bool attr = false;
  if (!attr) {
    if (cudaFuncSetAttribute(conv3_tcs_kernel<CIN, COUT, BPU>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM) !=
        cudaSuccess)
      return TBSG_ERR_CUDA;
    attr = true;
  }
  auto enc = encoder();
  if (!enc) return TBSG_ERR_CUDA;
  CUtensorMap tmx, tmw;
  {  // activations [B][D][H][W][CIN], boxes [3][18][8 BPU + 2][8 ch]
    cuuint64_t dims[5] = {(cuuint64_t)CIN, (cuuint64_t)a.W, (cuuint64_t)a.H, (cuuint64_t)a.D, (cuuint64_t)a.B};
    cuuint64_t strides[4] = {(cuuint64_t)CIN * 2, (cuuint64_t)a.W * CIN * 2, (cuuint64_t)a.H * a.W * CIN * 2,
                             (cuuint64_t)a.D * a.H * a.W * CIN * 2};
    cuuint32_t box[5] = {8, (cuuint32_t)C::XW, (cuuint32_t)XH, (cuuint32_t)XD, 1};
    cuuint32_t es[5] = {1, 1, 1, 1, 1};
    if (enc(&tmx, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, (void*)a.x, dims, strides, box, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return TBSG_ERR_ARG;
  }
  {  // weights [27][COUT][CIN] as (ci, co, tap), boxes [N][8 ch]
    cuuint64_t dims[3] = {(cuuint64_t)CIN, (cuuint64_t)COUT, 27};
    cuuint64_t strides[2] = {(cuuint64_t)CIN * 2, (cuuint64_t)COUT * CIN * 2};
    cuuint32_t box[3] = {8, (cuuint32_t)C::N, 1};
    cuuint32_t es[3] = {1, 1, 1};
    if (enc(&tmw, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, (void*)a.w, dims, strides, box, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return TBSG_ERR_ARG;
  }
  const long long nunits = (long long)a.B * a.D * ((a.H + BH - 1) / BH) * ((a.W + BW * BPU - 1) / (BW * BPU)) *
                           C::NSPLIT;
  if (nunits >= (1ll << 31)) return TBSG_ERR_SHAPE;   // unit indices are 32-bit in the kernel
  const int g = (int)(nunits < sm_count() ? nunits : sm_count());
  conv3_tcs_kernel<CIN, COUT, BPU><<<g, NTHR, SMEM, st>>>(tmx, tmw, a);
  return cudaGetLastError() == cudaSuccess ? TBSG_OK : TBSG_ERR_CUDA;
}

// two bricks per unit where that still gives every SM a unit, else one
template <int CIN, int COUT>
int launch(const Args& a, cudaStream_t st) {
  constexpr int NSPLIT = Cfg<CIN, COUT, 1>::NSPLIT;
  const long long pairs = (long long)a.B * a.D * ((a.H + BH - 1) / BH) * ((a.W + 2 * BW - 1) / (2 * BW)) * NSPLIT;
  if (pairs >= sm_count()) return launch_bpu<CIN, COUT, 2>(a, st);
  return launch_bpu<CIN, COUT, 1>(a, st);
}

}  // namespace tcs

// streamed-weight tcgen05 path for the 64/128-channel pairs; TBSG_ERR_SHAPE for the others
int conv3_fwd_tcs(const void* x, int cin, const void* w, const float* bias, const void* skip, void* y, float* yf,
                  int yf_accumulate, int cout, int batch, int D, int H, int W, int act, float slope, const void* yact,
                  float* dskip, cudaStream_t st) {
  tcs::Args a;
  a.x = (const bf16*)x; a.w = (const bf16*)w; a.bias = bias; a.skip = (const bf16*)skip;
  a.y = (bf16*)y; a.yf = yf;
  a.B = batch; a.D = D; a.H = H; a.W = W;
  a.act = act; a.slope = slope;
  a.mode = yact ? 3 : (yf ? (yf_accumulate ? 1 : 2) : 0);
  a.yact = (const bf16*)yact; a.dskip = dskip;
  if ((uintptr_t)x % 16 || (uintptr_t)w % 16) return TBSG_ERR_SHAPE;   // TMA needs 16-byte aligned bases
  if (cin == 32 && cout == 64) return tcs::launch<32, 64>(a, st);
  if (cin == 64 && cout == 32) return tcs::launch<64, 32>(a, st);
  if (cin == 64 && cout == 64) return tcs::launch<64, 64>(a, st);
  if (cin == 64 && cout == 128) return tcs::launch<64, 128>(a, st);
  if (cin == 128 && cout == 64) return tcs::launch<128, 64>(a, st);
  if (cin == 128 && cout == 128) return tcs::launch<128, 128>(a, st);
  return TBSG_ERR_SHAPE;
}

// whether a streamed-weight launch gave up waiting (and clear the flag)
int conv_tcs_timed_out(int* v) {
  if (cudaMemcpyFromSymbol(v, tcs::g_timeout, sizeof(int)) != cudaSuccess) return TBSG_ERR_CUDA;
  if (*v) {
    int z = 0;
    if (cudaMemcpyToSymbol(tcs::g_timeout, &z, sizeof(int)) != cudaSuccess) return TBSG_ERR_CUDA;
  }
  return TBSG_OK;
}

}  // namespace sg
