// sg_conv_tc.cu -- 3x3x3 convolutions of the warm-start surrogate on the
// 5th-generation tensor cores (tcgen05.mma, accumulators in TMEM) for the
// layers with 16 or 32 input and output channels, which carry most of the
// network's FLOPs (the 128^3 and 64^3 levels).
//
// Implicit GEMM per 1 x 16 x 8 output brick: M = 128 voxels, N = Cout,
// K = 27 taps x Cin.  The halo (3 x 18 x 10 voxels) lands K-chunked in shared
// memory, one TMA box [3][18][10][8 channels] per 8-channel chunk (out-of-
// range voxels zero-filled by the TMA unit): the 8 voxels of one brick row
// are 8 consecutive 16-byte rows, i.e. one core matrix of the no-swizzle
// K-major operand layout, the next brick row is 160 bytes on (the stride
// between 8-row groups) and the next 8 channels one chunk on (the stride
// between K core matrices), so the A operand of every tap is the same
// descriptor with a different start address.  The layer's weights stay
// resident in the same layout, [27][Cin/8][Cout][8].
//
// Warp-specialised persistent CTAs: warp 0 issues the TMA loads of each
// brick's halo into a ring of stages, warp 1 issues the 27 x Cin/16 MMAs
// (M=128, N=Cout, K=16, FP32 accumulate) into one of two TMEM accumulators
// and commits them to mbarriers, warps 2-5 read a finished accumulator from
// TMEM (a warp reads the 32 lanes of its quarter = 32 brick voxels), release
// it, and run the fused bias + skip + leaky-ReLU epilogue.  All hand-offs are
// mbarrier phases; every wait is bounded in time; TMEM is always released.
#include "../../include/trapbec_surrogate.h"
#include "sg_tc_common.cuh"

namespace sg {
namespace tc {

using namespace tcc;

constexpr int BH = 16, BW = 8;                  // output brick rows (h) x columns (w); M = 128
constexpr int XD = 3, XH = BH + 2, XW = BW + 2;
constexpr int XV = XD * XH * XW;                // 540 halo voxels
constexpr int CHUNK = 8704;                     // one 8-channel chunk (540 x 16 B), padded to 128 B
constexpr int NTHR = 192;                       // 6 warps: TMA, MMA, 4 x epilogue
constexpr uint32_t ACC_COLS = 32;               // one accumulator: 128 lanes x Cout <= 32 columns
constexpr uint32_t TMEM_COLS = 2 * ACC_COLS;    // two accumulators
__device__ int g_timeout = 0;                   // set when a wait gave up

constexpr int SM_SMEM = 232448;                 // shared memory of one SM (bytes)

template <int CIN, int COUT> struct Cfg {
  static constexpr int KC = CIN / 8;
  static constexpr int STAGE = KC * CHUNK;                       // one halo
  static constexpr int W_BYTES = 27 * KC * COUT * 16;
  // CTAs per SM that a halo ring of `ns` stages leaves room for (1 KB per CTA reserved)
  static constexpr int fit(int ns) { return SM_SMEM / (ns * STAGE + W_BYTES + 128 + 1024); }
  // halo ring depth: 3, or 2 where 3 leaves room for one CTA only and 2 for more (more MMA issuers
  // per SM; measured: 32 -> 16 channels 201 -> 166 us per launch; with 2 or more CTAs already the
  // deeper ring was as fast or faster)
  static constexpr int NS = (fit(3) < 2 && fit(2) > fit(3)) ? 2 : 3;
  static constexpr int W_OFF = NS * STAGE;
  static constexpr int BAR_OFF = (W_OFF + W_BYTES + 127) / 128 * 128;
  static constexpr int SMEM = BAR_OFF + 128;
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
  const bf16* yact;    // mode 3: the output of the activation whose input gradient this is
  float* dskip;        // mode 3: optional FP32 accumulation
};

template <int CIN, int COUT>
__global__ void __launch_bounds__(NTHR, 1) conv3_tc_kernel(const __grid_constant__ CUtensorMap tmx, Args a) {
  using C = Cfg<CIN, COUT>;
  constexpr int NS = C::NS;
  static_assert(COUT % 16 == 0 && COUT <= (int)ACC_COLS, "accumulator columns");
  extern __shared__ __align__(1024) unsigned char smem[];
  const uint32_t s0 = smem_u32(smem);
  const uint32_t ws_a = s0 + C::W_OFF;
  // barriers: full[NS], empty[NS], acc_full[2], acc_empty[2]; then the TMEM address
  const uint32_t full0 = s0 + C::BAR_OFF, empty0 = full0 + 8 * NS;
  const uint32_t afull0 = empty0 + 8 * NS, aempty0 = afull0 + 16;
  uint32_t* taddr_s = (uint32_t*)(smem + C::BAR_OFF + 8 * (2 * NS + 4));
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  // resident weights: [27][COUT][CIN] -> [27][KC][COUT][8]
  for (int i = tid; i < 27 * COUT * C::KC; i += NTHR) {
    const int kc = i % C::KC;
    const int r = i / C::KC;   // tap * COUT + co
    const int co = r % COUT, tap = r / COUT;
    cp_async16(smem + C::W_OFF + ((size_t)(tap * C::KC + kc) * COUT + co) * 16, a.w + (size_t)r * CIN + kc * 8, 16);
  }
  cp_async_commit();
  if (tid == 0) {
    for (int s = 0; s < NS; ++s) { bar_init(full0 + 8 * s, 1); bar_init(empty0 + 8 * s, 1); }
    for (int k = 0; k < 2; ++k) { bar_init(afull0 + 8 * k, 1); bar_init(aempty0 + 8 * k, 4); }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(taddr_s)),
                 "r"(TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  cp_async_wait<0>();
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");   // weights -> tensor-core reads
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t taddr = *taddr_s;

  const int nbw = (a.W + BW - 1) / BW, nbh = (a.H + BH - 1) / BH;
  const long long nbricks = (long long)a.B * a.D * nbh * nbw;
  const int nmine = blockIdx.x < nbricks ? (int)((nbricks - 1 - blockIdx.x) / gridDim.x + 1) : 0;
  bool ok = true;

  if (warp == 0) {
    // ---- TMA producer --------------------------------------------------------
    if (lane == 0) {
      for (int j = 0; j < nmine && ok; ++j) {
        const int s = j % NS;
        if (j >= NS) ok = bar_wait(empty0 + 8 * s, (uint32_t)((j / NS - 1) & 1));
        if (!ok) break;
        unsigned r = blockIdx.x + (unsigned)j * gridDim.x;
        const int bw = (int)(r % (unsigned)nbw); r /= (unsigned)nbw;
        const int bh = (int)(r % (unsigned)nbh); r /= (unsigned)nbh;
        const int d = (int)(r % (unsigned)a.D), b = (int)(r / (unsigned)a.D);
        bar_expect_tx(full0 + 8 * s, (uint32_t)(C::KC * XV * 16));
        for (int kc = 0; kc < C::KC; ++kc)
          tma_load_5d(s0 + s * C::STAGE + kc * CHUNK, &tmx, kc * 8, bw * BW - 1, bh * BH - 1, d - 1, b, full0 + 8 * s);
      }
      // let the last loads land before the CTA can end
      for (int j = nmine - NS > 0 ? nmine - NS : 0; j < nmine; ++j)
        (void)bar_wait(full0 + 8 * (j % NS), (uint32_t)((j / NS) & 1));
    }
  } else if (warp == 1) {
    // ---- MMA issuer ------------------------------------------------------------
    if (lane == 0) {
      constexpr uint32_t IDESC = idesc_bf16(128, COUT);
      for (int j = 0; j < nmine && ok; ++j) {
        const int s = j % NS, k = j & 1;
        ok = bar_wait(full0 + 8 * s, (uint32_t)((j / NS) & 1));
        if (ok && j >= 2) ok = bar_wait(aempty0 + 8 * k, (uint32_t)((j / 2 - 1) & 1));
        if (!ok) break;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t tacc = taddr + (uint32_t)k * ACC_COLS;
        // the start-address field counts 16-byte units: per-tap operands are
        // the base descriptors plus compile-time offsets
        const uint64_t ad0 = sdesc(s0 + s * C::STAGE, CHUNK, XW * 16);
        const uint64_t bd0 = sdesc(ws_a, COUT * 16, 128);
#pragma unroll
        for (int tap = 0; tap < 27; ++tap) {
          const int kd = tap / 9, kh = (tap / 3) % 3, kw = tap % 3;
#pragma unroll
          for (int q = 0; q < CIN / 16; ++q) {
            const uint64_t ad = ad0 + (uint64_t)((2 * q) * (CHUNK / 16) + (kd * XH + kh) * XW + kw);
            const uint64_t bd = bd0 + (uint64_t)((tap * C::KC + 2 * q) * COUT);
            const uint32_t acc = (tap | q) ? 1u : 0u;
            asm volatile(
                "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tacc),
                "l"(ad), "l"(bd), "r"(IDESC), "r"(acc));
          }
        }
        // the halo stage is free once these MMAs are done; so is the accumulator for reading
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(empty0 + 8 * s)
                     : "memory");
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(afull0 + 8 * k)
                     : "memory");
      }
    }
  } else {
    // ---- epilogue: warps 2..5, TMEM lane quarter = warp % 4 ----------------------
    const int quarter = warp & 3;
    const int m = quarter * 32 + lane;   // brick voxel of this thread
    float bias_r[COUT];
#pragma unroll
    for (int c = 0; c < COUT; ++c) bias_r[c] = (a.mode == 0 && a.bias) ? a.bias[c] : 0.f;
    for (int j = 0; j < nmine && ok; ++j) {
      const int k = j & 1;
      ok = bar_wait(afull0 + 8 * k, (uint32_t)((j / 2) & 1));
      if (!__all_sync(0xffffffffu, ok)) { ok = false; break; }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      uint32_t r[COUT];
#pragma unroll
      for (int c0 = 0; c0 < COUT; c0 += 16)
        tmem_ld16(taddr + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(k * ACC_COLS + c0), r + c0);
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0) bar_arrive(aempty0 + 8 * k);   // the accumulator may be overwritten
      unsigned rr = blockIdx.x + (unsigned)j * gridDim.x;
      const int bw = (int)(rr % (unsigned)nbw); rr /= (unsigned)nbw;
      const int bh = (int)(rr % (unsigned)nbh); rr /= (unsigned)nbh;
      const int d = (int)(rr % (unsigned)a.D), b = (int)(rr / (unsigned)a.D);
      const int gh = bh * BH + (m >> 3), gw = bw * BW + (m & 7);
      if (gh >= a.H || gw >= a.W) continue;
      const size_t gv = (((size_t)b * a.D + d) * a.H + gh) * a.W + gw;
#pragma unroll
      for (int c0 = 0; c0 < COUT; c0 += 16) {
        float v[16];
#pragma unroll
        for (int jj = 0; jj < 16; ++jj) v[jj] = __uint_as_float(r[c0 + jj]);
        if (a.mode == 0) {
#pragma unroll
          for (int jj = 0; jj < 16; ++jj) v[jj] += bias_r[c0 + jj];
          if (a.skip) {
            const uint4* sp = (const uint4*)(a.skip + gv * COUT + c0);
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
          uint4* op = (uint4*)(a.y + gv * COUT + c0);
          op[0] = o0;
          op[1] = o1;
        } else if (a.mode == 3) {
          act_grad16(v, a.yact, a.y, a.dskip, gv * COUT + c0, a.slope);
        } else {
          float4* op = (float4*)(a.yf + gv * COUT + c0);
#pragma unroll
          for (int qq = 0; qq < 4; ++qq) {
            float4 t = make_float4(v[4 * qq], v[4 * qq + 1], v[4 * qq + 2], v[4 * qq + 3]);
            if (a.mode == 1) {
              const float4 o = op[qq];
              t.x += o.x; t.y += o.y; t.z += o.z; t.w += o.w;
            }
            op[qq] = t;
          }
        }
      }
    }
  }
  if (!ok) atomicExch(&g_timeout, 1);
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 1) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(TMEM_COLS));
}

template <int CIN, int COUT>
int launch(const Args& a, cudaStream_t st) {
  using C = Cfg<CIN, COUT>;
  static int grid = 0;
  if (!grid) {
    if (cudaFuncSetAttribute(conv3_tc_kernel<CIN, COUT>, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM) !=
        cudaSuccess)
      return TBSG_ERR_CUDA;
    // CTAs per SM: as many as the SM's shared memory holds (the TMEM of one
    // SM, 512 columns, holds 8 of them); all of the SM's shared memory is
    // given to the carveout
    if (cudaFuncSetAttribute(conv3_tc_kernel<CIN, COUT>, cudaFuncAttributePreferredSharedMemoryCarveout, 100) !=
        cudaSuccess)
      return TBSG_ERR_CUDA;
    int dev = 0, nsm = 0, smem_sm = 0, reserved = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
    cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev);
    int nb = smem_sm / (C::SMEM + reserved);
    if (nb * (int)TMEM_COLS > 512) nb = 512 / (int)TMEM_COLS;   // TMEM of one SM
    if (nb * NTHR > 2048) nb = 2048 / NTHR;
    cudaFuncAttributes fa;
    if (cudaFuncGetAttributes(&fa, conv3_tc_kernel<CIN, COUT>) != cudaSuccess) return TBSG_ERR_CUDA;
    const int regs = (fa.numRegs + 7) / 8 * 8;   // allocated per thread in units of 8
    if (regs > 0 && nb * NTHR * regs > 65536) nb = 65536 / (NTHR * regs);
    if (nsm < 1 || nb < 1) return TBSG_ERR_CUDA;
    grid = nb * nsm;
  }
  // the activation tensor [B][D][H][W][CIN] as a 5-D TMA map (innermost first)
  auto enc = encoder();
  if (!enc) return TBSG_ERR_CUDA;
  CUtensorMap tm;
  cuuint64_t dims[5] = {(cuuint64_t)CIN, (cuuint64_t)a.W, (cuuint64_t)a.H, (cuuint64_t)a.D, (cuuint64_t)a.B};
  cuuint64_t strides[4] = {(cuuint64_t)CIN * 2, (cuuint64_t)a.W * CIN * 2, (cuuint64_t)a.H * a.W * CIN * 2,
                           (cuuint64_t)a.D * a.H * a.W * CIN * 2};
  cuuint32_t box[5] = {8, (cuuint32_t)XW, (cuuint32_t)XH, (cuuint32_t)XD, 1};
  cuuint32_t es[5] = {1, 1, 1, 1, 1};
  if (enc(&tm, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, (void*)a.x, dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
          CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) !=
      CUDA_SUCCESS)
    return TBSG_ERR_ARG;
  const long long nbricks = (long long)a.B * a.D * ((a.H + BH - 1) / BH) * ((a.W + BW - 1) / BW);
  if (nbricks >= (1ll << 31)) return TBSG_ERR_SHAPE;   // brick indices are 32-bit in the kernel
  const int g = (int)(nbricks < grid ? nbricks : grid);
  conv3_tc_kernel<CIN, COUT><<<g, NTHR, C::SMEM, st>>>(tm, a);
  return cudaGetLastError() == cudaSuccess ? TBSG_OK : TBSG_ERR_CUDA;
}

}  // namespace tc

// tcgen05 path for 16/32 -> 16/32 channels; TBSG_ERR_SHAPE for the others
int conv3_fwd_tc(const void* x, int cin, const void* w, const float* bias, const void* skip, void* y, float* yf,
                 int yf_accumulate, int cout, int batch, int D, int H, int W, int act, float slope, const void* yact,
                 float* dskip, cudaStream_t st) {
  tc::Args a;
  a.x = (const bf16*)x; a.w = (const bf16*)w; a.bias = bias; a.skip = (const bf16*)skip;
  a.y = (bf16*)y; a.yf = yf;
  a.B = batch; a.D = D; a.H = H; a.W = W;
  a.act = act; a.slope = slope;
  a.mode = yact ? 3 : (yf ? (yf_accumulate ? 1 : 2) : 0);
  a.yact = (const bf16*)yact; a.dskip = dskip;
  if ((uintptr_t)x % 16) return TBSG_ERR_SHAPE;   // TMA needs a 16-byte aligned base
  if (cin == 16 && cout == 16) return tc::launch<16, 16>(a, st);
  if (cin == 16 && cout == 32) return tc::launch<16, 32>(a, st);
  if (cin == 32 && cout == 16) return tc::launch<32, 16>(a, st);
  if (cin == 32 && cout == 32) return tc::launch<32, 32>(a, st);
  return TBSG_ERR_SHAPE;
}

}  // namespace sg

namespace sg {
int wgrad_tc_timed_out(int* v);
int conv_tcs_timed_out(int* v);
}

extern "C" int tbsg_tc_status(int* timed_out) {
  if (!timed_out) return TBSG_ERR_ARG;
  int v = 0;
  if (cudaMemcpyFromSymbol(&v, sg::tc::g_timeout, sizeof(int)) != cudaSuccess) return TBSG_ERR_CUDA;
  if (v) {
    int z = 0;
    if (cudaMemcpyToSymbol(sg::tc::g_timeout, &z, sizeof(int)) != cudaSuccess) return TBSG_ERR_CUDA;
  }
  int vw = 0, vs = 0;
  int rc = sg::wgrad_tc_timed_out(&vw);
  if (rc != TBSG_OK) return rc;
  rc = sg::conv_tcs_timed_out(&vs);
  if (rc != TBSG_OK) return rc;
  *timed_out = v | vw | vs;
  return TBSG_OK;
}
