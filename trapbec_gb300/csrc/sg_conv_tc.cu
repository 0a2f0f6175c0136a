// sg_conv_tc.cu -- 3x3x3 convolutions of the warm-start surrogate on the
// 5th-generation tensor cores (tcgen05.mma, accumulators in TMEM) for the
// layers with 16 or 32 input and output channels, which carry most of the
// network's FLOPs (the 128^3 and 64^3 levels).
//
// Implicit GEMM per 1 x 16 x 8 output brick: M = 128 voxels, N = Cout,
// K = 27 taps x Cin.  The halo (3 x 18 x 10 voxels) is staged K-chunked in
// shared memory, [Cin/8][3][18][10][8 BF16]: the 8 voxels of one brick row
// are 8 consecutive 16-byte rows, i.e. one core matrix of the no-swizzle
// K-major operand layout, the next brick row is 160 bytes on (the stride
// between 8-row groups) and the next 8 channels one chunk on (the stride
// between K core matrices).  So the A operand of every tap is the same
// descriptor with a different start address.  The weights of the whole
// layer stay resident in the same layout, [27][Cin/8][Cout][8 BF16].  One
// thread issues the 27 x Cin/16 MMAs (M=128, N=Cout, K=16, FP32 accumulate),
// commits them to an mbarrier, and four warps read the 128 x Cout
// accumulator from TMEM (warp w owns lanes 32w..32w+31 = brick rows) for the
// fused bias + skip + leaky-ReLU epilogue.  CTAs are persistent and run a
// two-stage pipeline over their bricks with two halo buffers and two TMEM
// accumulators: while the tensor cores work on brick i, the halo of brick
// i+1 is in flight and the epilogue drains brick i-1.  Waits are bounded in
// time; TMEM is always released.
#include "../../include/trapbec_surrogate.h"
#include "sg_common.cuh"

namespace sg {
namespace tc {

constexpr int BH = 16, BW = 8;                  // output brick rows (h) x columns (w); M = 128
constexpr int XD = 3, XH = BH + 2, XW = BW + 2;
constexpr int XV = XD * XH * XW;                // 540 halo voxels
constexpr int NTHR = 128;
constexpr uint32_t ACC_COLS = 32;               // one accumulator: 128 lanes x Cout <= 32 columns
constexpr uint32_t TMEM_COLS = 2 * ACC_COLS;    // double-buffered
constexpr uint64_t WAIT_NS = 2000000000ull;     // 2 s

__device__ int g_timeout = 0;                   // set when an MMA-completion wait gave up

template <int CIN, int COUT> struct Cfg {
  static constexpr int KC = CIN / 8;
  static constexpr int X_BYTES = KC * XV * 16;                 // one halo buffer
  static constexpr int X_STRIDE = (X_BYTES + 1023) / 1024 * 1024;
  static constexpr int W_OFF = 2 * X_STRIDE;
  static constexpr int W_BYTES = 27 * KC * COUT * 16;
  static constexpr int BAR_OFF = W_OFF + W_BYTES;
  static constexpr int SMEM = BAR_OFF + 64;
};

__device__ __forceinline__ uint64_t now_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// shared-memory operand descriptor: K-major, no swizzle
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;   // between K core matrices
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;   // between 8-row groups (M or N)
  d |= (uint64_t)1 << 46;                        // descriptor version
  return d;
}
// instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both K-major
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ bool bar_try(uint32_t bar, uint32_t par) {
  uint32_t ok;
  asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
               : "=r"(ok)
               : "r"(bar), "r"(par)
               : "memory");
  return ok != 0;
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float v[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
}

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
  int mode;            // 0: BF16 epilogue, 1: FP32 +=, 2: FP32 =
};

template <int CIN, int COUT>
__global__ void __launch_bounds__(NTHR) conv3_tc_kernel(Args a) {
  using C = Cfg<CIN, COUT>;
  static_assert(COUT % 16 == 0 && COUT <= (int)ACC_COLS, "accumulator columns");
  extern __shared__ __align__(1024) unsigned char smem[];
  unsigned char* ws = smem + C::W_OFF;
  const uint32_t bar0 = smem_u32(smem + C::BAR_OFF);          // bars[k] at bar0 + 8k
  uint32_t* taddr_s = (uint32_t*)(smem + C::BAR_OFF + 16);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  // resident weights: [27][COUT][CIN] -> [27][KC][COUT][8]
  for (int i = tid; i < 27 * COUT * C::KC; i += NTHR) {
    const int kc = i % C::KC;
    const int r = i / C::KC;   // tap * COUT + co
    const int co = r % COUT, tap = r / COUT;
    cp_async16(ws + ((size_t)(tap * C::KC + kc) * COUT + co) * 16, a.w + (size_t)r * CIN + kc * 8, 16);
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar0));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar0 + 8));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(taddr_s)),
                 "r"(TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }

  const int nbw = (a.W + BW - 1) / BW, nbh = (a.H + BH - 1) / BH;
  const long long nbricks = (long long)a.B * a.D * nbh * nbw;
  const uint32_t ws_a = smem_u32(ws);
  constexpr uint32_t IDESC = idesc_bf16(128, COUT);
  struct Pos { int b, d, h0, w0; };
  auto pos_of = [&](long long brick) {
    Pos q;
    long long r = brick;
    const int bw = (int)(r % nbw); r /= nbw;
    const int bh = (int)(r % nbh); r /= nbh;
    q.d = (int)(r % a.D);
    q.b = (int)(r / a.D);
    q.h0 = bh * BH;
    q.w0 = bw * BW;
    return q;
  };
  // halo of a brick into buffer k, K-chunked, zero outside the grid
  auto load_halo = [&](const Pos& q, int k) {
    unsigned char* xs = smem + k * C::X_STRIDE;
    for (int i = tid; i < C::KC * XV; i += NTHR) {
      const int hv = i % XV, kc = i / XV;
      const int hw = hv % XW, hh = (hv / XW) % XH, hd = hv / (XW * XH);
      const int gd = q.d + hd - 1, gh = q.h0 + hh - 1, gw = q.w0 + hw - 1;
      const bool in = gd >= 0 && gd < a.D && gh >= 0 && gh < a.H && gw >= 0 && gw < a.W;
      const bf16* src = in ? a.x + ((((size_t)q.b * a.D + gd) * a.H + gh) * a.W + gw) * CIN + kc * 8 : a.x;
      cp_async16(xs + (size_t)(kc * XV + hv) * 16, src, in ? 16 : 0);
    }
    cp_async_commit();
  };
  // bounded wait for completion number n of bars[k] (parity n & 1)
  auto wait_bar = [&](int k, uint32_t n) -> bool {
    const uint32_t bar = bar0 + 8u * (uint32_t)k, par = n & 1u;
    bool ok = bar_try(bar, par);
    if (!ok) {
      const uint64_t t0 = now_ns();
      while (!(ok = bar_try(bar, par)))
        if (now_ns() - t0 > WAIT_NS) break;
    }
    return ok;
  };
  auto epilogue = [&](const Pos& q, int k) {
    const uint32_t tacc = *taddr_s + (uint32_t)k * ACC_COLS;
    const int m = warp * 32 + lane;
    const int gh = q.h0 + (m >> 3), gw = q.w0 + (m & 7);
    const bool store = gh < a.H && gw < a.W;
    const size_t gv = (((size_t)q.b * a.D + q.d) * a.H + gh) * a.W + gw;
#pragma unroll
    for (int c0 = 0; c0 < COUT; c0 += 16) {
      float v[16];
      tmem_ld16(tacc + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
      if (!store) continue;
      if (a.mode == 0) {
        if (a.bias) {
#pragma unroll
          for (int j = 0; j < 16; ++j) v[j] += a.bias[c0 + j];
        }
        if (a.skip) {
          const uint4* sp = (const uint4*)(a.skip + gv * COUT + c0);
          uint4 s0 = sp[0], s1 = sp[1];
          const bf16* e0 = (const bf16*)&s0;
          const bf16* e1 = (const bf16*)&s1;
#pragma unroll
          for (int j = 0; j < 8; ++j) { v[j] += __bfloat162float(e0[j]); v[8 + j] += __bfloat162float(e1[j]); }
        }
        if (a.act) {
#pragma unroll
          for (int j = 0; j < 16; ++j) v[j] = leaky(v[j], a.slope);
        }
        uint4 o0, o1;
        bf16* f0 = (bf16*)&o0;
        bf16* f1 = (bf16*)&o1;
#pragma unroll
        for (int j = 0; j < 8; ++j) { f0[j] = __float2bfloat16_rn(v[j]); f1[j] = __float2bfloat16_rn(v[8 + j]); }
        uint4* op = (uint4*)(a.y + gv * COUT + c0);
        op[0] = o0;
        op[1] = o1;
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
  };

  // prologue: the weights and the first halo
  long long brick = blockIdx.x;
  Pos cur = pos_of(brick), prev{};
  load_halo(cur, 0);
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  bool failed = false;
  int i = 0;
  for (; brick < nbricks; brick += gridDim.x, ++i) {
    const int k = i & 1;
    // halo i (and, the first time, the weights) has landed
    cp_async_wait<0>();
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");   // cp.async data -> tensor-core reads
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t taddr = *taddr_s;
    if (tid == 0) {   // brick i: 27 x CIN/16 MMAs into accumulator k
      const uint32_t xs_a = smem_u32(smem + k * C::X_STRIDE);
      const uint32_t tacc = taddr + (uint32_t)k * ACC_COLS;
#pragma unroll 1
      for (int tap = 0; tap < 27; ++tap) {
        const int kd = tap / 9, kh = (tap / 3) % 3, kw = tap % 3;
#pragma unroll
        for (int s = 0; s < CIN / 16; ++s) {
          const uint32_t a_addr = xs_a + (uint32_t)((2 * s) * XV + (kd * XH + kh) * XW + kw) * 16u;
          const uint32_t b_addr = ws_a + (uint32_t)((tap * C::KC + 2 * s) * COUT) * 16u;
          const uint64_t ad = sdesc(a_addr, XV * 16, XW * 16);
          const uint64_t bd = sdesc(b_addr, COUT * 16, 128);
          const uint32_t acc = (tap | s) ? 1u : 0u;
          asm volatile(
              "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
              " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tacc),
              "l"(ad), "l"(bd), "r"(IDESC), "r"(acc));
        }
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar0 + 8u * k)
                   : "memory");
    }
    // brick i-1's MMAs read the other halo buffer: wait for them, then refill it
    if (i > 0) {
      if (__syncthreads_or(!wait_bar(k ^ 1, (uint32_t)(i - 1) >> 1))) { failed = true; break; }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    }
    const long long next = brick + gridDim.x;
    Pos nxt{};
    if (next < nbricks) {
      nxt = pos_of(next);
      load_halo(nxt, k ^ 1);
    }
    if (i > 0) epilogue(prev, k ^ 1);   // overlaps brick i's MMAs and brick i+1's loads
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    prev = cur;
    cur = nxt;
  }
  // drain: the last brick's accumulator
  if (!failed && i > 0) {
    const int k = (i - 1) & 1;
    if (__syncthreads_or(!wait_bar(k, (uint32_t)(i - 1) >> 1))) {
      failed = true;
    } else {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      epilogue(prev, k);
    }
  }
  if (failed && tid == 0) atomicExch(&g_timeout, 1);
  cp_async_wait<0>();   // no copy may outlive the CTA
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(*taddr_s), "r"(TMEM_COLS));
}

template <int CIN, int COUT>
int launch(const Args& a, cudaStream_t st) {
  using C = Cfg<CIN, COUT>;
  static int grid = 0;
  if (!grid) {
    if (cudaFuncSetAttribute(conv3_tc_kernel<CIN, COUT>, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM) !=
        cudaSuccess)
      return TBSG_ERR_CUDA;
    int dev = 0, nsm = 0, nb = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, conv3_tc_kernel<CIN, COUT>, NTHR, C::SMEM) != cudaSuccess ||
        nb < 1)
      return TBSG_ERR_CUDA;
    if (nb * (int)TMEM_COLS > 512) nb = 512 / (int)TMEM_COLS;   // TMEM of one SM
    grid = nb * nsm;
  }
  const long long nbricks = (long long)a.B * a.D * ((a.H + BH - 1) / BH) * ((a.W + BW - 1) / BW);
  const int g = (int)(nbricks < grid ? nbricks : grid);
  conv3_tc_kernel<CIN, COUT><<<g, NTHR, C::SMEM, st>>>(a);
  return cudaGetLastError() == cudaSuccess ? TBSG_OK : TBSG_ERR_CUDA;
}

}  // namespace tc

// tcgen05 path for 16/32 -> 16/32 channels; TBSG_ERR_SHAPE for the others
int conv3_fwd_tc(const void* x, int cin, const void* w, const float* bias, const void* skip, void* y, float* yf,
                 int yf_accumulate, int cout, int batch, int D, int H, int W, int act, float slope, cudaStream_t st) {
  tc::Args a;
  a.x = (const bf16*)x; a.w = (const bf16*)w; a.bias = bias; a.skip = (const bf16*)skip;
  a.y = (bf16*)y; a.yf = yf;
  a.B = batch; a.D = D; a.H = H; a.W = W;
  a.act = act; a.slope = slope;
  a.mode = yf ? (yf_accumulate ? 1 : 2) : 0;
  if (cin == 16 && cout == 16) return tc::launch<16, 16>(a, st);
  if (cin == 16 && cout == 32) return tc::launch<16, 32>(a, st);
  if (cin == 32 && cout == 16) return tc::launch<32, 16>(a, st);
  if (cin == 32 && cout == 32) return tc::launch<32, 32>(a, st);
  return TBSG_ERR_SHAPE;
}

}  // namespace sg

extern "C" int tbsg_tc_status(int* timed_out) {
  if (!timed_out) return TBSG_ERR_ARG;
  int v = 0;
  if (cudaMemcpyFromSymbol(&v, sg::tc::g_timeout, sizeof(int)) != cudaSuccess) return TBSG_ERR_CUDA;
  *timed_out = v;
  if (v) {
    int z = 0;
    if (cudaMemcpyToSymbol(sg::tc::g_timeout, &z, sizeof(int)) != cudaSuccess) return TBSG_ERR_CUDA;
  }
  return TBSG_OK;
}
