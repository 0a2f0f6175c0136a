// sg_conv.cu -- 3x3x3 convolutions of the warm-start surrogate as implicit
// GEMMs on the BF16 tensor cores (FP32 accumulation).
//
// Forward (and input gradient, which is the forward pass of the flipped,
// transposed kernel): one CTA per 2x8x8 output brick.  The 4x10x10 input halo
// brick is staged once in shared memory (cp.async, zero fill outside the
// grid) and reused by all 27 taps; the per-tap weight slices [COUT][CIN] are
// double-buffered.  Eight warps each own 16 output voxels x all COUT
// channels: A fragments (voxel rows of the tap-shifted halo) and B fragments
// (weight rows) come from ldmatrix, products from mma.sync m16n8k16.
// Rows are padded by 8 BF16 so the eight 16-byte rows of every ldmatrix
// phase fall into distinct bank groups.
//
// Weight gradient: dW[tap][co][ci] = sum_v dZ[v][co] X[v + tap][ci] is, per
// tap, a COUT x CIN GEMM over all voxels.  CTAs take (voxel chunk, tap);
// each stages 128-voxel tiles of dZ and of the tap-shifted X and runs
// ldmatrix.trans fragments through the tensor cores.  Per-chunk partials are
// reduced in a fixed order, so gradients are bitwise reproducible.
#include <cstdio>

#include "../../include/trapbec_surrogate.h"
#include "sg_common.cuh"

namespace sg {

template <int CIN, int COUT> struct FwdCfg {
  static constexpr int XS = CIN + 8;   // padded row, BF16 elements
  static constexpr int WS = CIN + 8;
  static constexpr size_t X_BYTES = (size_t)HV * XS * 2;
  static constexpr size_t W_BYTES = (size_t)COUT * WS * 2;
  static constexpr size_t SMEM = X_BYTES + 2 * W_BYTES;
};

struct FwdArgs {
  const bf16* x;       // [B][V][CIN]
  const bf16* w;       // [27][COUT][CIN]
  const float* bias;   // [COUT] or null
  const bf16* skip;    // [B][V][COUT] or null, added before the activation
  bf16* y;             // mode 0 output; mode 3: BF16(v act'(yact))
  float* yf;           // mode 1 (+=) / mode 2 (=) output
  int D, H, W;
  int act;
  float slope;
  int mode;
  const bf16* yact;    // mode 3: the output of the activation whose input gradient this is
  float* dskip;        // mode 3: optional FP32 accumulation of v act'(yact)
};

template <int CIN, int COUT>
__device__ __forceinline__ void load_wtap(bf16* ws, const bf16* w, int tap, int tid) {
  using C = FwdCfg<CIN, COUT>;
  constexpr int CH = CIN / 8;
  const bf16* src = w + (size_t)tap * COUT * CIN;
  for (int i = tid; i < COUT * CH; i += NTHR) {
    const int r = i / CH, c = i % CH;
    cp_async16(ws + r * C::WS + c * 8, src + (size_t)r * CIN + c * 8, 16);
  }
}

template <int CIN, int COUT>
__global__ void __launch_bounds__(NTHR, 1) conv3_fwd_kernel(FwdArgs a) {
  using C = FwdCfg<CIN, COUT>;
  constexpr int NT = COUT / 8;   // n8 tiles per warp
  extern __shared__ __align__(16) unsigned char smem[];
  bf16* xs = (bf16*)smem;
  bf16* wsb[2] = {(bf16*)(smem + C::X_BYTES), (bf16*)(smem + C::X_BYTES + C::W_BYTES)};
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int nbw = (a.W + TW - 1) / TW, nbh = (a.H + TH - 1) / TH;
  int bid = blockIdx.x;
  const int bw = bid % nbw;
  bid /= nbw;
  const int bh = bid % nbh, bd = bid / nbh;
  const int d0 = bd * TD, h0 = bh * TH, w0 = bw * TW;
  const size_t V = (size_t)a.D * a.H * a.W;
  const bf16* x = a.x + (size_t)blockIdx.z * V * CIN;

  {  // input halo brick
    constexpr int CH = CIN / 8;
    for (int i = tid; i < HV * CH; i += NTHR) {
      const int vox = i / CH, c = i % CH;
      const int hw = vox % HW, t = vox / HW, hh = t % HH, hd = t / HH;
      const int gd = d0 + hd - 1, gh = h0 + hh - 1, gw = w0 + hw - 1;
      const bool in = gd >= 0 && gd < a.D && gh >= 0 && gh < a.H && gw >= 0 && gw < a.W;
      const bf16* src = in ? x + (((size_t)gd * a.H + gh) * a.W + gw) * CIN + c * 8 : x;
      cp_async16(xs + vox * C::XS + c * 8, src, in ? 16 : 0);
    }
  }
  load_wtap<CIN, COUT>(wsb[0], a.w, 0, tid);
  cp_async_commit();

  float acc[NT][4];
#pragma unroll
  for (int j = 0; j < NT; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;

  // this lane's A row: voxel r of the warp's 16 (2 rows of h x 8 of w)
  const int ar = lane & 15;
  const int aod = warp >> 2, aoh = (warp & 3) * 2 + (ar >> 3), aow = ar & 7;
  const int akh = (lane >> 4) * 8;   // k half of the A fragment
  // this lane's B row inside a 16-channel pair of n tiles
  const int bn = (lane & 7) + ((lane >> 4) << 3), bk = ((lane >> 3) & 1) * 8;

  for (int tap = 0; tap < 27; ++tap) {
    if (tap + 1 < 27) {
      load_wtap<CIN, COUT>(wsb[(tap + 1) & 1], a.w, tap + 1, tid);
      cp_async_commit();
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();
    const int kd = tap / 9, kh = (tap / 3) % 3, kw = tap % 3;
    const bf16* arow = xs + (((aod + kd) * HH + (aoh + kh)) * HW + (aow + kw)) * C::XS + akh;
    const bf16* ws = wsb[tap & 1];
#pragma unroll
    for (int kc = 0; kc < CIN / 16; ++kc) {
      uint32_t af[4];
      ldsm_x4(af, arow + kc * 16);
#pragma unroll
      for (int p = 0; p < COUT / 16; ++p) {
        uint32_t bfr[4];
        ldsm_x4(bfr, ws + (p * 16 + bn) * C::WS + kc * 16 + bk);
        mma_bf16(acc[2 * p], af, bfr[0], bfr[1]);
        mma_bf16(acc[2 * p + 1], af, bfr[2], bfr[3]);
      }
    }
    __syncthreads();
  }

  // epilogue: rows lane/4 and lane/4 + 8 of the warp's voxels
#pragma unroll
  for (int hr = 0; hr < 2; ++hr) {
    const int r = (lane >> 2) + hr * 8;
    const int od = d0 + (warp >> 2), oh = h0 + (warp & 3) * 2 + (r >> 3), ow = w0 + (r & 7);
    if (od >= a.D || oh >= a.H || ow >= a.W) continue;
    const size_t gv = (size_t)blockIdx.z * V + ((size_t)od * a.H + oh) * a.W + ow;
#pragma unroll
    for (int j = 0; j < NT; ++j) {
      const int c = j * 8 + (lane & 3) * 2;
      float v0 = acc[j][hr * 2], v1 = acc[j][hr * 2 + 1];
      if (a.mode == 0) {
        if (a.bias) { v0 += a.bias[c]; v1 += a.bias[c + 1]; }
        if (a.skip) {
          const __nv_bfloat162 s = *(const __nv_bfloat162*)(a.skip + gv * COUT + c);
          v0 += __bfloat162float(s.x);
          v1 += __bfloat162float(s.y);
        }
        if (a.act) { v0 = leaky(v0, a.slope); v1 = leaky(v1, a.slope); }
        *(__nv_bfloat162*)(a.y + gv * COUT + c) = __floats2bfloat162_rn(v0, v1);
      } else if (a.mode == 3) {
        const __nv_bfloat162 yy = *(const __nv_bfloat162*)(a.yact + gv * COUT + c);
        const float g0 = v0 * (__bfloat162float(yy.x) > 0.f ? 1.f : a.slope);
        const float g1 = v1 * (__bfloat162float(yy.y) > 0.f ? 1.f : a.slope);
        *(__nv_bfloat162*)(a.y + gv * COUT + c) = __floats2bfloat162_rn(g0, g1);
        if (a.dskip) {
          float2* sp = (float2*)(a.dskip + gv * COUT + c);
          float2 t = *sp;
          t.x += g0; t.y += g1;
          *sp = t;
        }
      } else {
        float2* o = (float2*)(a.yf + gv * COUT + c);
        if (a.mode == 1) { float2 t = *o; t.x += v0; t.y += v1; *o = t; }
        else *o = make_float2(v0, v1);
      }
    }
  }
}

// ---- weight gradient --------------------------------------------------------

template <int CIN, int COUT> struct WgCfg {
  // warps split M (COUT) and N (CIN) until a warp holds <= 64 accumulators
  // per thread, then split K (the tile's 8 k16 steps)
  static constexpr int ACC1 = COUT * CIN / 32;
  static constexpr int WM = ACC1 > 256 ? 4 : (ACC1 > 64 ? 2 : 1);
  static constexpr int WN = ACC1 > 128 ? 2 : 1;
  static constexpr int WK = 8 / (WM * WN);
  static constexpr int MW = COUT / WM, NW = CIN / WN;
  static constexpr int MT = MW / 16, NT = NW / 8;
  static constexpr int ZS = COUT + 8, XS = CIN + 8;
  static constexpr size_t Z_BYTES = (size_t)WG_ROWS * ZS * 2;
  static constexpr size_t X_BYTES = (size_t)WG_ROWS * XS * 2;
  static constexpr size_t TILE = Z_BYTES + X_BYTES;
  static constexpr size_t RED = (size_t)WK * COUT * CIN * 4;
  static constexpr size_t SMEM = TILE > RED ? TILE : RED;
  static_assert(WM * WN * WK == 8, "8 warps");
  static_assert(MW % 16 == 0 && NW % 16 == 0, "warp tile");
};

struct WgArgs {
  const bf16* x;     // [B][V][CIN]
  const bf16* dz;    // [B][V][COUT]
  float* part;       // [nchunk][27][COUT][CIN]
  float* part_b;     // [nchunk][COUT]
  int B, D, H, W;
};

template <int CIN, int COUT>
__global__ void __launch_bounds__(NTHR, 1) conv3_wgrad_kernel(WgArgs a) {
  using C = WgCfg<CIN, COUT>;
  extern __shared__ __align__(16) unsigned char smem[];
  bf16* zs = (bf16*)smem;
  bf16* xs = (bf16*)(smem + C::Z_BYTES);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int tap = blockIdx.y;
  const int kd = tap / 9 - 1, kh = (tap / 3) % 3 - 1, kw = tap % 3 - 1;
  const size_t V = (size_t)a.D * a.H * a.W;
  const size_t total = (size_t)a.B * V;
  const size_t ntiles = (total + WG_ROWS - 1) / WG_ROWS;
  const int wk = warp % C::WK, wmn = warp / C::WK, wm = wmn % C::WM, wn = wmn / C::WM;

  float acc[C::MT][C::NT][4];
#pragma unroll
  for (int i = 0; i < C::MT; ++i)
#pragma unroll
    for (int j = 0; j < C::NT; ++j) acc[i][j][0] = acc[i][j][1] = acc[i][j][2] = acc[i][j][3] = 0.f;
  float bsum = 0.f;   // bias gradient (centre tap), thread tid < COUT owns channel tid

  const int q = lane >> 3, r8 = lane & 7;
  for (size_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const size_t v0 = t * WG_ROWS;
    constexpr int ZC = COUT / 8, XC = CIN / 8;
    for (int i = tid; i < WG_ROWS * ZC; i += NTHR) {
      const int row = i / ZC, c = i % ZC;
      const size_t gv = v0 + row;
      const bool in = gv < total;
      cp_async16(zs + row * C::ZS + c * 8, in ? a.dz + gv * COUT + c * 8 : a.dz, in ? 16 : 0);
    }
    for (int i = tid; i < WG_ROWS * XC; i += NTHR) {
      const int row = i / XC, c = i % XC;
      const size_t gv = v0 + row;
      bool in = gv < total;
      const bf16* src = a.x;
      if (in) {
        const size_t b = gv / V, v = gv % V;
        const int w = (int)(v % a.W), h = (int)((v / a.W) % a.H), d = (int)(v / ((size_t)a.W * a.H));
        const int nd = d + kd, nh = h + kh, nw = w + kw;
        in = nd >= 0 && nd < a.D && nh >= 0 && nh < a.H && nw >= 0 && nw < a.W;
        if (in) src = a.x + (b * V + ((size_t)nd * a.H + nh) * a.W + nw) * CIN + c * 8;
      }
      cp_async16(xs + row * C::XS + c * 8, src, in ? 16 : 0);
    }
    cp_async_commit();
    cp_async_wait<0>();
    __syncthreads();
    if (tap == 13 && tid < COUT)
      for (int row = 0; row < WG_ROWS; ++row) bsum += __bfloat162float(zs[row * C::ZS + tid]);
    for (int ks = wk; ks < WG_ROWS / 16; ks += C::WK) {
      const int k0 = ks * 16;
      uint32_t af[C::MT][4];
#pragma unroll
      for (int i = 0; i < C::MT; ++i) {
        const int m0 = wm * C::MW + i * 16;
        ldsm_x4_t(af[i], zs + (k0 + (q >> 1) * 8 + r8) * C::ZS + m0 + (q & 1) * 8);
      }
#pragma unroll
      for (int p = 0; p < C::NT / 2; ++p) {
        const int n0 = wn * C::NW + p * 16;
        uint32_t bfr[4];
        ldsm_x4_t(bfr, xs + (k0 + (q & 1) * 8 + r8) * C::XS + n0 + (q >> 1) * 8);
#pragma unroll
        for (int i = 0; i < C::MT; ++i) {
          mma_bf16(acc[i][2 * p], af[i], bfr[0], bfr[1]);
          mma_bf16(acc[i][2 * p + 1], af[i], bfr[2], bfr[3]);
        }
      }
    }
    __syncthreads();
  }

  // combine the K-split warps in a fixed order, write this chunk's partial
  float* red = (float*)smem;
#pragma unroll
  for (int i = 0; i < C::MT; ++i)
#pragma unroll
    for (int j = 0; j < C::NT; ++j)
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const int m = wm * C::MW + i * 16 + (lane >> 2) + (e >> 1) * 8;
        const int n = wn * C::NW + j * 8 + (lane & 3) * 2 + (e & 1);
        red[((size_t)wk * COUT + m) * CIN + n] = acc[i][j][e];
      }
  __syncthreads();
  float* out = a.part + ((size_t)blockIdx.x * 27 + tap) * COUT * CIN;
  for (int i = tid; i < COUT * CIN; i += NTHR) {
    float s = red[i];
    for (int k = 1; k < C::WK; ++k) s += red[(size_t)k * COUT * CIN + i];
    out[i] = s;
  }
  if (tap == 13 && tid < COUT) a.part_b[(size_t)blockIdx.x * COUT + tid] = bsum;
}

__global__ void reduce_chunks_kernel(const float* part, int nchunk, size_t n, float* out) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int c = 0; c < nchunk; ++c) s += part[(size_t)c * n + i];
    out[i] = s;
  }
}

// ---- dispatch -----------------------------------------------------------------

inline int nchunks(int B, int D, int H, int W) {
  const size_t tiles = ((size_t)B * D * H * W + WG_ROWS - 1) / WG_ROWS;
  const size_t want = 8;   // x 27 taps = 216 CTAs, about 1.4 waves on 152 SMs
  return (int)(tiles < want ? tiles : want);
}

template <int CIN, int COUT>
int fwd_launch(const FwdArgs& a, int B, cudaStream_t st) {
  using C = FwdCfg<CIN, COUT>;
  static bool attr = false;
  if (!attr) {
    if (cudaFuncSetAttribute(conv3_fwd_kernel<CIN, COUT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)C::SMEM) != cudaSuccess)
      return TBSG_ERR_CUDA;
    attr = true;
  }
  const int nb = ((a.D + TD - 1) / TD) * ((a.H + TH - 1) / TH) * ((a.W + TW - 1) / TW);
  conv3_fwd_kernel<CIN, COUT><<<dim3(nb, 1, B), NTHR, C::SMEM, st>>>(a);
  return cudaGetLastError() == cudaSuccess ? TBSG_OK : TBSG_ERR_CUDA;
}

template <int CIN, int COUT>
int wgrad_launch(const WgArgs& a, int nch, float* dw, float* db, cudaStream_t st) {
  using C = WgCfg<CIN, COUT>;
  static bool attr = false;
  if (!attr) {
    if (cudaFuncSetAttribute(conv3_wgrad_kernel<CIN, COUT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)C::SMEM) != cudaSuccess)
      return TBSG_ERR_CUDA;
    attr = true;
  }
  conv3_wgrad_kernel<CIN, COUT><<<dim3(nch, 27, 1), NTHR, C::SMEM, st>>>(a);
  const size_t nw = (size_t)27 * COUT * CIN;
  reduce_chunks_kernel<<<(int)((nw + 255) / 256), 256, 0, st>>>(a.part, nch, nw, dw);
  if (db) reduce_chunks_kernel<<<1, 256, 0, st>>>(a.part_b, nch, COUT, db);
  return cudaGetLastError() == cudaSuccess ? TBSG_OK : TBSG_ERR_CUDA;
}

// the (CIN, COUT) pairs of the network; the input gradient uses the reversed pair
#define SG_PAIRS(X) X(16, 16) X(16, 32) X(32, 16) X(32, 32) X(32, 64) X(64, 32) X(64, 64) X(64, 128) X(128, 64) X(128, 128)

int conv3_fwd_tc(const void* x, int cin, const void* w, const float* bias, const void* skip, void* y, float* yf,
                 int yf_accumulate, int cout, int batch, int D, int H, int W, int act, float slope, const void* yact,
                 float* dskip, cudaStream_t st);
int conv3_fwd_tcs(const void* x, int cin, const void* w, const float* bias, const void* skip, void* y, float* yf,
                  int yf_accumulate, int cout, int batch, int D, int H, int W, int act, float slope, const void* yact,
                  float* dskip, cudaStream_t st);
int g_conv_path = 0;   // 0: tcgen05 where built, else mma.sync; 1: mma.sync only
size_t wgrad_tc_scratch_bytes(int cin, int cout, int batch, int D, int H, int W);
int wgrad_tc(const void* x, int cin, const void* dz, int cout, int batch, int D, int H, int W, float* dw, float* db,
             void* scratch, cudaStream_t st);

}  // namespace sg

namespace sg {

// The convolution of tbsg_conv3_fwd / tbsg_conv3_dgrad_act: tcgen05 kernels
// where built (path 0), else (or with path 1) the mma.sync kernels.
int conv3_any(const void* x, int cin, const void* w, const float* bias, const void* skip, void* y, float* yf,
              int yf_accumulate, int cout, int batch, int D, int H, int W, int act, float slope, const void* yact,
              float* dskip, cudaStream_t st) {
  FwdArgs a;
  a.x = (const bf16*)x; a.w = (const bf16*)w; a.bias = bias; a.skip = (const bf16*)skip;
  a.y = (bf16*)y; a.yf = yf;
  a.D = D; a.H = H; a.W = W;
  a.act = act; a.slope = slope;
  a.mode = yact ? 3 : (yf ? (yf_accumulate ? 1 : 2) : 0);
  a.yact = (const bf16*)yact; a.dskip = dskip;
  if (g_conv_path == 0) {
    int rc = conv3_fwd_tc(x, cin, w, bias, skip, y, yf, yf_accumulate, cout, batch, D, H, W, act, slope, yact, dskip,
                          st);
    if (rc != TBSG_ERR_SHAPE) return rc;
    rc = conv3_fwd_tcs(x, cin, w, bias, skip, y, yf, yf_accumulate, cout, batch, D, H, W, act, slope, yact, dskip, st);
    if (rc != TBSG_ERR_SHAPE) return rc;
  }
#define SG_FWD(I, O) \
  if (cin == I && cout == O) return fwd_launch<I, O>(a, batch, st);
  SG_PAIRS(SG_FWD)
#undef SG_FWD
  return TBSG_ERR_SHAPE;
}

}  // namespace sg

using namespace sg;

extern "C" {

int tbsg_set_conv_path(int path) {
  if (path < 0 || path > 1) return TBSG_ERR_ARG;
  g_conv_path = path;
  return TBSG_OK;
}

int tbsg_conv3_fwd(const void* x, int cin, const void* w, const float* bias, const void* skip, void* y,
                   float* yf, int yf_accumulate, int cout, int batch, int D, int H, int W, int act, float slope,
                   void* stream) {
  if (!x || !w || (!y && !yf) || batch <= 0 || D <= 0 || H <= 0 || W <= 0) return TBSG_ERR_ARG;
  return conv3_any(x, cin, w, bias, skip, y, yf, yf_accumulate, cout, batch, D, H, W, act, slope, nullptr, nullptr,
                   (cudaStream_t)stream);
}

int tbsg_conv3_dgrad_act(const void* dz, int cout, const void* wt, const void* y_in, void* dz_in, float* dskip,
                         int cin, int batch, int D, int H, int W, float slope, void* stream) {
  if (!dz || !wt || !y_in || !dz_in || batch <= 0 || D <= 0 || H <= 0 || W <= 0) return TBSG_ERR_ARG;
  if (((uintptr_t)y_in | (uintptr_t)dz_in | (uintptr_t)dskip) % 16) return TBSG_ERR_ARG;
  return conv3_any(dz, cout, wt, nullptr, nullptr, dz_in, nullptr, 0, cin, batch, D, H, W, 0, slope, y_in, dskip,
                   (cudaStream_t)stream);
}

size_t tbsg_conv3_wgrad_scratch_bytes(int cin, int cout, int batch, int D, int H, int W) {
  const int nch = nchunks(batch, D, H, W);
  const size_t ms = ((size_t)nch * 27 * cout * cin + (size_t)nch * cout) * sizeof(float);
  const size_t tc = wgrad_tc_scratch_bytes(cin, cout, batch, D, H, W);
  return ms > tc ? ms : tc;
}

int tbsg_conv3_wgrad(const void* x, int cin, const void* dz, int cout, int batch, int D, int H, int W,
                     float* dw, float* db, void* scratch, size_t scratch_bytes, void* stream) {
  if (!x || !dz || !dw || !scratch || batch <= 0 || D <= 0 || H <= 0 || W <= 0) return TBSG_ERR_ARG;
  if (scratch_bytes < tbsg_conv3_wgrad_scratch_bytes(cin, cout, batch, D, H, W)) return TBSG_ERR_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  if (g_conv_path == 0) {
    const int rc = wgrad_tc(x, cin, dz, cout, batch, D, H, W, dw, db, scratch, st);
    if (rc != TBSG_ERR_SHAPE) return rc;
  }
  const int nch = nchunks(batch, D, H, W);
  WgArgs a;
  a.x = (const bf16*)x; a.dz = (const bf16*)dz;
  a.part = (float*)scratch;
  a.part_b = (float*)scratch + (size_t)nch * 27 * cout * cin;
  a.B = batch; a.D = D; a.H = H; a.W = W;
#define SG_WG(I, O) \
  if (cin == I && cout == O) return wgrad_launch<I, O>(a, nch, dw, db, st);
  SG_PAIRS(SG_WG)
#undef SG_WG
  return TBSG_ERR_SHAPE;
}

}  // extern "C"
