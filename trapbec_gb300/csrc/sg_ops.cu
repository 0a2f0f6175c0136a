// sg_ops.cu -- the memory-bound pieces of the warm-start surrogate: weight
// preparation, activation gradient, pooling/upsampling and their gradients,
// the FP32 output head with its loss, Adam.  Grid-stride loops over
// 16-byte (8 x BF16) or 4 x FP32 vectors where the layout allows.
#include "../../include/trapbec_surrogate.h"
#include "sg_common.cuh"

namespace sg {

inline int grid_for(size_t n, int per_thread = 1) {
  size_t b = (n / per_thread + 255) / 256;
  if (b < 1) b = 1;
  if (b > 152 * 16) b = 152 * 16;
  return (int)b;
}

__global__ void weight_prep_kernel(const float* w32, bf16* w, bf16* wt, int cin, int cout) {
  const size_t n = (size_t)27 * cout * cin;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int ci = (int)(i % cin);
    const size_t r = i / cin;
    const int co = (int)(r % cout), tap = (int)(r / cout);
    const bf16 v = __float2bfloat16_rn(w32[i]);
    w[i] = v;
    wt[((size_t)(26 - tap) * cin + ci) * cout + co] = v;
  }
}

__global__ void act_bwd_kernel(const float* dy, const bf16* y, bf16* dz, float* dskip, size_t n, float slope) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const float g = dy[i] * (__bfloat162float(y[i]) > 0.f ? 1.f : slope);
    const bf16 gb = __float2bfloat16_rn(g);
    dz[i] = gb;
    if (dskip) dskip[i] += g;
  }
}

// the same, 8 elements per thread (n % 8 == 0, 16-byte aligned arrays)
__global__ void act_bwd8_kernel(const float4* dy, const uint4* y, uint4* dz, float4* dskip, size_t n8, float slope) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n8; i += (size_t)gridDim.x * blockDim.x) {
    const float4 a = dy[2 * i], b = dy[2 * i + 1];
    const uint4 yu = y[i];
    const bf16* ye = (const bf16*)&yu;
    float g[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
#pragma unroll
    for (int k = 0; k < 8; ++k) g[k] *= __bfloat162float(ye[k]) > 0.f ? 1.f : slope;
    uint4 o;
    bf16* oe = (bf16*)&o;
#pragma unroll
    for (int k = 0; k < 8; ++k) oe[k] = __float2bfloat16_rn(g[k]);
    dz[i] = o;
    if (dskip) {
      float4 s0 = dskip[2 * i], s1 = dskip[2 * i + 1];
      s0.x += g[0]; s0.y += g[1]; s0.z += g[2]; s0.w += g[3];
      s1.x += g[4]; s1.y += g[5]; s1.z += g[6]; s1.w += g[7];
      dskip[2 * i] = s0;
      dskip[2 * i + 1] = s1;
    }
  }
}

// fine grid (D, H, W) -> coarse (D/2, H/2, W/2); one thread per coarse voxel x 8 channels
__global__ void pool2_fwd_kernel(const bf16* x, bf16* y, int c, int B, int D, int H, int W) {
  const int Dc = D / 2, Hc = H / 2, Wc = W / 2, c8 = c / 8;
  const size_t n = (size_t)B * Dc * Hc * Wc * c8;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int cc = (int)(i % c8);
    size_t r = i / c8;
    const int w = (int)(r % Wc); r /= Wc;
    const int h = (int)(r % Hc); r /= Hc;
    const int d = (int)(r % Dc);
    const size_t b = r / Dc;
    float s[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int o = 0; o < 8; ++o) {
      const int fd = 2 * d + (o >> 2), fh = 2 * h + ((o >> 1) & 1), fw = 2 * w + (o & 1);
      const uint4 u = *(const uint4*)(x + (((b * D + fd) * H + fh) * W + fw) * c + cc * 8);
      const bf16* e = (const bf16*)&u;
      for (int k = 0; k < 8; ++k) s[k] += __bfloat162float(e[k]);
    }
    uint4 o4;
    bf16* e = (bf16*)&o4;
    for (int k = 0; k < 8; ++k) e[k] = __float2bfloat16_rn(s[k] * 0.125f);
    *(uint4*)(y + (((b * Dc + d) * Hc + h) * Wc + w) * c + cc * 8) = o4;
  }
}

// one thread per coarse voxel x 4 channels: dx of its 8 fine voxels += dy / 8
__global__ void pool2_bwd4_kernel(const float* dy, float* dx, int c, int B, int D, int H, int W) {
  const int Dc = D / 2, Hc = H / 2, Wc = W / 2, c4 = c / 4;
  const size_t n = (size_t)B * Dc * Hc * Wc * c4;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int cc = (int)(i % c4);
    size_t r = i / c4;
    const int w = (int)(r % Wc); r /= Wc;
    const int h = (int)(r % Hc); r /= Hc;
    const int d = (int)(r % Dc);
    const size_t b = r / Dc;
    float4 g = *(const float4*)(dy + i * 4);
    g.x *= 0.125f; g.y *= 0.125f; g.z *= 0.125f; g.w *= 0.125f;
#pragma unroll
    for (int o = 0; o < 8; ++o) {
      const int fd = 2 * d + (o >> 2), fh = 2 * h + ((o >> 1) & 1), fw = 2 * w + (o & 1);
      float4* q = (float4*)(dx + (((b * D + fd) * H + fh) * W + fw) * c + cc * 4);
      float4 t = *q;
      t.x += g.x; t.y += g.y; t.z += g.z; t.w += g.w;
      *q = t;
    }
  }
}

__global__ void pool2_bwd_kernel(const float* dy, float* dx, int c, int B, int D, int H, int W) {
  const int Dc = D / 2, Hc = H / 2, Wc = W / 2;
  const size_t n = (size_t)B * D * H * W * c;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int cc = (int)(i % c);
    size_t r = i / c;
    const int w = (int)(r % W); r /= W;
    const int h = (int)(r % H); r /= H;
    const int d = (int)(r % D);
    const size_t b = r / D;
    dx[i] += 0.125f * dy[(((b * Dc + d / 2) * Hc + h / 2) * Wc + w / 2) * c + cc];
  }
}

// coarse (D, H, W) -> fine (2D, 2H, 2W)
__global__ void up2_fwd_kernel(const bf16* x, bf16* y, int c, int B, int D, int H, int W) {
  const int c8 = c / 8, Df = 2 * D, Hf = 2 * H, Wf = 2 * W;
  const size_t n = (size_t)B * Df * Hf * Wf * c8;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int cc = (int)(i % c8);
    size_t r = i / c8;
    const int w = (int)(r % Wf); r /= Wf;
    const int h = (int)(r % Hf); r /= Hf;
    const int d = (int)(r % Df);
    const size_t b = r / Df;
    *(uint4*)(y + i * 8) = *(const uint4*)(x + (((b * D + d / 2) * H + h / 2) * W + w / 2) * c + cc * 8);
  }
}

// one thread per coarse voxel x 8 channels: its 16 bytes read once and
// written to its 8 fine voxels (a warp's writes cover whole fine rows)
__global__ void up2_fwd8_kernel(const bf16* x, bf16* y, int c, int B, int D, int H, int W) {
  const int c8 = c / 8, Df = 2 * D, Hf = 2 * H, Wf = 2 * W;
  const size_t n = (size_t)B * D * H * W * c8;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int cc = (int)(i % c8);
    size_t r = i / c8;
    const int w = (int)(r % W); r /= W;
    const int h = (int)(r % H); r /= H;
    const int d = (int)(r % D);
    const size_t b = r / D;
    const uint4 v = *(const uint4*)(x + i * 8);
#pragma unroll
    for (int o = 0; o < 8; ++o) {
      const int fd = 2 * d + (o >> 2), fh = 2 * h + ((o >> 1) & 1), fw = 2 * w + (o & 1);
      *(uint4*)(y + (((b * Df + fd) * Hf + fh) * Wf + fw) * c + cc * 8) = v;
    }
  }
}

// one thread per coarse voxel x 4 channels: the sum of its 8 fine gradients
__global__ void up2_bwd4_kernel(const float* dy, float* dx, int c, int B, int D, int H, int W) {
  const int Hf = 2 * H, Wf = 2 * W, Df = 2 * D, c4 = c / 4;
  const size_t n = (size_t)B * D * H * W * c4;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int cc = (int)(i % c4);
    size_t r = i / c4;
    const int w = (int)(r % W); r /= W;
    const int h = (int)(r % H); r /= H;
    const int d = (int)(r % D);
    const size_t b = r / D;
    float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int o = 0; o < 8; ++o) {
      const int fd = 2 * d + (o >> 2), fh = 2 * h + ((o >> 1) & 1), fw = 2 * w + (o & 1);
      const float4 t = *(const float4*)(dy + (((b * Df + fd) * Hf + fh) * Wf + fw) * c + cc * 4);
      s.x += t.x; s.y += t.y; s.z += t.z; s.w += t.w;
    }
    *(float4*)(dx + i * 4) = s;
  }
}

__global__ void up2_bwd_kernel(const float* dy, float* dx, int c, int B, int D, int H, int W) {
  const int Hf = 2 * H, Wf = 2 * W, Df = 2 * D;
  const size_t n = (size_t)B * D * H * W * c;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int cc = (int)(i % c);
    size_t r = i / c;
    const int w = (int)(r % W); r /= W;
    const int h = (int)(r % H); r /= H;
    const int d = (int)(r % D);
    const size_t b = r / D;
    float s = 0.f;
    for (int o = 0; o < 8; ++o) {
      const int fd = 2 * d + (o >> 2), fh = 2 * h + ((o >> 1) & 1), fw = 2 * w + (o & 1);
      s += dy[(((b * Df + fd) * Hf + fh) * Wf + fw) * c + cc];
    }
    dx[i] = s;
  }
}

// The activation-gradient fusions of the backward pass: the same operations,
// in the same order, as the gradient kernel followed by act_bwd, without the
// FP32 gradient in memory.  dz = BF16(g * act'(y)), act' = 1 where y > 0,
// else slope, for 8 channels of one voxel.
__device__ __forceinline__ uint4 act_dz8(const float g[8], const uint4 yu, float slope) {
  const bf16* ye = (const bf16*)&yu;
  uint4 o;
  bf16* oe = (bf16*)&o;
#pragma unroll
  for (int k = 0; k < 8; ++k) oe[k] = __float2bfloat16_rn(g[k] * (__bfloat162float(ye[k]) > 0.f ? 1.f : slope));
  return o;
}

// pooling gradient + activation: one thread per coarse voxel x 8 channels;
// each of its 8 fine voxels takes g = g_fine + dy / 8, then dz_fine
__global__ void pool2_bwd_act8_kernel(const float* dy, const float* gf, const bf16* y, bf16* dz, int c, int B, int D,
                                      int H, int W, float slope) {
  const int Dc = D / 2, Hc = H / 2, Wc = W / 2, c8 = c / 8;
  const size_t n = (size_t)B * Dc * Hc * Wc * c8;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int cc = (int)(i % c8);
    size_t r = i / c8;
    const int w = (int)(r % Wc); r /= Wc;
    const int h = (int)(r % Hc); r /= Hc;
    const int d = (int)(r % Dc);
    const size_t b = r / Dc;
    const float4 a0 = *(const float4*)(dy + i * 8), a1 = *(const float4*)(dy + i * 8 + 4);
    const float q[8] = {0.125f * a0.x, 0.125f * a0.y, 0.125f * a0.z, 0.125f * a0.w,
                        0.125f * a1.x, 0.125f * a1.y, 0.125f * a1.z, 0.125f * a1.w};
#pragma unroll
    for (int o = 0; o < 8; ++o) {
      const int fd = 2 * d + (o >> 2), fh = 2 * h + ((o >> 1) & 1), fw = 2 * w + (o & 1);
      const size_t f = (((b * D + fd) * H + fh) * W + fw) * c + cc * 8;
      const float4 g0 = *(const float4*)(gf + f), g1 = *(const float4*)(gf + f + 4);
      const float g[8] = {g0.x + q[0], g0.y + q[1], g0.z + q[2], g0.w + q[3],
                          g1.x + q[4], g1.y + q[5], g1.z + q[6], g1.w + q[7]};
      *(uint4*)(dz + f) = act_dz8(g, *(const uint4*)(y + f), slope);
    }
  }
}

// upsampling gradient + activation: one thread per coarse voxel x 8 channels:
// g = the sum of its 8 fine gradients (in fine-voxel order), then dz_coarse
__global__ void up2_bwd_act8_kernel(const float* dy, const bf16* y, bf16* dz, int c, int B, int D, int H, int W,
                                    float slope) {
  const int Hf = 2 * H, Wf = 2 * W, Df = 2 * D, c8 = c / 8;
  const size_t n = (size_t)B * D * H * W * c8;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int cc = (int)(i % c8);
    size_t r = i / c8;
    const int w = (int)(r % W); r /= W;
    const int h = (int)(r % H); r /= H;
    const int d = (int)(r % D);
    const size_t b = r / D;
    float g[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int o = 0; o < 8; ++o) {
      const int fd = 2 * d + (o >> 2), fh = 2 * h + ((o >> 1) & 1), fw = 2 * w + (o & 1);
      const float* src = dy + (((b * Df + fd) * Hf + fh) * Wf + fw) * c + cc * 8;
      const float4 t0 = *(const float4*)src, t1 = *(const float4*)(src + 4);
      g[0] += t0.x; g[1] += t0.y; g[2] += t0.z; g[3] += t0.w;
      g[4] += t1.x; g[5] += t1.y; g[6] += t1.z; g[7] += t1.w;
    }
    *(uint4*)(dz + i * 8) = act_dz8(g, *(const uint4*)(y + i * 8), slope);
  }
}

constexpr int HEAD_THREADS = 256;
constexpr int HEAD_BLOCKS = 1024;

__global__ void head_fwd_kernel(const bf16* feat, int c, const float* wh, const float* bh, const float* base,
                                float* amp, size_t nvox) {
  for (size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x; v < nvox; v += (size_t)gridDim.x * blockDim.x) {
    float s = bh[0];
    for (int k = 0; k < c; ++k) s += __bfloat162float(feat[v * c + k]) * wh[k];
    amp[v] = base[v] + s;
  }
}

// per-block partials [blocks][c + 2]: loss, dwh[c], dbh
__global__ void head_loss_kernel(const bf16* feat, int c, const float* wh, const float* bh, const float* base,
                                 const float* target, size_t nvox, float* dfeat, float* partials) {
  extern __shared__ float red[];   // [HEAD_THREADS][c + 2]
  const int np = c + 2;
  float acc[130];
  for (int k = 0; k < np; ++k) acc[k] = 0.f;
  const float inv = 1.f / (float)nvox;
  for (size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x; v < nvox; v += (size_t)gridDim.x * blockDim.x) {
    float s = bh[0];
    for (int k = 0; k < c; ++k) s += __bfloat162float(feat[v * c + k]) * wh[k];
    const float diff = base[v] + s - target[v];
    const float g = 2.f * diff * inv;
    acc[0] += diff * diff * inv;
    for (int k = 0; k < c; ++k) {
      acc[1 + k] += g * __bfloat162float(feat[v * c + k]);
      dfeat[v * c + k] = g * wh[k];
    }
    acc[c + 1] += g;
  }
  for (int k = 0; k < np; ++k) red[threadIdx.x * np + k] = acc[k];
  __syncthreads();
  for (int s = HEAD_THREADS / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s)
      for (int k = 0; k < np; ++k) red[threadIdx.x * np + k] += red[(threadIdx.x + s) * np + k];
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int k = 0; k < np; ++k) partials[(size_t)blockIdx.x * np + k] = red[k];
}

// 16 feature channels: one voxel per thread, the channels as two 16-byte loads
__global__ void head_fwd16_kernel(const uint4* feat, const float* wh, const float* bh, const float* base, float* amp,
                                  size_t nvox) {
  float w[16];
#pragma unroll
  for (int k = 0; k < 16; ++k) w[k] = wh[k];
  const float b0 = bh[0];
  for (size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x; v < nvox; v += (size_t)gridDim.x * blockDim.x) {
    const uint4 u0 = feat[2 * v], u1 = feat[2 * v + 1];
    const bf16* e0 = (const bf16*)&u0;
    const bf16* e1 = (const bf16*)&u1;
    float s = b0;
#pragma unroll
    for (int k = 0; k < 8; ++k) s += __bfloat162float(e0[k]) * w[k];
#pragma unroll
    for (int k = 0; k < 8; ++k) s += __bfloat162float(e1[k]) * w[8 + k];
    amp[v] = base[v] + s;
  }
}

template <bool ACT>
__global__ void __launch_bounds__(HEAD_THREADS) head_loss16_kernel(const uint4* feat, const float* wh, const float* bh,
                                                                   const float* base, const float* target, size_t nvox,
                                                                   float4* dfeat, uint4* dz, float slope,
                                                                   float* partials) {
  constexpr int NP = 18;
  __shared__ float red[HEAD_THREADS * NP];
  float w[16], acc[NP];
#pragma unroll
  for (int k = 0; k < 16; ++k) w[k] = wh[k];
#pragma unroll
  for (int k = 0; k < NP; ++k) acc[k] = 0.f;
  const float b0 = bh[0];
  const float inv = 1.f / (float)nvox;
  for (size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x; v < nvox; v += (size_t)gridDim.x * blockDim.x) {
    const uint4 u0 = feat[2 * v], u1 = feat[2 * v + 1];
    const bf16* e0 = (const bf16*)&u0;
    const bf16* e1 = (const bf16*)&u1;
    float f[16];
#pragma unroll
    for (int k = 0; k < 8; ++k) { f[k] = __bfloat162float(e0[k]); f[8 + k] = __bfloat162float(e1[k]); }
    float s = b0;
#pragma unroll
    for (int k = 0; k < 16; ++k) s += f[k] * w[k];
    const float diff = base[v] + s - target[v];
    const float g = 2.f * diff * inv;
    acc[0] += diff * diff * inv;
#pragma unroll
    for (int k = 0; k < 16; ++k) acc[1 + k] += g * f[k];
    acc[17] += g;
    if (ACT) {   // dz = BF16(d loss/d feat * act'(feat)): the head's input is a leaky ReLU's output
      float t[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) t[k] = g * w[k];
      dz[2 * v] = act_dz8(t, u0, slope);
#pragma unroll
      for (int k = 0; k < 8; ++k) t[k] = g * w[8 + k];
      dz[2 * v + 1] = act_dz8(t, u1, slope);
    } else {
#pragma unroll
      for (int q = 0; q < 4; ++q)
        dfeat[4 * v + q] = make_float4(g * w[4 * q], g * w[4 * q + 1], g * w[4 * q + 2], g * w[4 * q + 3]);
    }
  }
#pragma unroll
  for (int k = 0; k < NP; ++k) red[k * HEAD_THREADS + threadIdx.x] = acc[k];
  __syncthreads();
  for (int h = HEAD_THREADS / 2; h > 0; h >>= 1) {
    if ((int)threadIdx.x < h)
#pragma unroll
      for (int k = 0; k < NP; ++k) red[k * HEAD_THREADS + threadIdx.x] += red[k * HEAD_THREADS + threadIdx.x + h];
    __syncthreads();
  }
  if ((int)threadIdx.x < NP) partials[(size_t)blockIdx.x * NP + threadIdx.x] = red[threadIdx.x * HEAD_THREADS];
}

// out[k] = sum over the blocks' partials of quantity k: each of 256 threads
// adds a fixed strided subset, then one fixed shared-memory tree per quantity
__global__ void __launch_bounds__(256) head_final_kernel(const float* partials, int nblk, int np, float* out) {
  __shared__ float red[256];
  for (int k = 0; k < np; ++k) {
    float s = 0.f;
    for (int b = threadIdx.x; b < nblk; b += 256) s += partials[(size_t)b * np + k];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int h = 128; h > 0; h >>= 1) {
      if ((int)threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
      __syncthreads();
    }
    if (threadIdx.x == 0) out[k] = red[0];
    __syncthreads();
  }
}

__global__ void adam_kernel(float* p, const float* g, float* m, float* v, size_t n, float lr, float b1, float b2,
                            float eps, float wd, float bc1, float bc2, const float* gscale) {
  const float gs = gscale ? gscale[0] : 1.f;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const float gi = g[i] * gs;
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float mh = mi / bc1, vh = vi / bc2;
    p[i] -= lr * (mh / (sqrtf(vh) + eps) + wd * p[i]);
  }
}

constexpr int CLIP_BLOCKS = 1024;

__global__ void sumsq_kernel(const float* g, size_t n, float* partials) {
  __shared__ double red[256];
  double s = 0.0;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    s += (double)g[i] * g[i];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int k = 128; k > 0; k >>= 1) {
    if ((int)threadIdx.x < k) red[threadIdx.x] += red[threadIdx.x + k];
    __syncthreads();
  }
  if (threadIdx.x == 0) partials[blockIdx.x] = (float)red[0];
}

// the block partials summed in FP64 by 256 threads (fixed strided subsets and
// a fixed tree), then the norm and the clipping factor
__global__ void __launch_bounds__(256) clip_final_kernel(const float* partials, int nblk, float max_norm, float* out) {
  __shared__ double red[256];
  double s = 0.0;
  for (int b = threadIdx.x; b < nblk; b += 256) s += partials[b];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int h = 128; h > 0; h >>= 1) {
    if ((int)threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double nrm = sqrt(red[0]);
    out[0] = (float)nrm;
    out[1] = nrm > max_norm ? (float)(max_norm / nrm) : 1.f;
  }
}

__global__ void f32_to_bf16_kernel(const float* x, bf16* y, size_t n) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    y[i] = __float2bfloat16_rn(x[i]);
}

// Input channels of one instance: one thread per voxel writes the 16 BF16
// channels (channels-last) and the FP32 Thomas-Fermi amplitude.  Coordinates,
// harmonic potential and amplitude follow the host recipe operation by
// operation in FP64 with explicit rounding (no contraction), then round to
// FP32 and from FP32 to BF16, so the result equals the converted host arrays.
struct FeatConsts { float c[8]; };   // channels 2-9 (constant over the grid)

__device__ __forceinline__ double feat_coord(int idx, int m, double L) {   // ((2(idx+1)-1)/(2m) L - L/2) / L
  const double q = __ddiv_rn((double)(2 * idx + 1), 2.0 * (double)m);
  return __ddiv_rn(__dsub_rn(__dmul_rn(q, L), L / 2.0), L);
}

__global__ void features_kernel(bf16* __restrict__ x, float* __restrict__ base, int nx, int ny, int nz, double lx,
                                double ly, double lz, double wx, double wy, double wz, FeatConsts fc) {
  const size_t n = (size_t)nx * ny * nz;
  for (size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (size_t)gridDim.x * blockDim.x) {
    const int k = (int)(v % nz);
    const int j = (int)((v / nz) % ny);
    const int i = (int)(v / ((size_t)ny * nz));
    const double X = feat_coord(i, nx, lx), Y = feat_coord(j, ny, ly), Z = feat_coord(k, nz, lz);
    const double pot = __dadd_rn(__dadd_rn(__dmul_rn(wx, __dmul_rn(X, X)), __dmul_rn(wy, __dmul_rn(Y, Y))),
                                 __dmul_rn(wz, __dmul_rn(Z, Z)));
    const float b = __double2float_rn(sqrt(fmax(0.0, __dsub_rn(1.0, pot))));
    bf16* o = x + v * 16;
    o[0] = __float2bfloat16_rn(__double2float_rn(fmin(pot, 2.0)));
    o[1] = __float2bfloat16_rn(b);
#pragma unroll
    for (int q = 0; q < 8; ++q) o[2 + q] = __float2bfloat16_rn(fc.c[q]);
#pragma unroll
    for (int q = 10; q < 16; ++q) o[q] = __float2bfloat16_rn(0.0f);
    base[v] = b;
  }
}

inline int done() { return cudaGetLastError() == cudaSuccess ? TBSG_OK : TBSG_ERR_CUDA; }

}  // namespace sg

using namespace sg;

extern "C" {

int tbsg_weight_prep(const float* w32, void* w, void* wt, int cin, int cout, void* stream) {
  if (!w32 || !w || !wt || cin <= 0 || cout <= 0) return TBSG_ERR_ARG;
  weight_prep_kernel<<<grid_for((size_t)27 * cin * cout), 256, 0, (cudaStream_t)stream>>>(w32, (bf16*)w, (bf16*)wt,
                                                                                          cin, cout);
  return done();
}

int tbsg_act_bwd(const float* dy, const void* y, void* dz, float* dskip, size_t n, float slope, void* stream) {
  if (!dy || !y || !dz) return TBSG_ERR_ARG;
  const bool vec = n % 8 == 0 && ((uintptr_t)dy | (uintptr_t)y | (uintptr_t)dz | (uintptr_t)dskip) % 16 == 0;
  if (vec)
    act_bwd8_kernel<<<grid_for(n / 8), 256, 0, (cudaStream_t)stream>>>(
        (const float4*)dy, (const uint4*)y, (uint4*)dz, (float4*)dskip, n / 8, slope);
  else
    act_bwd_kernel<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(dy, (const bf16*)y, (bf16*)dz, dskip, n, slope);
  return done();
}

int tbsg_pool2_fwd(const void* x, void* y, int c, int batch, int D, int H, int W, void* stream) {
  if (!x || !y || c % 8 || (D | H | W) & 1) return TBSG_ERR_ARG;
  pool2_fwd_kernel<<<grid_for((size_t)batch * D * H * W * c / 64), 256, 0, (cudaStream_t)stream>>>(
      (const bf16*)x, (bf16*)y, c, batch, D, H, W);
  return done();
}

int tbsg_pool2_bwd(const float* dy, float* dx, int c, int batch, int D, int H, int W, void* stream) {
  if (!dy || !dx || (D | H | W) & 1) return TBSG_ERR_ARG;
  if (c % 4 == 0 && ((uintptr_t)dy | (uintptr_t)dx) % 16 == 0)
    pool2_bwd4_kernel<<<grid_for((size_t)batch * D * H * W * c / 32), 256, 0, (cudaStream_t)stream>>>(dy, dx, c, batch,
                                                                                                    D, H, W);
  else
    pool2_bwd_kernel<<<grid_for((size_t)batch * D * H * W * c), 256, 0, (cudaStream_t)stream>>>(dy, dx, c, batch, D,
                                                                                                H, W);
  return done();
}

int tbsg_up2_fwd(const void* x, void* y, int c, int batch, int D, int H, int W, void* stream) {
  if (!x || !y || c % 8) return TBSG_ERR_ARG;
  if (((uintptr_t)x | (uintptr_t)y) % 16 == 0)
    up2_fwd8_kernel<<<grid_for((size_t)batch * D * H * W * c / 8), 256, 0, (cudaStream_t)stream>>>(
        (const bf16*)x, (bf16*)y, c, batch, D, H, W);
  else
    up2_fwd_kernel<<<grid_for((size_t)batch * D * H * W * c), 256, 0, (cudaStream_t)stream>>>(
        (const bf16*)x, (bf16*)y, c, batch, D, H, W);
  return done();
}

int tbsg_up2_bwd(const float* dy, float* dx, int c, int batch, int D, int H, int W, void* stream) {
  if (!dy || !dx) return TBSG_ERR_ARG;
  if (c % 4 == 0 && ((uintptr_t)dy | (uintptr_t)dx) % 16 == 0)
    up2_bwd4_kernel<<<grid_for((size_t)batch * D * H * W * c / 4), 256, 0, (cudaStream_t)stream>>>(dy, dx, c, batch, D,
                                                                                                  H, W);
  else
    up2_bwd_kernel<<<grid_for((size_t)batch * D * H * W * c), 256, 0, (cudaStream_t)stream>>>(dy, dx, c, batch, D, H,
                                                                                              W);
  return done();
}

int tbsg_head_fwd(const void* feat, int c, const float* wh, const float* bh, const float* base, float* amp,
                  size_t nvox, void* stream) {
  if (!feat || !wh || !bh || !base || !amp || c <= 0) return TBSG_ERR_ARG;
  if (c == 16 && (uintptr_t)feat % 16 == 0)
    head_fwd16_kernel<<<grid_for(nvox), 256, 0, (cudaStream_t)stream>>>((const uint4*)feat, wh, bh, base, amp, nvox);
  else
    head_fwd_kernel<<<grid_for(nvox), 256, 0, (cudaStream_t)stream>>>((const bf16*)feat, c, wh, bh, base, amp, nvox);
  return done();
}

size_t tbsg_head_partials(size_t nvox, int c) {
  (void)nvox;
  return (size_t)HEAD_BLOCKS * (c + 2);
}

int tbsg_head_loss(const void* feat, int c, const float* wh, const float* bh, const float* base,
                   const float* target, size_t nvox, float* dfeat, float* partials, float* out, void* stream) {
  if (!feat || !wh || !bh || !base || !target || !dfeat || !partials || !out || c <= 0 || c > 128)
    return TBSG_ERR_ARG;
  const size_t smem = (size_t)HEAD_THREADS * (c + 2) * sizeof(float);
  if (smem > 48 * 1024) {
    if (cudaFuncSetAttribute(head_loss_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess)
      return TBSG_ERR_CUDA;
  }
  cudaStream_t st = (cudaStream_t)stream;
  if (c == 16 && ((uintptr_t)feat | (uintptr_t)dfeat) % 16 == 0)
    head_loss16_kernel<false><<<HEAD_BLOCKS, HEAD_THREADS, 0, st>>>((const uint4*)feat, wh, bh, base, target, nvox,
                                                                    (float4*)dfeat, nullptr, 0.f, partials);
  else
    head_loss_kernel<<<HEAD_BLOCKS, HEAD_THREADS, smem, st>>>((const bf16*)feat, c, wh, bh, base, target, nvox, dfeat,
                                                              partials);
  head_final_kernel<<<1, 256, 0, st>>>(partials, HEAD_BLOCKS, c + 2, out);
  return done();
}

int tbsg_head_loss_act(const void* feat, const float* wh, const float* bh, const float* base, const float* target,
                       size_t nvox, void* dz, float slope, float* partials, float* out, void* stream) {
  if (!feat || !wh || !bh || !base || !target || !dz || !partials || !out) return TBSG_ERR_ARG;
  if (((uintptr_t)feat | (uintptr_t)dz) % 16) return TBSG_ERR_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  head_loss16_kernel<true><<<HEAD_BLOCKS, HEAD_THREADS, 0, st>>>((const uint4*)feat, wh, bh, base, target, nvox,
                                                                 nullptr, (uint4*)dz, slope, partials);
  head_final_kernel<<<1, 256, 0, st>>>(partials, HEAD_BLOCKS, 16 + 2, out);
  return done();
}

int tbsg_pool2_bwd_act(const float* dy, const float* g, const void* y, void* dz, int c, int batch, int D, int H, int W,
                       float slope, void* stream) {
  if (!dy || !g || !y || !dz || (D | H | W) & 1 || c % 8) return TBSG_ERR_ARG;
  if (((uintptr_t)dy | (uintptr_t)g | (uintptr_t)y | (uintptr_t)dz) % 16) return TBSG_ERR_ARG;
  pool2_bwd_act8_kernel<<<grid_for((size_t)batch * D * H * W * c / 64), 256, 0, (cudaStream_t)stream>>>(
      dy, g, (const bf16*)y, (bf16*)dz, c, batch, D, H, W, slope);
  return done();
}

int tbsg_up2_bwd_act(const float* dy, const void* y, void* dz, int c, int batch, int D, int H, int W, float slope,
                     void* stream) {
  if (!dy || !y || !dz || c % 8) return TBSG_ERR_ARG;
  if (((uintptr_t)dy | (uintptr_t)y | (uintptr_t)dz) % 16) return TBSG_ERR_ARG;
  up2_bwd_act8_kernel<<<grid_for((size_t)batch * D * H * W * c / 8), 256, 0, (cudaStream_t)stream>>>(
      dy, (const bf16*)y, (bf16*)dz, c, batch, D, H, W, slope);
  return done();
}

int tbsg_adam(float* p, const float* g, float* m, float* v, size_t n, float lr, float beta1, float beta2, float eps,
              float weight_decay, int t, const float* grad_scale, void* stream) {
  if (!p || !g || !m || !v || t < 1) return TBSG_ERR_ARG;
  const float bc1 = 1.f - powf(beta1, (float)t), bc2 = 1.f - powf(beta2, (float)t);
  adam_kernel<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(p, g, m, v, n, lr, beta1, beta2, eps, weight_decay, bc1,
                                                            bc2, grad_scale);
  return done();
}

int tbsg_clip_scale(const float* g, size_t n, float max_norm, float* partials, float* out, void* stream) {
  if (!g || !partials || !out || !(max_norm > 0.f)) return TBSG_ERR_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  sumsq_kernel<<<CLIP_BLOCKS, 256, 0, st>>>(g, n, partials);
  clip_final_kernel<<<1, 256, 0, st>>>(partials, CLIP_BLOCKS, max_norm, out);
  return done();
}

int tbsg_features(void* x, float* base, int nx, int ny, int nz, double lx, double ly, double lz, double wx, double wy,
                  double wz, const float* consts, void* stream) {
  if (!x || !base || !consts || nx <= 0 || ny <= 0 || nz <= 0 || !(lx > 0) || !(ly > 0) || !(lz > 0)) return TBSG_ERR_ARG;
  FeatConsts fc;
  for (int q = 0; q < 8; ++q) fc.c[q] = consts[q];
  const size_t n = (size_t)nx * ny * nz;
  features_kernel<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>((bf16*)x, base, nx, ny, nz, lx, ly, lz, wx, wy, wz, fc);
  return done();
}

int tbsg_f32_to_bf16(const float* x, void* y, size_t n, void* stream) {
  if (!x || !y) return TBSG_ERR_ARG;
  f32_to_bf16_kernel<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(x, (bf16*)y, n);
  return done();
}

}  // extern "C"
