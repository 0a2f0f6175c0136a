// sg_common.cuh -- shared pieces of the warm-start surrogate's kernels.
//
// The surrogate is a 3D convolutional encoder-decoder over channels-last
// BF16 activations [batch][D][H][W][C] (C innermost, a multiple of 16).
// Convolutions are 3x3x3, stride 1, zero padding, computed as implicit GEMMs
// on the BF16 tensor cores with FP32 accumulation (mma.sync m16n8k16,
// operands fetched from shared memory with ldmatrix).
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace sg {

using bf16 = __nv_bfloat16;

constexpr int TD = 2, TH = 8, TW = 8;                  // output brick of one CTA (128 voxels)
constexpr int HD = TD + 2, HH = TH + 2, HW = TW + 2;   // brick plus the 1-voxel halo
constexpr int HV = HD * HH * HW;                       // 400 halo voxels
constexpr int NTHR = 256;                              // 8 warps x 16 voxels
constexpr int WG_ROWS = 128;                           // voxels per weight-gradient tile

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// 16-byte asynchronous global->shared copy; bytes = 0 fills zeros
__device__ __forceinline__ void cp_async16(void* dst, const void* src, int bytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(smem_u32(dst)), "l"(src), "r"(bytes));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N> __device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N));
}

__device__ __forceinline__ void ldsm_x4(uint32_t r[4], const void* p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(smem_u32(p)));
}
__device__ __forceinline__ void ldsm_x4_t(uint32_t r[4], const void* p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(smem_u32(p)));
}

// D += A(16x16, row) * B(16x8, col), BF16 inputs, FP32 accumulators
__device__ __forceinline__ void mma_bf16(float d[4], const uint32_t a[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ float leaky(float v, float s) { return v > 0.f ? v : v * s; }

// Input-gradient epilogue fused with the leaky ReLU's derivative (mode 3):
// for 16 consecutive channels at element offset o, g = v * act'(y) with y
// the activation's output, dz = BF16(g), dskip += g -- the same operations,
// in the same order, as storing v in FP32 and running the activation-
// gradient kernel on it.
__device__ __forceinline__ void act_grad16(const float v[16], const bf16* yact, bf16* dz, float* dskip, size_t o,
                                           float slope) {
  const uint4* yp = (const uint4*)(yact + o);
  const uint4 q0 = yp[0], q1 = yp[1];
  const bf16* e0 = (const bf16*)&q0;
  const bf16* e1 = (const bf16*)&q1;
  float g[16];
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    g[j] = v[j] * (__bfloat162float(e0[j]) > 0.f ? 1.f : slope);
    g[8 + j] = v[8 + j] * (__bfloat162float(e1[j]) > 0.f ? 1.f : slope);
  }
  uint4 o0, o1;
  bf16* f0 = (bf16*)&o0;
  bf16* f1 = (bf16*)&o1;
#pragma unroll
  for (int j = 0; j < 8; ++j) { f0[j] = __float2bfloat16_rn(g[j]); f1[j] = __float2bfloat16_rn(g[8 + j]); }
  uint4* dp = (uint4*)(dz + o);
  dp[0] = o0;
  dp[1] = o1;
  if (dskip) {
    float4* sp = (float4*)(dskip + o);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      float4 t = sp[q];
      t.x += g[4 * q]; t.y += g[4 * q + 1]; t.z += g[4 * q + 2]; t.w += g[4 * q + 3];
      sp[q] = t;
    }
  }
}

}  // namespace sg
