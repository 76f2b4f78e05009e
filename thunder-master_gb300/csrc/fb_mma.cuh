// fb_mma.cuh -- warp-level BF16 tensor-core tiles (mma.sync m16n8k16, FP32
// accumulation) used by the MLP-3c surrogate's training GEMMs.
//
// Fragment layout of mma.m16n8k16 with BF16 operands (PTX ISA, "Matrix
// fragments for mma.m16n8k16"), g = lane / 4, t = lane % 4:
//   A (16 x 16, row major), 4 registers of two BF16 each:
//     a0 = A[g][2t..2t+1]    a1 = A[g+8][2t..2t+1]
//     a2 = A[g][2t+8..+9]    a3 = A[g+8][2t+8..+9]
//   B (16 x 8, column major), 2 registers: b0 = B[2t..2t+1][g], b1 = B[2t+8..+9][g]
//   C (16 x 8, FP32): c0 = C[g][2t], c1 = C[g][2t+1], c2 = C[g+8][2t], c3 = C[g+8][2t+1]
// The C fragments of two neighboring n-tiles are, register for register, the
// A fragment of one k-tile of the next product, so layers chain in registers.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cstdint>

namespace fb {

__device__ __forceinline__ void mma_bf16(float c[4], const uint32_t a[4], const uint32_t b[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// two floats -> packed BF16 pair (round to nearest even), first in the low half
__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<uint32_t *>(&v);
}

__device__ __forceinline__ float silu(float z) { return z / (1.0f + __expf(-z)); }
__device__ __forceinline__ float sigmoid(float z) { return 1.0f / (1.0f + __expf(-z)); }
// sigmoid(z) = (1 + tanh(z / 2)) / 2 with the hardware tanh approximation
// (one special-function op instead of two; its ~2^-11 relative error is
// below the BF16 rounding the activations get next)
__device__ __forceinline__ float sigmoid_fast(float z) {
  float t;
  asm("tanh.approx.f32 %0, %1;" : "=f"(t) : "f"(0.5f * z));
  return fmaf(0.5f, t, 0.5f);
}
// d silu / dz = s (1 + z (1 - s)), s = sigmoid(z)
__device__ __forceinline__ float dsilu(float z) {
  float s = 1.0f / (1.0f + __expf(-z));
  return s * (1.0f + z * (1.0f - s));
}

}  // namespace fb
