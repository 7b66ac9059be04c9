// Fused epilogue arithmetic of the tensor-core kernels: one thread turns 64
// FP32 accumulators of its output row into 32 packed BF16 pairs,
//   y = relu?(acc * scale + shift),
// with two-wide FMAs (fma.rn.f32x2: each lane rounds exactly as fmaf) and the
// ReLU folded into the BF16 conversion (cvt.rn.relu.bf16x2.f32).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace tc {

template <bool RELU>
__device__ __forceinline__ uint32_t cvt_bf16x2(float lo, float hi) {
    uint32_t d;
    if (RELU)
        asm("cvt.rn.relu.bf16x2.f32 %0, %1, %2;" : "=r"(d) : "f"(hi), "f"(lo));
    else
        asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(d) : "f"(hi), "f"(lo));
    return d;
}

// v0: columns 0-31, v1: columns 32-63 (tcgen05.ld 32x32b.x32 results); sc/sh:
// the 64 columns' scale and shift, 16-byte aligned (shared memory).
template <bool RELU>
__device__ __forceinline__ void epi_bf16_64(const uint32_t (&v0)[32], const uint32_t (&v1)[32],
                                            const float *__restrict__ sc, const float *__restrict__ sh,
                                            uint32_t (&pk)[32]) {
    const float4 *s4 = reinterpret_cast<const float4 *>(sc);
    const float4 *t4 = reinterpret_cast<const float4 *>(sh);
#pragma unroll
    for (int q = 0; q < 16; q++) {
        const float4 s = s4[q], t = t4[q];
        const int j = 4 * q;
        float2 a = make_float2(__uint_as_float(j < 32 ? v0[j] : v1[j - 32]),
                               __uint_as_float(j < 32 ? v0[j + 1] : v1[j - 31]));
        float2 b = make_float2(__uint_as_float(j < 32 ? v0[j + 2] : v1[j - 30]),
                               __uint_as_float(j < 32 ? v0[j + 3] : v1[j - 29]));
        a = __ffma2_rn(a, make_float2(s.x, s.y), make_float2(t.x, t.y));
        b = __ffma2_rn(b, make_float2(s.z, s.w), make_float2(t.z, t.w));
        pk[2 * q] = cvt_bf16x2<RELU>(a.x, a.y);
        pk[2 * q + 1] = cvt_bf16x2<RELU>(b.x, b.y);
    }
}

}  // namespace tc
