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

// One transpose-reduction round over the warp: lanes with bit `O` set keep the upper
// half of x[0..S), the others the lower half; each adds the half its partner lane O
// away kept for it.  After the rounds O = 16, 8, 4, 2, 1 lane l holds column l.
template <int S, int O>
__device__ __forceinline__ void stats_round(float (&x)[16], float (&y)[16], int lane) {
    const bool up = (lane & O) != 0;
#pragma unroll
    for (int i = 0; i < S / 2; i++) {
        const float kx = up ? x[i + S / 2] : x[i], sx = up ? x[i] : x[i + S / 2];
        const float ky = up ? y[i + S / 2] : y[i], sy = up ? y[i] : y[i + S / 2];
        x[i] = kx + __shfl_xor_sync(0xFFFFFFFFu, sx, O);
        y[i] = ky + __shfl_xor_sync(0xFFFFFFFFu, sy, O);
    }
}

// Batch statistics of 32 accumulator columns of the warp's 32 rows (one row per
// lane): z = acc * scale + shift (FP32, before ReLU and rounding; 0 for rows outside
// the output), summed over the 32 rows.  Lane l returns the sum and the sum of
// squares of column l.
__device__ __forceinline__ void stats_cols32(const uint32_t (&v)[32], const float *__restrict__ sc,
                                             const float *__restrict__ sh, bool valid, float &sum, float &sq) {
    const int lane = threadIdx.x & 31;
    float x[16], y[16];
    const bool up = (lane & 16) != 0;
#pragma unroll
    for (int i = 0; i < 16; i++) {
        const float za = valid ? fmaf(__uint_as_float(v[i]), sc[i], sh[i]) : 0.0f;
        const float zb = valid ? fmaf(__uint_as_float(v[i + 16]), sc[i + 16], sh[i + 16]) : 0.0f;
        const float kz = up ? zb : za, sz = up ? za : zb;
        x[i] = kz + __shfl_xor_sync(0xFFFFFFFFu, sz, 16);
        y[i] = kz * kz + __shfl_xor_sync(0xFFFFFFFFu, sz * sz, 16);
    }
    stats_round<16, 8>(x, y, lane);
    stats_round<8, 4>(x, y, lane);
    stats_round<4, 2>(x, y, lane);
    stats_round<2, 1>(x, y, lane);
    sum = x[0];
    sq = y[0];
}

}  // namespace tc
