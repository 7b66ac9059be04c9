// Preparation kernels of the tensor-core forms: weight packing into the
// K-major operand the tcgen05 kernels load with TMA, the FP64 batch-norm fold,
// activation casts, and the fixed-order reduction of weight-gradient splits.
#include <cuda_bf16.h>
#include <cuda_fp8.h>

#include "cg_common.cuh"
#include "prep.h"
#include "tc_ptx.cuh"

namespace {

using bf16 = __nv_bfloat16;

// Weight element (ci, kx, ky, co) of the reference layouts:
//   NHWC API: [c][kh][kw][kn]  (src/convGemm.c:66, ld = kn)
//   NCHW API: [kn][c][kh][kw]  (src/convGemm.c:117, ld = K)
__device__ __forceinline__ float wref(const float *w, int nchw, int C, int kh, int kw, int kn, int ci, int kx, int ky,
                                      int co) {
    const size_t k = ((size_t) ci * kh + kx) * kw + ky;
    return nchw ? w[(size_t) co * ((size_t) C * kh * kw) + k] : w[k * kn + co];
}

// out[co][k], k = (kx*kw + ky)*Cp + ci, zero for padded ci and k.  One 32x32 tile of
// (ci, co) at one tap per block: reads along co (contiguous in the NHWC-API layout),
// writes along ci (contiguous in the packed row) through shared memory.
__global__ void pack_fwd_tiled_kernel(const float *__restrict__ w, int C, int khw, int kn, int Cp, int Kpad,
                                      bf16 *__restrict__ out) {
    __shared__ float tile[32][33];
    const int tap = blockIdx.z, ci0 = blockIdx.x * 32, co0 = blockIdx.y * 32;
    const int tx = threadIdx.x, ty = threadIdx.y;
    for (int i = ty; i < 32; i += 8) {
        const int ci = ci0 + i, co = co0 + tx;
        tile[i][tx] = (ci < C && co < kn) ? w[((size_t) ci * khw + tap) * kn + co] : 0.0f;
    }
    __syncthreads();
    for (int j = ty; j < 32; j += 8) {
        const int co = co0 + j, ci = ci0 + tx;
        if (co < kn && ci < Cp) out[(size_t) co * Kpad + (size_t) tap * Cp + ci] = __float2bfloat16_rn(tile[tx][j]);
    }
}

// zero of the K padding columns [khw*Cp, Kpad) of every row
__global__ void pack_fwd_tail_kernel(int kn, int Kbeg, int Kpad, bf16 *__restrict__ out) {
    const int width = Kpad - Kbeg;
    const long long total = (long long) kn * width;
    for (long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < total;
         i += (long long) gridDim.x * blockDim.x)
        out[(i / width) * Kpad + Kbeg + i % width] = __float2bfloat16_rn(0.0f);
}

__global__ void pack_fwd_kernel(const float *__restrict__ w, int nchw, int C, int kh, int kw, int kn, int Cp,
                                int Kpad, bf16 *__restrict__ out) {
    const long long total = (long long) kn * Kpad;
    for (long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < total;
         i += (long long) gridDim.x * blockDim.x) {
        const int co = (int) (i / Kpad), k = (int) (i % Kpad);
        const int tap = k / Cp, ci = k % Cp;
        float v = 0.0f;
        if (tap < kh * kw && ci < C) v = wref(w, nchw, C, kh, kw, kn, ci, tap / kw, tap % kw, co);
        out[i] = __float2bfloat16_rn(v);
    }
}

// Input-gradient operand: out[ci][kbeg_c + t*knp + co] = W(ci, kx_t, ky_t, co) for each class c.
__global__ void pack_dgrad_kernel(const float *__restrict__ w, int nchw, int C, int kh, int kw, int kn, int knp,
                                  const PackDgradInfo info, bf16 *__restrict__ out) {
    const long long total = (long long) C * info.Ktot;
    for (long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < total;
         i += (long long) gridDim.x * blockDim.x) {
        const int ci = (int) (i / info.Ktot), col = (int) (i % info.Ktot);
        int c = 0;
        while (c + 1 < info.ncls && col >= info.kbeg[c + 1]) c++;
        const int k = col - info.kbeg[c];
        const int t = k / knp, co = k % knp;
        float v = 0.0f;
        if (t < info.ntaps[c] && co < kn) v = wref(w, nchw, C, kh, kw, kn, ci, info.kx[c][t], info.ky[c][t], co);
        out[i] = __float2bfloat16_rn(v);
    }
}

// scale = gamma*inv_std, shift = beta + (bias - mean)*scale, in double (the one place
// besides the oracle where FP64 runs on the GPU).
__global__ void fold_kernel(int kn, const float *bias, const float *mean, const float *inv_std, const float *gamma,
                            const float *beta, float *scale, float *shift) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= kn) return;
    double s = 1.0, t = bias ? (double) bias[n] : 0.0;
    if (mean) {
        s = (double) gamma[n] * (double) inv_std[n];
        t = (double) beta[n] + (t - (double) mean[n]) * s;
    }
    scale[n] = (float) s;
    shift[n] = (float) t;
}

// FP32 NHWC or NCHW [B][C][H][W] -> BF16 NHWC [B][H][W][Cp] (padding channels zero).
__global__ void to_bf16_nhwc_kernel(const float *__restrict__ in, int nchw, int B, int C, int H, int W, int Cp,
                                    bf16 *__restrict__ out) {
    const long long total = (long long) B * H * W * Cp;
    for (long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < total;
         i += (long long) gridDim.x * blockDim.x) {
        const int c = (int) (i % Cp);
        const long long pix = i / Cp;
        float v = 0.0f;
        if (c < C) {
            if (nchw) {
                const long long hw = (long long) H * W;
                const long long b = pix / hw, q = pix % hw;
                v = in[(b * C + c) * hw + q];
            } else {
                v = in[pix * C + c];
            }
        }
        out[i] = __float2bfloat16_rn(v);
    }
}

// ------------------------------------------------------ FP8 and 3xBF16 forms
constexpr float E4M3_MAX = 448.0f;

__device__ __forceinline__ uint8_t to_e4m3(float v) {
    return (uint8_t) __nv_cvt_float_to_fp8(v, __NV_SATFINITE, __NV_E4M3);
}

// amax (as the bit pattern of a non-negative float, so atomicMax on unsigned orders it)
__global__ void amax_kernel(const void *__restrict__ in, int in_bf16, long long n, unsigned *amax_bits) {
    float m = 0.0f;
    for (long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < n; i += (long long) gridDim.x * blockDim.x) {
        const float v = in_bf16 ? __bfloat162float(((const bf16 *) in)[i]) : ((const float *) in)[i];
        m = fmaxf(m, fabsf(v));
    }
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(amax_bits, __float_as_uint(m));
}

// per-tensor scale = amax / 448 (1 for an all-zero tensor); x_q = e4m3(x / scale)
__global__ void quant_e4m3_kernel(const void *__restrict__ in, int in_bf16, long long n, const unsigned *amax_bits,
                                  uint8_t *__restrict__ out, float *scale_out) {
    const float amax = __uint_as_float(*amax_bits);
    const float sc = amax > 0.0f ? amax / E4M3_MAX : 1.0f;
    const float inv = 1.0f / sc;
    if (blockIdx.x == 0 && threadIdx.x == 0) *scale_out = sc;
    for (long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < n; i += (long long) gridDim.x * blockDim.x) {
        const float v = in_bf16 ? __bfloat162float(((const bf16 *) in)[i]) : ((const float *) in)[i];
        out[i] = to_e4m3(v * inv);
    }
}

// per-output-channel weight scale (NHWC-API weights [K][kn]: threads along co, loop over K)
__global__ void wscale_kernel(const float *__restrict__ w, int nchw, int K, int kn, float *wscale) {
    const int co = blockIdx.x * blockDim.x + threadIdx.x;
    if (co >= kn) return;
    float m = 0.0f;
    for (int k = 0; k < K; k++) m = fmaxf(m, fabsf(nchw ? w[(size_t) co * K + k] : w[(size_t) k * kn + co]));
    wscale[co] = m > 0.0f ? m / E4M3_MAX : 1.0f;
}

// E4M3 operand [co][tap*Cp + ci] = w / wscale[co]
__global__ void pack_fp8_kernel(const float *__restrict__ w, int nchw, int C, int kh, int kw, int kn, int Cp, int Kpad,
                                const float *__restrict__ wscale, uint8_t *__restrict__ out) {
    const long long total = (long long) kn * Kpad;
    for (long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < total;
         i += (long long) gridDim.x * blockDim.x) {
        const int co = (int) (i / Kpad), k = (int) (i % Kpad);
        const int tap = k / Cp, ci = k % Cp;
        float v = 0.0f;
        if (tap < kh * kw && ci < C) v = wref(w, nchw, C, kh, kw, kn, ci, tap / kw, tap % kw, co) / wscale[co];
        out[i] = to_e4m3(v);
    }
}

// scale' = scale * wscale * xscale (the two quantisation scales folded into the epilogue)
__global__ void fp8_scales_kernel(int kn, const float *scale, const float *shift, const float *wscale,
                                  const float *xscale, float *out_scale, float *out_shift) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= kn) return;
    out_scale[n] = (scale ? scale[n] : 1.0f) * wscale[n] * xscale[0];
    out_shift[n] = shift ? shift[n] : 0.0f;
}

// x = hi + lo with hi = bf16(x), lo = bf16(x - hi)
__global__ void split_kernel(const float *__restrict__ in, long long n, bf16 *__restrict__ hi, bf16 *__restrict__ lo) {
    for (long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < n; i += (long long) gridDim.x * blockDim.x) {
        const float v = in[i];
        const bf16 h = __float2bfloat16_rn(v);
        hi[i] = h;
        lo[i] = __float2bfloat16_rn(v - __bfloat162float(h));
    }
}

__global__ void pack_split_kernel(const float *__restrict__ w, int nchw, int C, int kh, int kw, int kn, int Cp, int Kpad,
                                  bf16 *__restrict__ hi, bf16 *__restrict__ lo) {
    const long long total = (long long) kn * Kpad;
    for (long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < total;
         i += (long long) gridDim.x * blockDim.x) {
        const int co = (int) (i / Kpad), k = (int) (i % Kpad);
        const int tap = k / Cp, ci = k % Cp;
        float v = 0.0f;
        if (tap < kh * kw && ci < C) v = wref(w, nchw, C, kh, kw, kn, ci, tap / kw, tap % kw, co);
        const bf16 h = __float2bfloat16_rn(v);
        hi[i] = h;
        lo[i] = __float2bfloat16_rn(v - __bfloat162float(h));
    }
}

// Grouped preparation: every block finds its job by binary search over the jobs'
// first blocks and runs that job's body for its block (256 threads).
// The jobs' first blocks (b0, njobs ints) are staged in shared memory first, so the
// search costs one global round trip.
__global__ void __launch_bounds__(256) prep_group_kernel(const PrepJob *__restrict__ jobs, const int *__restrict__ b0,
                                                         int njobs) {
    __shared__ float tile[64][65];
    extern __shared__ int s_b0[];
    tc::pdl_wait();
    tc::pdl_trigger();
    for (int i = threadIdx.x; i < njobs; i += blockDim.x) s_b0[i] = __ldg(b0 + i);
    __syncthreads();
    int lo = 0, hi = njobs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (s_b0[mid] <= (int) blockIdx.x) lo = mid;
        else hi = mid - 1;
    }
    const PrepJob &J = jobs[lo];
    const int lb = blockIdx.x - J.block0;
    const int t = threadIdx.x;
    switch (J.type) {
        case PREP_FOLD: {
            const int n = lb * 256 + t;
            if (n >= J.kn) return;
            double sc = 1.0, sh = J.bias ? (double) J.bias[n] : 0.0;
            if (J.mean) {
                sc = (double) J.gamma[n] * (double) J.inv_std[n];
                sh = (double) J.beta[n] + (sh - (double) J.mean[n]) * sc;
            }
            J.scale[n] = (float) sc;
            J.shift[n] = (float) sh;
            return;
        }
        case PREP_FWD_TILED: {
            // NHWC-API weights [ci][tap][co] -> out[co][tap*Cp + ci]: one block per (tap, 64 ci x 64 co
            // tile); four independent 16-byte loads per thread along co, a padded shared-memory
            // transpose, 8-byte stores of four BF16 along ci
            const int nci = (J.Cp + 63) / 64, nco = (J.kn + 63) / 64, khw = J.kh * J.kw;
            const int tap = lb / (nci * nco), rem = lb % (nci * nco);
            const int ci0 = (rem % nci) * 64, co0 = (rem / nci) * 64;
            const int cq = (t & 15) * 4, r0 = t >> 4;   // 4 co per thread; rows r0 + 16 i
            const bool vec_in = ((J.kn & 3) == 0) && (((uintptr_t) J.w & 15) == 0);
            const bool vec_out = ((J.Kpad & 3) == 0) && ((J.Cp & 3) == 0) && (((uintptr_t) J.out & 7) == 0);
            float4 v[4];
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const int ci = ci0 + r0 + 16 * i, co = co0 + cq;
                const float *src = J.w + ((size_t) ci * khw + tap) * J.kn + co;
                if (ci < J.C && co + 4 <= J.kn && vec_in) {
                    v[i] = __ldg(reinterpret_cast<const float4 *>(src));
                } else {
                    float e[4];
#pragma unroll
                    for (int q = 0; q < 4; q++) e[q] = (ci < J.C && co + q < J.kn) ? __ldg(src + q) : 0.0f;
                    v[i] = make_float4(e[0], e[1], e[2], e[3]);
                }
            }
#pragma unroll
            for (int i = 0; i < 4; i++) {
                float *d = &tile[r0 + 16 * i][cq];
                d[0] = v[i].x;
                d[1] = v[i].y;
                d[2] = v[i].z;
                d[3] = v[i].w;
            }
            __syncthreads();
            bf16 *out = (bf16 *) J.out;
            const int cw = (t & 15) * 4, o0 = t >> 4;   // 4 ci per thread; co rows o0 + 16 j
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const int co = co0 + o0 + 16 * j, ci = ci0 + cw;
                if (co >= J.kn || ci >= J.Cp) continue;
                bf16 *dst = out + (size_t) co * J.Kpad + (size_t) tap * J.Cp + ci;
                const int cc = o0 + 16 * j;
                if (ci + 4 <= J.Cp && vec_out) {
                    __nv_bfloat162 lo = __floats2bfloat162_rn(tile[cw][cc], tile[cw + 1][cc]);
                    __nv_bfloat162 hi = __floats2bfloat162_rn(tile[cw + 2][cc], tile[cw + 3][cc]);
                    uint2 u;
                    u.x = *reinterpret_cast<uint32_t *>(&lo);
                    u.y = *reinterpret_cast<uint32_t *>(&hi);
                    *reinterpret_cast<uint2 *>(dst) = u;
                } else {
                    for (int q = 0; q < 4 && ci + q < J.Cp; q++) dst[q] = __float2bfloat16_rn(tile[cw + q][cc]);
                }
            }
            return;
        }
        case PREP_FWD_ELEM: {
            // block = (row co, 256 columns of K): 32-bit index math, no division by the row length
            const int nch = (J.Kpad + 255) / 256;
            const int co = lb / nch, k = (lb % nch) * 256 + t;
            if (k >= J.Kpad) return;
            const int tap = k / J.Cp, ci = k - tap * J.Cp;
            float v = 0.0f;
            if (tap < J.kh * J.kw && ci < J.C) v = wref(J.w, J.nchw, J.C, J.kh, J.kw, J.kn, ci, tap / J.kw, tap % J.kw, co);
            ((bf16 *) J.out)[(size_t) co * J.Kpad + k] = __float2bfloat16_rn(v);
            return;
        }
        case PREP_FWD_TAIL: {
            const int kbeg = J.kh * J.kw * J.Cp, width = J.Kpad - kbeg;
            const int i = lb * 256 + t;
            if (i >= J.kn * width) return;
            const int co = i / width;
            ((bf16 *) J.out)[(size_t) co * J.Kpad + kbeg + (i - co * width)] = __float2bfloat16_rn(0.0f);
            return;
        }
        default: {   // PREP_DGRAD: block = (4 input channels, one stride-phase class): the class's
                     // K segment of those rows, taps x knp output channels and the K padding after them
            const int c = lb % J.info.ncls, ci0 = (lb / J.info.ncls) * 4;
            const int beg = J.info.kbeg[c], end = c + 1 < J.info.ncls ? J.info.kbeg[c + 1] : J.info.Ktot;
            const int nt = J.info.ntaps[c];
            if (!J.nchw && (J.kn & 3) == 0 && (J.knp & 3) == 0 && ((beg | end | J.info.Ktot) & 3) == 0 &&
                ((uintptr_t) J.w & 15) == 0 && ((uintptr_t) J.out & 7) == 0) {
                // NHWC-API weights: four consecutive output channels per 16-byte load and 8-byte
                // store, unrolled for several loads in flight
                const int nq = (end - beg) >> 2;
                for (int r = 0; r < 4; r++) {
                    const int ci = ci0 + r;
                    if (ci >= J.C) break;
                    bf16 *row = (bf16 *) J.out + (size_t) ci * J.info.Ktot + beg;
#pragma unroll 4
                    for (int q = t; q < nq; q += 256) {
                        const int idx = q * 4;
                        const int g = (int) J.dknp.div((uint32_t) idx), co = idx - g * J.knp;
                        float4 v = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                        if (g < nt && co < J.kn) {
                            const int tap = J.info.kx[c][g] * J.kw + J.info.ky[c][g];
                            v = __ldg(reinterpret_cast<const float4 *>(J.w + ((size_t) ci * J.kh * J.kw + tap) * J.kn + co));
                        }
                        __nv_bfloat162 lo = __floats2bfloat162_rn(v.x, v.y), hi = __floats2bfloat162_rn(v.z, v.w);
                        uint2 u;
                        u.x = *reinterpret_cast<uint32_t *>(&lo);
                        u.y = *reinterpret_cast<uint32_t *>(&hi);
                        *reinterpret_cast<uint2 *>(row + idx) = u;
                    }
                }
                return;
            }
            for (int r = 0; r < 4; r++) {
                const int ci = ci0 + r;
                if (ci >= J.C) break;
                bf16 *row = (bf16 *) J.out + (size_t) ci * J.info.Ktot + beg;
                for (int idx = t; idx < end - beg; idx += 256) {
                    const int g = (int) J.dknp.div((uint32_t) idx), co = idx - g * J.knp;
                    float v = 0.0f;
                    if (g < nt && co < J.kn) v = wref(J.w, J.nchw, J.C, J.kh, J.kw, J.kn, ci, J.info.kx[c][g], J.info.ky[c][g], co);
                    row[idx] = __float2bfloat16_rn(v);
                }
            }
        }
    }
}

int grid_for(long long n) {
    long long g = (n + 255) / 256;
    return (int) (g > 152 * 32 ? 152 * 32 : (g < 1 ? 1 : g));
}

}  // namespace

cudaError_t prep_pack_fwd(const float *w, int nchw, int C, int kh, int kw, int kn, int Cp, int Kpad, void *out,
                          cudaStream_t st) {
    if (nchw) {
        pack_fwd_kernel<<<grid_for((long long) kn * Kpad), 256, 0, st>>>(w, nchw, C, kh, kw, kn, Cp, Kpad,
                                                                        (bf16 *) out); cg_note_launch();
        return cudaGetLastError();
    }
    const int khw = kh * kw;
    dim3 grid((Cp + 31) / 32, (kn + 31) / 32, khw), block(32, 8);
    pack_fwd_tiled_kernel<<<grid, block, 0, st>>>(w, C, khw, kn, Cp, Kpad, (bf16 *) out); cg_note_launch();
    if (Kpad > khw * Cp)
        pack_fwd_tail_kernel<<<grid_for((long long) kn * (Kpad - khw * Cp)), 256, 0, st>>>(kn, khw * Cp, Kpad,
                                                                                          (bf16 *) out); cg_note_launch();
    return cudaGetLastError();
}

cudaError_t prep_pack_dgrad(const float *w, int nchw, int C, int kh, int kw, int kn, int knp,
                            const PackDgradInfo &info, void *out, cudaStream_t st) {
    pack_dgrad_kernel<<<grid_for((long long) C * info.Ktot), 256, 0, st>>>(w, nchw, C, kh, kw, kn, knp, info,
                                                                          (bf16 *) out); cg_note_launch();
    return cudaGetLastError();
}

cudaError_t prep_fold(int kn, const float *bias, const float *mean, const float *inv_std, const float *gamma,
                      const float *beta, float *scale, float *shift, cudaStream_t st) {
    fold_kernel<<<(kn + 127) / 128, 128, 0, st>>>(kn, bias, mean, inv_std, gamma, beta, scale, shift); cg_note_launch();
    return cudaGetLastError();
}

cudaError_t prep_to_bf16_nhwc(const float *in, int nchw, int B, int C, int H, int W, int Cp, void *out,
                              cudaStream_t st) {
    to_bf16_nhwc_kernel<<<grid_for((long long) B * H * W * Cp), 256, 0, st>>>(in, nchw, B, C, H, W, Cp, (bf16 *) out); cg_note_launch();
    return cudaGetLastError();
}

cudaError_t prep_fp8_quantize(long long n, int in_bf16, const void *in, void *out, float *scale, unsigned *amax_tmp,
                              cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(amax_tmp, 0, sizeof(unsigned), st);
    if (e != cudaSuccess) return e;
    amax_kernel<<<grid_for(n), 256, 0, st>>>(in, in_bf16, n, amax_tmp); cg_note_launch();
    quant_e4m3_kernel<<<grid_for(n), 256, 0, st>>>(in, in_bf16, n, amax_tmp, (uint8_t *) out, scale); cg_note_launch();
    return cudaGetLastError();
}

cudaError_t prep_pack_fp8(const float *w, int nchw, int C, int kh, int kw, int kn, int Cp, int Kpad, void *out,
                          float *wscale, cudaStream_t st) {
    wscale_kernel<<<(kn + 127) / 128, 128, 0, st>>>(w, nchw, C * kh * kw, kn, wscale); cg_note_launch();
    pack_fp8_kernel<<<grid_for((long long) kn * Kpad), 256, 0, st>>>(w, nchw, C, kh, kw, kn, Cp, Kpad, wscale,
                                                                    (uint8_t *) out); cg_note_launch();
    return cudaGetLastError();
}

cudaError_t prep_fp8_scales(int kn, const float *scale, const float *shift, const float *wscale, const float *xscale,
                            float *out_scale, float *out_shift, cudaStream_t st) {
    fp8_scales_kernel<<<(kn + 127) / 128, 128, 0, st>>>(kn, scale, shift, wscale, xscale, out_scale, out_shift); cg_note_launch();
    return cudaGetLastError();
}

cudaError_t prep_split(long long n, const float *in, void *hi, void *lo, cudaStream_t st) {
    split_kernel<<<grid_for(n), 256, 0, st>>>(in, n, (bf16 *) hi, (bf16 *) lo); cg_note_launch();
    return cudaGetLastError();
}

cudaError_t prep_pack_split(const float *w, int nchw, int C, int kh, int kw, int kn, int Cp, int Kpad, void *hi,
                            void *lo, cudaStream_t st) {
    pack_split_kernel<<<grid_for((long long) kn * Kpad), 256, 0, st>>>(w, nchw, C, kh, kw, kn, Cp, Kpad, (bf16 *) hi,
                                                                      (bf16 *) lo); cg_note_launch();
    return cudaGetLastError();
}

cudaError_t prep_group_launch(const PrepJob *jobs, int njobs, int nblocks, cudaStream_t st) {
    const int *b0 = (const int *) (jobs + njobs);
    static bool attr = false;   // up to 12288 job offsets (48 KB) beside the 16.6 KB transpose tile
    if (!attr) {
        if (cudaError_t e = cudaFuncSetAttribute(prep_group_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 12288 * (int) sizeof(int)))
            return e;
        attr = true;
    }
    return cg_launch_pdl(prep_group_kernel, dim3(nblocks), dim3(256), sizeof(int) * njobs, st, jobs, b0, njobs);
}
