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
    __shared__ float tile[32][33];
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
            // the tiled transpose of pack_fwd_tiled_kernel for one (ci tile, co tile), all taps
            const int nci = (J.Cp + 31) / 32;
            const int ci0 = (lb % nci) * 32, co0 = (lb / nci) * 32;
            const int tx = t & 31, ty = t >> 5, khw = J.kh * J.kw;
            bf16 *out = (bf16 *) J.out;
            for (int tap = 0; tap < khw; tap++) {
                for (int i = ty; i < 32; i += 8) {
                    const int ci = ci0 + i, co = co0 + tx;
                    tile[i][tx] = (ci < J.C && co < J.kn) ? J.w[((size_t) ci * khw + tap) * J.kn + co] : 0.0f;
                }
                __syncthreads();
                for (int j = ty; j < 32; j += 8) {
                    const int co = co0 + j, ci = ci0 + tx;
                    if (co < J.kn && ci < J.Cp)
                        out[(size_t) co * J.Kpad + (size_t) tap * J.Cp + ci] = __float2bfloat16_rn(tile[tx][j]);
                }
                __syncthreads();
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
    return cg_launch_pdl(prep_group_kernel, dim3(nblocks), dim3(256), sizeof(int) * njobs, st, jobs, b0, njobs);
}
