// Preparation kernels of the tensor-core forms: weight packing into the
// K-major operand the tcgen05 kernels load with TMA, the FP64 batch-norm fold,
// activation casts, and the fixed-order reduction of weight-gradient splits.
#include <cuda_bf16.h>

#include "cg_common.cuh"
#include "prep.h"

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

int grid_for(long long n) {
    long long g = (n + 255) / 256;
    return (int) (g > 152 * 32 ? 152 * 32 : (g < 1 ? 1 : g));
}

}  // namespace

cudaError_t prep_pack_fwd(const float *w, int nchw, int C, int kh, int kw, int kn, int Cp, int Kpad, void *out,
                          cudaStream_t st) {
    if (nchw) {
        pack_fwd_kernel<<<grid_for((long long) kn * Kpad), 256, 0, st>>>(w, nchw, C, kh, kw, kn, Cp, Kpad,
                                                                        (bf16 *) out);
        return cudaGetLastError();
    }
    const int khw = kh * kw;
    dim3 grid((Cp + 31) / 32, (kn + 31) / 32, khw), block(32, 8);
    pack_fwd_tiled_kernel<<<grid, block, 0, st>>>(w, C, khw, kn, Cp, Kpad, (bf16 *) out);
    if (Kpad > khw * Cp)
        pack_fwd_tail_kernel<<<grid_for((long long) kn * (Kpad - khw * Cp)), 256, 0, st>>>(kn, khw * Cp, Kpad,
                                                                                          (bf16 *) out);
    return cudaGetLastError();
}

cudaError_t prep_pack_dgrad(const float *w, int nchw, int C, int kh, int kw, int kn, int knp,
                            const PackDgradInfo &info, void *out, cudaStream_t st) {
    pack_dgrad_kernel<<<grid_for((long long) C * info.Ktot), 256, 0, st>>>(w, nchw, C, kh, kw, kn, knp, info,
                                                                          (bf16 *) out);
    return cudaGetLastError();
}

cudaError_t prep_fold(int kn, const float *bias, const float *mean, const float *inv_std, const float *gamma,
                      const float *beta, float *scale, float *shift, cudaStream_t st) {
    fold_kernel<<<(kn + 127) / 128, 128, 0, st>>>(kn, bias, mean, inv_std, gamma, beta, scale, shift);
    return cudaGetLastError();
}

cudaError_t prep_to_bf16_nhwc(const float *in, int nchw, int B, int C, int H, int W, int Cp, void *out,
                              cudaStream_t st) {
    to_bf16_nhwc_kernel<<<grid_for((long long) B * H * W * Cp), 256, 0, st>>>(in, nchw, B, C, H, W, Cp, (bf16 *) out);
    return cudaGetLastError();
}
