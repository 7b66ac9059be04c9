// Training-mode batch normalisation around the BF16 forward: the convolution's
// epilogue writes, per group of 32 output pixels, the FP32 sum and sum of squares of
// z = acc * scale + shift for each channel (tc_conv.cu / tc_stem.cu); this file
//   * reduces those partials in a fixed order into FP64 per-channel sums (bit-for-bit
//     reproducible: no atomics),
//   * folds the batch mean / biased variance with gamma / beta into the per-channel
//     scale / shift of the normalisation,
//   * applies y = relu?(z * scale + shift) to the BF16 NHWC output.
// The reference's epilogue is inference-style batch norm only (running statistics,
// src/im2row_nhwc.c:279-280); these are the training-step kernels either side of it.
#include <cstring>

#include <cuda_bf16.h>

#include "../../include/convgemm_gpu.h"
#include "cg_common.cuh"
#include "cg_internal.h"
#include "tc_host.h"

namespace {

constexpr int BN_CHUNK = 256;   // statistics groups per block of the first pass

// Pass 1: block (x = 32 channels, y = a chunk of BN_CHUNK groups) sums its groups for
// its channels in FP64, the 8 thread rows strided over the chunk, then in a fixed
// order across the rows.  part: [ngroups][2][kn] FP32; out: [nchunks][2][kn] FP64.
__global__ void __launch_bounds__(256) bn_stats_pass1(const float *__restrict__ part, int ngroups, int kn,
                                                      double *__restrict__ out) {
    __shared__ double red[2][8][33];
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int c = blockIdx.x * 32 + tx;
    const int g0 = blockIdx.y * BN_CHUNK, g1 = min(g0 + BN_CHUNK, ngroups);
    double s = 0.0, q = 0.0;
    if (c < kn)
        for (int g = g0 + ty; g < g1; g += 8) {
            s += (double) __ldg(part + (size_t) g * 2 * kn + c);
            q += (double) __ldg(part + (size_t) g * 2 * kn + kn + c);
        }
    red[0][ty][tx] = s;
    red[1][ty][tx] = q;
    __syncthreads();
    if (ty < 2 && c < kn) {
        double a = 0.0;
        for (int r = 0; r < 8; r++) a += red[ty][r][tx];
        out[(size_t) blockIdx.y * 2 * kn + (size_t) ty * kn + c] = a;
    }
}

// Pass 2: stats[0][c] = sum, stats[1][c] = sum of squares, over the chunks in order.
__global__ void bn_stats_pass2(const double *__restrict__ chunks, int nchunks, int kn, double *__restrict__ stats) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 2 * kn) return;
    double a = 0.0;
    for (int j = 0; j < nchunks; j++) a += chunks[(size_t) j * 2 * kn + i];
    stats[i] = a;
}

// Column sums in FP32 from the chunk sums of pass 1: out[c] = sum over the chunks, in order,
// of the first statistics plane.
__global__ void colsum_pass2_f32(const double *__restrict__ chunks, int nchunks, int kn, float *__restrict__ out) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= kn) return;
    double a = 0.0;
    for (int j = 0; j < nchunks; j++) a += chunks[(size_t) j * 2 * kn + c];
    out[c] = (float) a;
}

__global__ void bn_fold_kernel(int kn, const double *__restrict__ stats, double inv_count, const float *gamma,
                               const float *beta, float eps, float *scale, float *shift, float *mean_out,
                               float *var_out) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= kn) return;
    const double mean = stats[c] * inv_count;
    double var = stats[kn + c] * inv_count - mean * mean;
    if (var < 0.0) var = 0.0;
    const double sc = (gamma ? (double) gamma[c] : 1.0) / sqrt(var + (double) eps);
    scale[c] = (float) sc;
    shift[c] = (float) ((beta ? (double) beta[c] : 0.0) - mean * sc);
    if (mean_out) mean_out[c] = (float) mean;
    if (var_out) var_out[c] = (float) var;
}

// y = relu?(z * scale + shift), BF16 NHWC [npix][kn], 8 channels per thread step.
__global__ void bn_apply_kernel(long long n8, int kn, const __nv_bfloat16 *z, const float *__restrict__ scale,
                                const float *__restrict__ shift, int relu, __nv_bfloat16 *y) {
    const int k8 = kn / 8;
    for (long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < n8;
         i += (long long) gridDim.x * blockDim.x) {
        const int c0 = (int) (i % k8) * 8;
        const uint4 u = reinterpret_cast<const uint4 *>(z)[i];   // z may be y: read before the write
        const uint32_t w[4] = {u.x, u.y, u.z, u.w};
        uint32_t o[4];
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const __nv_bfloat162 h = *reinterpret_cast<const __nv_bfloat162 *>(&w[j]);
            float a = fmaf(__bfloat162float(h.x), __ldg(scale + c0 + 2 * j), __ldg(shift + c0 + 2 * j));
            float b = fmaf(__bfloat162float(h.y), __ldg(scale + c0 + 2 * j + 1), __ldg(shift + c0 + 2 * j + 1));
            if (relu) {
                a = fmaxf(a, 0.0f);
                b = fmaxf(b, 0.0f);
            }
            const __nv_bfloat162 r = __floats2bfloat162_rn(a, b);
            o[j] = *reinterpret_cast<const uint32_t *>(&r);
        }
        reinterpret_cast<uint4 *>(y)[i] = make_uint4(o[0], o[1], o[2], o[3]);
    }
}

// statistics groups of the forward's path for this shape: the small-channel kernel
// groups per (output row, 128-pixel chunk), the general kernel per 32 output pixels
int stat_groups(const cg_shape &s, bool *stem) {
    const ConvGeom g = make_geom(s);
    *stem = tc_stem_applicable(s);
    return *stem ? tc_stem_stat_groups(s) : (int) (((long long) s.b * g.ho * g.wo + 31) / 32);
}

size_t stats_ws_bytes(const cg_shape &s) {
    bool stem;
    const long long ng = stat_groups(s, &stem);
    const long long nchunks = (ng + BN_CHUNK - 1) / BN_CHUNK;
    // FP64 chunk sums first (8-byte aligned), then the FP32 group partials
    return (size_t) (nchunks * 2 * s.kn * 8 + ng * 2 * s.kn * 4);
}

}  // namespace

size_t cg_colsum_ws_bytes(long long ngroups, int kn) {
    const long long nchunks = (ngroups + BN_CHUNK - 1) / BN_CHUNK;
    return (size_t) (nchunks * 2 * kn * 8 + ngroups * 2 * kn * 4);
}

cudaError_t cg_colsum_reduce(void *workspace, int ngroups, int kn, float *out, cudaStream_t st) {
    const int nchunks = (ngroups + BN_CHUNK - 1) / BN_CHUNK;
    double *chunks = (double *) workspace;
    const float *part = (const float *) ((uint8_t *) workspace + (size_t) nchunks * 2 * kn * 8);
    dim3 g1((kn + 31) / 32, nchunks);
    bn_stats_pass1<<<g1, 256, 0, st>>>(part, ngroups, kn, chunks);
    cg_note_launch();
    colsum_pass2_f32<<<(kn + 127) / 128, 128, 0, st>>>(chunks, nchunks, kn, out);
    cg_note_launch();
    return cudaGetLastError();
}

extern "C" size_t convgemm_fwd_bf16_stats_workspace_size(const convgemm_shape_t *shape) {
    if (!shape || shape->b < 1 || shape->kn < 1 || shape->c < 1) return 0;
    if (convgemm_bf16_weights_size(shape, CONVGEMM_OPERAND_FWD) == 0) return 0;
    return stats_ws_bytes(cg_from_public(*shape));
}

extern "C" convgemm_status_t convgemm_fwd_bf16_stats(const convgemm_shape_t *shape, const void *x,
                                                     const void *wpacked, void *y, const float *scale,
                                                     const float *shift, int relu, double *stats, void *workspace,
                                                     size_t workspace_bytes, void *stream) {
    const char *fn = "convgemm_fwd_bf16_stats";
    if (!shape || !x || !wpacked || !y || !stats || !workspace)
        return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "%s: NULL argument", fn);
    const size_t need = convgemm_fwd_bf16_stats_workspace_size(shape);
    if (need == 0) return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "%s: invalid shape", fn);
    if (workspace_bytes < need || ((uintptr_t) workspace & 15))
        return cg_set_error(CONVGEMM_ERROR_WORKSPACE, "%s: workspace needs %zu bytes, 16-byte aligned", fn, need);
    if (shape->kn % 8) return cg_set_error(CONVGEMM_ERROR_NOT_SUPPORTED, "%s: kn must be a multiple of 8", fn);
    const cg_shape s = cg_from_public(*shape);
    bool stem;
    const int ng = stat_groups(s, &stem);
    const int nchunks = (ng + BN_CHUNK - 1) / BN_CHUNK;
    double *chunks = (double *) workspace;
    float *part = (float *) ((uint8_t *) workspace + (size_t) nchunks * 2 * s.kn * 8);
    const cudaStream_t st = (cudaStream_t) stream;
    TcPlan pl;
    tc_plan_fwd(s, pl);
    convgemm_status_t e;
    if (stem) {
        if (((uintptr_t) y & 15) || ((uintptr_t) wpacked & 15) || ((uintptr_t) x & 15))
            return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "%s: tensors must be 16-byte aligned", fn);
        e = tc_stem_run(s, x, wpacked, pl.Ktot, y, scale, shift, relu, st, part);
    } else {
        if (pl.ncls != 1) return cg_set_error(CONVGEMM_ERROR_NOT_SUPPORTED, "%s: forward plan with several classes", fn);
        TcTune t{0, 0};
        tc_tune_get(CONVGEMM_TUNE_FWD, *shape, &t);
        e = tc_run(pl, s, x, wpacked, y, scale, shift, relu, st, 0, nullptr, nullptr, t.bn, t.splits, nullptr, part);
    }
    if (e) return e;
    dim3 g1((s.kn + 31) / 32, nchunks);
    bn_stats_pass1<<<g1, 256, 0, st>>>(part, ng, s.kn, chunks);
    cg_note_launch();
    bn_stats_pass2<<<(2 * s.kn + 127) / 128, 128, 0, st>>>(chunks, nchunks, s.kn, stats);
    cg_note_launch();
    return cg_cuda_check(cudaGetLastError(), "batch statistics reduction");
}

extern "C" convgemm_status_t convgemm_bn_stats_fold(int kn, const double *stats, long long count, const float *gamma,
                                                    const float *beta, float eps, float *scale, float *shift,
                                                    float *batch_mean, float *batch_var, void *stream) {
    if (kn < 1 || !stats || count < 1 || !scale || !shift || !(eps >= 0.0f))
        return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "convgemm_bn_stats_fold: bad arguments");
    bn_fold_kernel<<<(kn + 127) / 128, 128, 0, (cudaStream_t) stream>>>(kn, stats, 1.0 / (double) count, gamma, beta,
                                                                        eps, scale, shift, batch_mean, batch_var);
    cg_note_launch();
    return cg_cuda_check(cudaGetLastError(), "convgemm_bn_stats_fold");
}

extern "C" convgemm_status_t convgemm_bn_apply_bf16(long long npix, int kn, const void *z, const float *scale,
                                                    const float *shift, int relu, void *y, void *stream) {
    if (npix < 1 || kn < 8 || kn % 8 || !z || !scale || !shift || !y)
        return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "convgemm_bn_apply_bf16: bad arguments (kn % 8 == 0)");
    if (((uintptr_t) z & 15) || ((uintptr_t) y & 15))
        return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "convgemm_bn_apply_bf16: tensors must be 16-byte aligned");
    const long long n8 = npix * (kn / 8);
    long long blocks = (n8 + 255) / 256;
    if (blocks > 152 * 16) blocks = 152 * 16;
    bn_apply_kernel<<<(int) blocks, 256, 0, (cudaStream_t) stream>>>(n8, kn, (const __nv_bfloat16 *) z, scale, shift,
                                                                     relu, (__nv_bfloat16 *) y);
    cg_note_launch();
    return cg_cuda_check(cudaGetLastError(), "convgemm_bn_apply_bf16");
}
