/*
 * convGemm drop-in interface, GB300 (sm_103a) implementation.
 *
 * The five declarations below keep the names, argument order and meaning of
 * the reference's public header (hpca-uji/convGemm src/convGemm.h:20-64) so a
 * program built against libconvGemm.so links against this library unchanged.
 * The one difference in this file is that it includes <stdbool.h> itself
 * (the reference header uses `bool` without it, src/convGemm.h:32).
 *
 * Semantics (all FP32, results within 1e-5 relative of the reference; forward
 * and weight gradient follow the reference's KC=384 blocked summation order):
 *
 *   sconvGemmNHWC(trans='N')  out[b][ho][wo][kn] = epi(conv(x, in))      (src/convGemm.c:65-70)
 *       in  = weights [c][kh][kw][kn], x = input NHWC [b][h][w][c]
 *       epi = +bias, then (v-mean)*inv_std*gamma+beta, then ReLU, each optional
 *   sconvGemmNHWC(trans!='N') out = dW [c][kh][kw][kn],  in = dY NHWC  (src/convGemm.c:71-76)
 *   sconvGemmNHWC_back        dx[b][h][w][c] += dgrad(weights, dy)     (src/convGemm.c:82-97)
 *   sconvGemmNCHW(...)        the same in NCHW, weights [kn][c][kh][kw] (src/convGemm.c:99-125)
 *   sconvGemmNCHW_back        dx[b][c][h][w] += dgrad(weights, dy)     (src/convGemm.c:130-146)
 *
 * The _back functions take the strides BEFORE the paddings, as in the reference.
 *
 * Pointers may be device pointers (the work runs on the legacy default
 * stream, ordered with other work on it) or host pointers (the library stages
 * them through device buffers and returns when the results are back in host
 * memory).  ac_pack / bc_pack are accepted and ignored; NULL is fine.
 *
 * These functions return nothing, like the reference.  Errors (invalid
 * geometry, CUDA failures) are recorded and can be read with
 * convgemm_get_last_error() from convgemm_gpu.h.
 */
#ifndef CONVGEMM_H
#define CONVGEMM_H

#include <stdbool.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Replaces src/convGemm.h:20.  Returns 0 and sets both pointers to NULL: the
 * GPU kernels need no packing buffers (the reference allocates
 * omp_get_max_threads()*MC*KC and *KC*NC floats, src/convGemm.c:30-40). */
int alloc_pack_buffs(float **Ac_pack, float **Bc_pack);

/* Replaces src/convGemm.h:22-33. */
void sconvGemmNHWC(char trans,
                   int b, int h, int w, int c,
                   int kn, int kh, int kw,
                   int vpadding, int hpadding,
                   int vstride, int hstride,
                   int vdilation, int hdilation,
                   const float *in,
                   const float *x,
                   float *out, const float *bias_vector,
                   const float *bn_running_mean, const float *bn_inv_std,
                   const float *bn_gamma, const float *bn_beta, bool relu,
                   float *ac_pack, float *bc_pack);

/* Replaces src/convGemm.h:35-42. */
void sconvGemmNHWC_back(int b, int h, int w, int c,
                        int kn, int kh, int kw,
                        int vstride, int hstride,
                        int vpadding, int hpadding,
                        int vdilation, int hdilation,
                        const float *weights,
                        const float *dy, float *dx,
                        float *ac_pack, float *bc_pack);

/* Replaces src/convGemm.h:44-55. */
void sconvGemmNCHW(char trans,
                   int b, int c, int h, int w,
                   int kn, int kh, int kw,
                   int vpadding, int hpadding,
                   int vstride, int hstride,
                   int vdilation, int hdilation,
                   const float *in,
                   const float *x,
                   float *out, const float *bias_vector,
                   const float *bn_running_mean, const float *bn_inv_std,
                   const float *bn_gamma, const float *bn_beta, bool relu,
                   float *ac_pack, float *bc_pack);

/* Replaces src/convGemm.h:57-64. */
void sconvGemmNCHW_back(int b, int c, int h, int w,
                        int kn, int kh, int kw,
                        int vstride, int hstride,
                        int vpadding, int hpadding,
                        int vdilation, int hdilation,
                        const float *weights,
                        const float *dy, float *dx,
                        float *ac_pack, float *bc_pack);

#ifdef __cplusplus
}
#endif

#endif /* CONVGEMM_H */
