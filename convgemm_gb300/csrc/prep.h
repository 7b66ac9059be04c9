// Launchers of the preparation kernels (prep.cu).
#pragma once
#include <cuda_runtime.h>

#include "tc_conv.h"

// Where each stride-phase class of the input gradient sits in the packed operand.
struct PackDgradInfo {
    int ncls, Ktot;
    int kbeg[TC_MAXCLS], ntaps[TC_MAXCLS];
    int8_t kx[TC_MAXCLS][TC_MAXTAPS], ky[TC_MAXCLS][TC_MAXTAPS];
};

cudaError_t prep_pack_fwd(const float *w, int nchw, int C, int kh, int kw, int kn, int Cp, int Kpad, void *out,
                          cudaStream_t st);
cudaError_t prep_pack_dgrad(const float *w, int nchw, int C, int kh, int kw, int kn, int knp,
                            const PackDgradInfo &info, void *out, cudaStream_t st);
cudaError_t prep_fold(int kn, const float *bias, const float *mean, const float *inv_std, const float *gamma,
                      const float *beta, float *scale, float *shift, cudaStream_t st);
cudaError_t prep_to_bf16_nhwc(const float *in, int nchw, int B, int C, int H, int W, int Cp, void *out,
                              cudaStream_t st);

cudaError_t prep_fp8_quantize(long long n, int in_bf16, const void *in, void *out, float *scale, unsigned *amax_tmp,
                              cudaStream_t st);
cudaError_t prep_pack_fp8(const float *w, int nchw, int C, int kh, int kw, int kn, int Cp, int Kpad, void *out,
                          float *wscale, cudaStream_t st);
cudaError_t prep_fp8_scales(int kn, const float *scale, const float *shift, const float *wscale, const float *xscale,
                            float *out_scale, float *out_shift, cudaStream_t st);
cudaError_t prep_split(long long n, const float *in, void *hi, void *lo, cudaStream_t st);
cudaError_t prep_pack_split(const float *w, int nchw, int C, int kh, int kw, int kn, int Cp, int Kpad, void *hi,
                            void *lo, cudaStream_t st);
