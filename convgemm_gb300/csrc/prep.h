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

// One job of the grouped preparation launch (prep_group_launch): a block range of
// one batch-norm fold or one weight packing.
enum { PREP_FOLD = 0, PREP_FWD_TILED = 1, PREP_FWD_ELEM = 2, PREP_FWD_TAIL = 3, PREP_DGRAD = 4 };
struct PrepJob {
    int type, block0, nblocks;                 // blocks [block0, block0 + nblocks) of the launch
    int nchw, C, kh, kw, kn, Cp, Kpad, knp;    // weight geometry (packing jobs)
    const float *w;
    void *out;
    const float *bias, *mean, *inv_std, *gamma, *beta;   // fold job
    float *scale, *shift;
    PackDgradInfo info;                        // input-gradient packing job
    FastDiv dknp;                              // division by knp
};
// jobs: device array sorted by block0, followed by the njobs block0 values as ints
// (at most 12288 jobs); nblocks: total blocks of all jobs.
cudaError_t prep_group_launch(const PrepJob *jobs, int njobs, int nblocks, cudaStream_t st);

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
