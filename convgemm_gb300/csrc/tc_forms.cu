// Public entry points of the FP8-E4M3 and 3xBF16 forward forms.
//
// FP8-E4M3: activations quantised per tensor (scale = amax/448), weights per
// output channel; the tensor cores multiply E4M3 x E4M3 (tcgen05 kind::f8f6f4)
// into FP32 TMEM accumulators and the two scales fold into the epilogue scale.
// 3xBF16: every FP32 operand is split x = hi + lo (both BF16) and the kernel
// accumulates hi*hi + hi*lo + lo*hi (kind::f16) in FP32, recovering most of the
// FP32 accuracy at three BF16 MMAs per product.  Both generalise
// sconvGemmNHWC('N') (src/convGemm.c:65-70) and need c % 64 == 0.
#include <cstring>

#include "../../include/convgemm_gpu.h"
#include "cg_common.cuh"
#include "prep.h"
#include "tc_host.h"

namespace {

convgemm_status_t check_form_shape(const convgemm_shape_t *shape, const char *fn) {
    if (!shape) return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "%s: shape is NULL", fn);
    const convgemm_shape_t &s = *shape;
    if (s.b < 1 || s.h < 1 || s.w < 1 || s.c < 1 || s.kn < 1 || s.kh < 1 || s.kw < 1 || s.vstride < 1 ||
        s.hstride < 1 || s.vdil < 1 || s.hdil < 1 || s.vpad < 0 || s.hpad < 0 ||
        s.h + 2LL * s.vpad - (long long) s.vdil * (s.kh - 1) < 1 ||
        s.w + 2LL * s.hpad - (long long) s.hdil * (s.kw - 1) < 1)
        return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "%s: invalid geometry", fn);
    if (s.c % 64 || s.kn % 8)
        return cg_set_error(CONVGEMM_ERROR_NOT_SUPPORTED, "%s: needs c %% 64 == 0 and kn %% 8 == 0", fn);
    if (s.kh * s.kw > TC_MAXTAPS)
        return cg_set_error(CONVGEMM_ERROR_NOT_SUPPORTED, "%s: filters above 49 taps", fn);
    return CONVGEMM_SUCCESS;
}

}  // namespace

extern "C" convgemm_status_t convgemm_fp8_quantize(size_t n, int in_is_bf16, const void *in, void *out,
                                                   float *scale, void *stream) {
    if (!in || !out || !scale || n == 0)
        return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "convgemm_fp8_quantize: bad arguments");
    // scale[0] receives the per-tensor scale, scale[1] is the amax accumulator
    return cg_cuda_check(prep_fp8_quantize((long long) n, in_is_bf16, in, out, scale, (unsigned *) (scale + 1),
                                           (cudaStream_t) stream),
                         "fp8 quantise");
}

extern "C" size_t convgemm_fp8_weights_size(const convgemm_shape_t *shape) {
    if (check_form_shape(shape, "convgemm_fp8_weights_size")) return 0;
    TcPlan pl;
    tc_plan_fwd(cg_from_public(*shape), pl);
    return (size_t) pl.Cout * pl.Ktot;
}

extern "C" convgemm_status_t convgemm_fp8_pack_weights(convgemm_layout_t layout, const convgemm_shape_t *shape,
                                                       const float *weights, void *packed, float *wscale,
                                                       void *stream) {
    if (convgemm_status_t e = check_form_shape(shape, "convgemm_fp8_pack_weights")) return e;
    if (!weights || !packed || !wscale)
        return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "convgemm_fp8_pack_weights: NULL");
    const cg_shape s = cg_from_public(*shape);
    TcPlan pl;
    tc_plan_fwd(s, pl);
    return cg_cuda_check(prep_pack_fp8(weights, layout == CONVGEMM_NCHW, s.c, s.kh, s.kw, s.kn, pl.Cin, pl.Ktot, packed,
                                       wscale, (cudaStream_t) stream),
                         "fp8 pack weights");
}

extern "C" convgemm_status_t convgemm_fp8_epilogue_scales(int kn, const float *scale, const float *shift,
                                                          const float *wscale, const float *xscale, float *out_scale,
                                                          float *out_shift, void *stream) {
    if (kn < 1 || !wscale || !xscale || !out_scale || !out_shift)
        return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "convgemm_fp8_epilogue_scales: bad arguments");
    return cg_cuda_check(prep_fp8_scales(kn, scale, shift, wscale, xscale, out_scale, out_shift, (cudaStream_t) stream),
                         "fp8 epilogue scales");
}

extern "C" convgemm_status_t convgemm_fwd_fp8(const convgemm_shape_t *shape, const void *x, const void *wpacked,
                                              void *y, const float *scale, const float *shift, int relu,
                                              void *stream) {
    if (convgemm_status_t e = check_form_shape(shape, "convgemm_fwd_fp8")) return e;
    if (!x || !wpacked || !y || !scale) return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "convgemm_fwd_fp8: NULL");
    const cg_shape s = cg_from_public(*shape);
    TcPlan pl;
    tc_plan_fwd(s, pl);
    TcTune t{0, 0};
    tc_tune_get(CONVGEMM_TUNE_FWD_FP8, *shape, &t);
    return tc_run(pl, s, x, wpacked, y, scale, shift, relu, (cudaStream_t) stream, 1, nullptr, nullptr, t.bn);
}

extern "C" convgemm_status_t convgemm_split_bf16x2(size_t n, const float *in, void *hi, void *lo, void *stream) {
    if (!in || !hi || !lo || n == 0)
        return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "convgemm_split_bf16x2: bad arguments");
    return cg_cuda_check(prep_split((long long) n, in, hi, lo, (cudaStream_t) stream), "split to bf16 pairs");
}

extern "C" convgemm_status_t convgemm_bf16x3_pack_weights(convgemm_layout_t layout, const convgemm_shape_t *shape,
                                                          const float *weights, void *hi, void *lo, void *stream) {
    if (convgemm_status_t e = check_form_shape(shape, "convgemm_bf16x3_pack_weights")) return e;
    if (!weights || !hi || !lo) return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "convgemm_bf16x3_pack_weights: NULL");
    const cg_shape s = cg_from_public(*shape);
    TcPlan pl;
    tc_plan_fwd(s, pl);
    return cg_cuda_check(prep_pack_split(weights, layout == CONVGEMM_NCHW, s.c, s.kh, s.kw, s.kn, pl.Cin, pl.Ktot, hi,
                                         lo, (cudaStream_t) stream),
                         "bf16x3 pack weights");
}

extern "C" convgemm_status_t convgemm_fwd_bf16x3(const convgemm_shape_t *shape, const void *x_hi, const void *x_lo,
                                                 const void *w_hi, const void *w_lo, float *y, const float *scale,
                                                 const float *shift, int relu, void *stream) {
    if (convgemm_status_t e = check_form_shape(shape, "convgemm_fwd_bf16x3")) return e;
    if (!x_hi || !x_lo || !w_hi || !w_lo || !y)
        return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "convgemm_fwd_bf16x3: NULL");
    const cg_shape s = cg_from_public(*shape);
    TcPlan pl;
    tc_plan_fwd(s, pl);
    TcTune t{0, 0};
    tc_tune_get(CONVGEMM_TUNE_FWD_BF16X3, *shape, &t);
    return tc_run(pl, s, x_hi, w_hi, y, scale, shift, relu, (cudaStream_t) stream, 2, x_lo, w_lo, t.bn);
}
