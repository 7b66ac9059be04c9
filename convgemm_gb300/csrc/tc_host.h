// Planning structures shared by the tensor-core host code.
#pragma once
#include <cuda.h>

#include "../../include/convgemm_gpu.h"
#include "cg_internal.h"
#include "prep.h"
#include "tc_conv.h"

// A planned tensor-core convolution: its classes, and the packed-operand geometry.
struct TcPlan {
    int Cin, Cout, Hin, Win, Hout, Wout;
    int ncls, Ktot, mtiles_max, bn;
    bool has_empty_class;
    TcClass cls[TC_MAXCLS];
    int8_t kx[TC_MAXCLS][TC_MAXTAPS], ky[TC_MAXCLS][TC_MAXTAPS];
};

bool tc_plan_fwd(const cg_shape &s, TcPlan &pl);
bool tc_plan_dgrad(const cg_shape &s, TcPlan &pl);
PackDgradInfo tc_pack_info(const TcPlan &pl);
convgemm_status_t tc_make_map_2d(CUtensorMap *map, CUtensorMapDataType dt, int elem_bytes, const void *ptr,
                                 long long rows, long long cols, int box_cols, int box_rows);
convgemm_status_t tc_make_map_2d_sw(CUtensorMap *map, CUtensorMapDataType dt, int elem_bytes, const void *ptr,
                                    long long rows, long long cols, int box_cols, int box_rows, CUtensorMapSwizzle sw);
convgemm_status_t tc_make_im2col_map(CUtensorMap *map, const void *ptr, int B, int H, int W, int C, int lo_h,
                                     int lo_w, int up_h, int up_w, int sh, int sw, int pixels, int elem_bytes,
                                     int chans = 64);
bool tc_plan_im2col(TcPlan &pl);
// BF16 tiled tensor map of any rank (<= 5): dims / box / element strides innermost first,
// strides_bytes of dims 1.. ; 128-byte swizzle or none.
convgemm_status_t tc_make_map_nd(CUtensorMap *map, int rank, const void *ptr, const unsigned long long *dims,
                                  const unsigned long long *strides_bytes, const unsigned *box, const unsigned *estr,
                                  int swizzle128);
// The same for another element type.
convgemm_status_t tc_make_map_nd_dt(CUtensorMap *map, CUtensorMapDataType dt, int rank, const void *ptr,
                                     const unsigned long long *dims, const unsigned long long *strides_bytes,
                                     const unsigned *box, const unsigned *estr, int swizzle128);
// Stride-1 convolutions with 64-channel input blocks and 2..16 taps, operands read from
// input slabs (tc_slab.cu): the forward or input-gradient plan decides.
bool tc_slab_applicable(const TcPlan &pl);
convgemm_status_t tc_slab_run(const TcPlan &pl, const cg_shape &s, const void *in, const void *wpacked, void *out,
                              const float *scale, const float *shift, int relu, cudaStream_t st);
// Forward of convolutions with at most 8 input channels (tc_stem.cu).
bool tc_stem_applicable(const cg_shape &s);
convgemm_status_t tc_stem_run(const cg_shape &s, const void *x, const void *wpacked, int Kpad, void *y,
                              const float *scale, const float *shift, int relu, cudaStream_t st,
                              float *stats = nullptr);
// Statistics groups the small-channel forward writes: 4 per (image row, 128-pixel chunk).
int tc_stem_stat_groups(const cg_shape &s);

int tc_num_sms();
// Argument and size checks shared by the tensor-core entry points (records the error).
convgemm_status_t tc_check_shape(const convgemm_shape_t *shape, const char *fn);
// Weight gradient of stride-2 convolutions with c <= 8 and kn == 64 (the ResNet stem) from
// input slabs: applicability, the number of FP32 partials (workspace planes before the
// reduction's groups), and the run (partials into ws, then the fixed-order reduction into dw
// in layout 0 NHWC-API / 1 NCHW-API).
bool tc_stem_wgrad_applicable(const cg_shape &s);
int tc_stem_wgrad_splits(const cg_shape &s);
convgemm_status_t tc_stem_wgrad_run(const cg_shape &s, const void *dy, const void *x, float *ws, float *dw,
                                    int layout, cudaStream_t st);
// Weight gradient of stride-1 convolutions with 128-channel input blocks from input slabs
// (tc_wgrad_slab.cu): the number of FP32 partials for a requested split count (0: the
// heuristic), 0 if the shape does not fit the kernel; and the run (partials into ws, then
// the fixed-order reduction into dw; one split writes dw directly).
int tc_wgrad_slab_splits(const cg_shape &s, int want_splits, int want_bn);
int tc_wgrad_slab_bn(const cg_shape &s, int want_bn);   // output-channel tile width (64 / 128)
convgemm_status_t tc_wgrad_slab_run(const cg_shape &s, int want_splits, int want_bn, const void *dy, const void *x,
                                    float *ws, float *dw, int layout, cudaStream_t st);
// Autotuned tile configuration of one operation on one shape (0 = heuristic):
// bn = output channels per tile; splits = pixel splits of the weight gradient,
// or M tiles per weight tile (1 or 2) of the forward / input gradient.
struct TcTune {
    int bn, splits;
};
bool tc_tune_get(int op, const convgemm_shape_t &s, TcTune *t);

// mode: 0 BF16, 1 FP8-E4M3 (in/wpacked are E4M3), 2 3xBF16 (in_lo/w_lo low parts, FP32 output)
convgemm_status_t tc_run(const TcPlan &pl, const cg_shape &s, const void *in, const void *wpacked, void *out,
                         const float *scale, const float *shift, int relu, cudaStream_t st, int mode = 0,
                         const void *in_lo = nullptr, const void *w_lo = nullptr, int bn_override = 0,
                         int aux_override = 0, const void *mask = nullptr,
                         float *stats = nullptr, int accum = 0);
