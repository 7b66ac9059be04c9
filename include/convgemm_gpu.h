/*
 * convGemm GB300 extended interface: explicit streams, device pointers,
 * status codes, caller-provided workspaces and the tensor-core precision forms.
 *
 * The reference has no counterpart for most of this file; each function says
 * which reference entry point it generalises.  All pointers are DEVICE
 * pointers; `stream` is a cudaStream_t (NULL = legacy default stream).
 * Nothing here synchronises the stream unless it says so.
 */
#ifndef CONVGEMM_GPU_H
#define CONVGEMM_GPU_H

#include <stddef.h>
#include <stdint.h>
#include <stdbool.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    CONVGEMM_SUCCESS = 0,
    CONVGEMM_ERROR_INVALID_VALUE = 1,  /* bad geometry, NULL pointer, bad enum */
    CONVGEMM_ERROR_NOT_SUPPORTED = 2,  /* no kernel for this shape / form */
    CONVGEMM_ERROR_CUDA = 3,           /* a CUDA runtime or driver call failed */
    CONVGEMM_ERROR_ALLOC = 4,          /* a device or host allocation failed */
    CONVGEMM_ERROR_TIMEOUT = 5,        /* a bounded device-side wait ran out */
    CONVGEMM_ERROR_WORKSPACE = 6       /* caller workspace smaller than required */
} convgemm_status_t;

typedef enum { CONVGEMM_NHWC = 0, CONVGEMM_NCHW = 1 } convgemm_layout_t;

/* One 2-D convolution.  Output size follows src/convGemm.c:60-61:
 * ho = (h + 2*vpad - vdil*(kh-1) - 1)/vstride + 1 (same for wo). */
typedef struct {
    int b, h, w, c;      /* batch, input height, width, channels */
    int kn, kh, kw;      /* output channels, filter height, width */
    int vpad, hpad;      /* symmetric zero padding */
    int vstride, hstride;
    int vdil, hdil;
} convgemm_shape_t;

/* Per-output-channel epilogue of the forward pass (src/im2row_nhwc.c:269-285):
 * v += bias; v = (v - mean)*inv_std; v = v*gamma + beta; v = max(v, 0).
 * Any pointer may be NULL; batch-norm is on when mean is set (then inv_std,
 * gamma and beta must be set too). */
typedef struct {
    const float *bias;
    const float *mean;
    const float *inv_std;
    const float *gamma;
    const float *beta;
    int relu;
} convgemm_epilogue_t;

/* ---------------------------------------------------------------- errors */

/* Status and message of the last failing call on this host thread. */
convgemm_status_t convgemm_get_last_status(void);

/* Self-test of the failure path: launches a kernel whose device-side wait runs
 * out after budget_ms (1..1000) because nothing completes its barrier; the kernel
 * records CONVGEMM_SELFTEST_WAIT_CODE in the device error word and returns, and
 * the next convgemm_check_device returns CONVGEMM_ERROR_TIMEOUT (and clears it). */
#define CONVGEMM_SELFTEST_WAIT_CODE 99
convgemm_status_t convgemm_selftest_wait_timeout(unsigned budget_ms, void *stream);

/* Number of GPU kernels the library has launched (or recorded into a stream
 * capture) in this process: a diagnostic for counting launches per step. */
unsigned long long convgemm_launch_count(void);
/* Programmatic dependent launch of the persistent forward / input-gradient kernels
 * (a kernel's prologue overlaps the previous kernel's tail on the same stream), for
 * the calling host thread: 1 on, 0 off, -1 back to the default (on unless the
 * environment sets CONVGEMM_NO_PDL=1).  Returns the previous setting (0 / 1).
 * Turn it off while other streams run work beside the chain: the early-launched
 * CTAs then hold SMs that the other streams' grids would fill. */
int convgemm_set_pdl(int on);
const char *convgemm_get_last_error(void);
void convgemm_clear_error(void);
/* Reads (and clears) the device-side error word that bounded waits set; it
 * synchronises the stream first.  One word per device serves every kernel of the
 * library, convgemm_wgrad_bf16_noalloc's included; it is a file-scope device
 * variable, so neither this call nor any kernel launch allocates for it. */
convgemm_status_t convgemm_check_device(void *stream);
/* Measurement of the FP32 FMA peak (no counterpart in the reference): launches one kernel of
 * independent FMA chains on every SM (`iters` loop trips per thread) on `stream` and returns in
 * *flops the FLOPs it performs; time it with events to get FLOP/s.  out: one device float. */
convgemm_status_t convgemm_measure_ffma(int iters, float *out, double *flops, void *stream);

/* ------------------------------------------------------- FP32 plain form */

/* sconvGemmNHWC/NCHW(trans='N') on device pointers (src/convGemm.c:65-70, 116-119). */
convgemm_status_t convgemm_fwd_f32(convgemm_layout_t layout, const convgemm_shape_t *shape,
                                   const float *weights, const float *x, float *y,
                                   const convgemm_epilogue_t *epi, void *stream);

/* Workspace of convgemm_wgrad_f32 in bytes (the per-KC-block partials that
 * the fixed-order reduction sums). */
size_t convgemm_wgrad_f32_workspace_size(const convgemm_shape_t *shape);

/* sconvGemmNHWC/NCHW(trans='T') on device pointers (src/convGemm.c:71-76, 120-124):
 * dw = dY x im2row(x)^T, overwritten; bit-reproducible run to run. */
convgemm_status_t convgemm_wgrad_f32(convgemm_layout_t layout, const convgemm_shape_t *shape,
                                     const float *dy, const float *x, float *dw,
                                     void *workspace, size_t workspace_bytes, void *stream);

/* sconvGemmNHWC_back / sconvGemmNCHW_back on device pointers
 * (src/convGemm.c:82-97, 130-146) in gather form (no col2im scatter, no
 * atomics, deterministic).  accumulate != 0 adds into dx as the reference
 * does; accumulate == 0 overwrites dx. */
convgemm_status_t convgemm_dgrad_f32(convgemm_layout_t layout, const convgemm_shape_t *shape,
                                     const float *weights, const float *dy, float *dx,
                                     int accumulate, void *stream);

/* -------------------------------------------- BF16 tensor-core form (NHWC) */

/* Which packed operand convgemm_bf16_pack_weights produces. */
#define CONVGEMM_OPERAND_FWD 0    /* forward:        [kn][taps * c8], c8 = c rounded up to 8 */
#define CONVGEMM_OPERAND_DGRAD 1  /* input gradient: [c][classes x taps x kn8], flipped taps */

/* Bytes of a packed BF16 weight operand (0 if the shape has no tensor-core kernel). */
size_t convgemm_bf16_weights_size(const convgemm_shape_t *shape, int kind);

/* Packs FP32 weights in the reference layout of `layout` (NHWC API: [c][kh][kw][kn];
 * NCHW API: [kn][c][kh][kw]) into the BF16 operand of the tensor-core kernels. */
convgemm_status_t convgemm_bf16_pack_weights(convgemm_layout_t layout, const convgemm_shape_t *shape, int kind,
                                             const float *weights, void *packed, void *stream);

/* Folds bias and batch-norm into per-channel scale/shift in FP64 on the GPU:
 * scale = gamma*inv_std, shift = beta + (bias - mean)*scale (identity without BN). */
convgemm_status_t convgemm_fold_epilogue(int kn, const convgemm_epilogue_t *epi, float *scale, float *shift,
                                         void *stream);

/* FP32 activations (NHWC, or NCHW [b][c][h][w]) -> BF16 NHWC with the channel
 * dimension padded to a multiple of 8 (padding zero), as the BF16 kernels read them. */
convgemm_status_t convgemm_to_bf16_nhwc(convgemm_layout_t layout, int b, int c, int h, int w, const float *in,
                                        void *out, void *stream);

/* Forward, BF16 tensor cores (tcgen05, FP32 accumulation in TMEM): generalises
 * sconvGemmNHWC('N') (src/convGemm.c:65-70).  x: BF16 NHWC [b][h][w][c8];
 * y: BF16 NHWC [b][ho][wo][kn] = relu?(acc*scale + shift); scale/shift may be NULL.
 * Needs kn % 8 == 0. */
convgemm_status_t convgemm_fwd_bf16(const convgemm_shape_t *shape, const void *x, const void *wpacked, void *y,
                                    const float *scale, const float *shift, int relu, void *stream);

/* Input gradient, BF16 tensor cores, gather form (no col2im scatter):
 * generalises sconvGemmNHWC_back (src/convGemm.c:82-97).  dy: BF16 NHWC
 * [b][ho][wo][kn8]; dx: BF16 NHWC [b][h][w][c], overwritten.  Needs c % 8 == 0. */
convgemm_status_t convgemm_dgrad_bf16(const convgemm_shape_t *shape, const void *dy, const void *wpacked, void *dx,
                                      void *stream);

/* ------------------------------------------- FP8-E4M3 and 3xBF16 forward forms */

/* Per-tensor E4M3 quantisation of n contiguous values (BF16 if in_is_bf16, else FP32):
 * scale[0] = amax/448, out = e4m3(in/scale[0]); scale must hold 2 floats (scale[1] is scratch). */
convgemm_status_t convgemm_fp8_quantize(size_t n, int in_is_bf16, const void *in, void *out, float *scale,
                                        void *stream);

/* Bytes of the packed E4M3 weight operand ([kn][taps*c], K padded to 64). */
size_t convgemm_fp8_weights_size(const convgemm_shape_t *shape);

/* Per-output-channel E4M3 weights: wscale[n] = amax_n/448, packed = e4m3(w/wscale[n]). */
convgemm_status_t convgemm_fp8_pack_weights(convgemm_layout_t layout, const convgemm_shape_t *shape,
                                            const float *weights, void *packed, float *wscale, void *stream);

/* Folds the quantisation scales into the epilogue: out_scale[n] = scale[n]*wscale[n]*xscale[0],
 * out_shift[n] = shift[n] (scale/shift from convgemm_fold_epilogue, or NULL for 1/0). */
convgemm_status_t convgemm_fp8_epilogue_scales(int kn, const float *scale, const float *shift, const float *wscale,
                                               const float *xscale, float *out_scale, float *out_shift, void *stream);

/* Forward, E4M3 x E4M3 tensor cores (tcgen05 kind::f8f6f4), FP32 accumulation:
 * x E4M3 NHWC [b][h][w][c], y BF16 NHWC = relu?(acc*scale + shift).  Needs c % 64 == 0. */
convgemm_status_t convgemm_fwd_fp8(const convgemm_shape_t *shape, const void *x, const void *wpacked, void *y,
                                   const float *scale, const float *shift, int relu, void *stream);

/* x = hi + lo, both BF16 (hi = bf16(x), lo = bf16(x - hi)), n contiguous FP32 values. */
convgemm_status_t convgemm_split_bf16x2(size_t n, const float *in, void *hi, void *lo, void *stream);

/* Packed hi/lo BF16 weight operands (each convgemm_bf16_weights_size(shape, CONVGEMM_OPERAND_FWD) bytes). */
convgemm_status_t convgemm_bf16x3_pack_weights(convgemm_layout_t layout, const convgemm_shape_t *shape,
                                               const float *weights, void *hi, void *lo, void *stream);

/* Forward with 3xBF16 split products (hi*hi + hi*lo + lo*hi accumulated in FP32):
 * x_hi/x_lo BF16 NHWC [b][h][w][c]; y FP32 NHWC.  Needs c % 64 == 0. */
convgemm_status_t convgemm_fwd_bf16x3(const convgemm_shape_t *shape, const void *x_hi, const void *x_lo,
                                      const void *w_hi, const void *w_lo, float *y, const float *scale,
                                      const float *shift, int relu, void *stream);

/* ------------------------------------------------------ packed-weight cache */

/* Operand kinds the cache keeps. */
#define CONVGEMM_CACHE_BF16_FWD 0    /* convgemm_bf16_pack_weights(..., CONVGEMM_OPERAND_FWD, ...) */
#define CONVGEMM_CACHE_BF16_DGRAD 1  /* convgemm_bf16_pack_weights(..., CONVGEMM_OPERAND_DGRAD, ...) */
#define CONVGEMM_CACHE_FP8_FWD 2     /* convgemm_fp8_pack_weights: packed E4M3 + kn per-channel scales */

/* The packed tensor-core operand of FP32 `weights` (reference layout of `layout`),
 * from a library-owned cache keyed on (device, weights pointer, layout, shape, kind).
 * The reference packs its weight operand on every call (pack_RB, src/gemm_blis.c:40-88);
 * here an entry is packed once and re-packed on `stream` only when `version` differs
 * from the one it was packed at (a caller-kept counter bumped whenever the weights
 * change, e.g. a torch tensor's _version).  A hit launches nothing.  *packed (and for
 * CONVGEMM_CACHE_FP8_FWD *wscale) stay valid until the entry is evicted.  A miss
 * allocates with cudaMalloc and is refused (CONVGEMM_ERROR_NOT_SUPPORTED) while
 * `stream` is being captured: fill the cache before capturing. */
convgemm_status_t convgemm_weights_cached(convgemm_layout_t layout, const convgemm_shape_t *shape, int kind,
                                          const float *weights, unsigned long long version, const void **packed,
                                          const float **wscale, void *stream);
/* Frees every entry packed from `weights` (all entries when NULL); returns how many.
 * It waits for device work still reading them (cudaFree). */
int convgemm_weights_cache_evict(const float *weights);
/* Device bytes the cache holds. */
size_t convgemm_weights_cache_bytes(void);

/* ------------------------------------------------ grouped weight preparation */

/* One layer's preparation for the BF16 forms: pack its FP32 weights (reference
 * layout of `layout`) into the forward and/or input-gradient operands, and fold
 * its bias / batch-norm into scale / shift (FP64 arithmetic).  NULL outputs are
 * skipped. */
typedef struct {
    convgemm_layout_t layout;
    convgemm_shape_t shape;
    const float *weights;
    void *packed_fwd;        /* convgemm_bf16_weights_size(shape, CONVGEMM_OPERAND_FWD) bytes, or NULL */
    void *packed_dgrad;      /* convgemm_bf16_weights_size(shape, CONVGEMM_OPERAND_DGRAD) bytes, or NULL */
    convgemm_epilogue_t epi; /* fold parameters (relu is not used here) */
    float *scale;            /* kn floats, or NULL (no fold) */
    float *shift;
} convgemm_prep_item_t;

/* Bytes of the device job table for n items (16-byte aligned memory). */
size_t convgemm_prep_table_size(int n);
/* Builds the job table of n items (synchronous copy: outside stream capture);
 * returns the job and block counts for the launch. */
convgemm_status_t convgemm_prep_prepare(int n, const convgemm_prep_item_t *items, void *table, size_t table_bytes,
                                        int *njobs, int *nblocks);
/* Every fold and packing of the table in one launch (capturable in a CUDA graph);
 * results are identical to the per-layer calls. */
convgemm_status_t convgemm_prep_launch(const void *table, int njobs, int nblocks, void *stream);

/* ------------------------------------------------ autotuned tile configuration */

/* Operations a tile configuration can be set for. */
enum {
    CONVGEMM_TUNE_FWD = 0,        /* convgemm_fwd_bf16 */
    CONVGEMM_TUNE_DGRAD = 1,      /* convgemm_dgrad_bf16 */
    CONVGEMM_TUNE_WGRAD = 2,      /* convgemm_wgrad_bf16 (and its workspace size) */
    CONVGEMM_TUNE_FWD_FP8 = 3,    /* convgemm_fwd_fp8 */
    CONVGEMM_TUNE_FWD_BF16X3 = 4  /* convgemm_fwd_bf16x3 */
};

/* Process-wide override of the built-in heuristics for one operation on one
 * shape, as chosen by an autotuner: bn = output channels per tile (64, 128 or
 * 256; for the weight gradient the width of its N side); aux = pixel splits of
 * the weight gradient (bits 0-15; 0 = heuristic) plus the CONVGEMM_WGRAD_* flags
 * below, or, for the BF16 forward / input gradient, the number of
 * 128-row M tiles (1 or 2) that share each weight tile, plus 4 for the kernel
 * form with eight epilogue warps (short-K layers; 0 = heuristic), plus 8 for the general
 * kernel instead of a slab kernel, plus 16 for one K block per ring stage and twice the
 * stages (64 / 128-wide tiles, one M tile, four epilogue warps).
 * bn = aux = 0 removes the entry.  Set the weight-gradient entry before querying
 * its workspace size.  Thread-safe. */
convgemm_status_t convgemm_tune_set(int op, const convgemm_shape_t *shape, int bn, int aux);
/* Weight-gradient flags (channels that are multiples of 64): X, not dY, as the
 * 128-row A operand of a layer with kn >= 128 (N widths 64 / 128 / 256 of kn);
 * X of a 1x1 stride-1 unpadded convolution by im2col boxes instead of tiled
 * boxes of the [pixels][channels] matrix.  Results equal the default's within
 * the BF16 bound (the tiled / im2col choice gives the same bits). */
#define CONVGEMM_WGRAD_X_ON_A 0x10000
#define CONVGEMM_WGRAD_IM2COL_X 0x20000
/* Weight gradient with more than 8 splits: instead of the separate fixed-order reduction
 * kernels, reduce inside the kernel with clusters of 2, 4 or 8 splits (their partial tiles
 * summed through distributed shared memory, the clusters' sums added by the last cluster of
 * each tile to arrive): CONVGEMM_WGRAD_GROUPS(2 / 4 / 8).  The split count is rounded up to
 * a multiple of the cluster size.  The sum order is fixed by the split count and cluster
 * size, so dW stays bit-reproducible. */
/* Weight gradient of a stride-1 layer whose channels are multiples of 128 and kn >= 64 (filters
 * 2..512/BN taps wide, output width + filter span <= 256): the slab kernel, whose MMAs read
 * each kernel row's taps as row-shifted windows of one input slab per band of output rows.
 * It is the default for such layers when the tuning table has no entry for the shape;
 * with an entry it runs when the entry carries this flag (its split count in bits 0-15,
 * 0 = heuristic). */
#define CONVGEMM_WGRAD_SLAB 0x80000
/* Weight gradient (im2col path): one 64-pixel chunk per ring stage and twice as many stages
 * (4 / 6 / 4 for 64 / 128 / 256-wide tiles) instead of two chunks per stage (2 / 3 / 2). */
#define CONVGEMM_WGRAD_STAGES1 0x400000
/* Weight gradient (im2col path, two chunks per stage): a second MMA-issuing warp takes the odd
 * chunks into a second accumulator, added in the epilogue (another summation order: results
 * stay within the FP32 accumulation bound and bit-reproducible). */
#define CONVGEMM_WGRAD_TWO_ISSUERS 0x800000
/* Weight gradient (im2col path): chunks of 128 pixels, one per ring stage, so that every TMA
 * box carries twice the bytes (the per-box cost, not the bytes, bounds a TMA stream of 8 KB
 * boxes); the MMAs run in the same order, so dW is bit-identical to the default's. */
#define CONVGEMM_WGRAD_WIDE_CHUNKS 0x1000000
/* im2col path: CTA pairs (thread-block clusters of two) share 256 x 256 (bn 256, the default) or
 * 256 x 128 (bn 128) tiles through cta_group::2 MMAs, each CTA loading its A rows and half of the
 * B columns (128-pixel chunks); several splits reduce through the workspace.  Other FP32 orders
 * than the default: reproducible, within FP32 accumulation. */
#define CONVGEMM_WGRAD_PAIR 0x2000000
#define CONVGEMM_WGRAD_GROUPS(csize) ((csize) == 8 ? 0x300000 : (csize) == 4 ? 0x200000 : (csize) == 2 ? 0x100000 : 0)
void convgemm_tune_clear(void);
/* What the tuning table (or the heuristic) selects for the forward, input gradient or weight
 * gradient on one shape: *kernel 0 the general implicit GEMM, 1 a slab kernel, 2 the
 * small-channel kernel; *bn the tile width; *stages the ring stages of the general kernels (0 for
 * the slab and small-channel kernels, which size their buffers at run time); *cluster 1, or the
 * thread-block cluster size of a weight gradient whose splits are reduced in a cluster.  The
 * reference chooses its blocking once, from the BLIS context (src/gemm_blis.h:181-188). */
convgemm_status_t convgemm_tune_describe(int op, const convgemm_shape_t *shape, int *kernel, int *bn, int *stages,
                                         int *cluster);

/* ----------------------------------------- grouped persistent forward launch */

/* One convolution of a grouped launch: BF16 NHWC x [b][h][w][c] (c % 8 == 0),
 * weights packed by convgemm_group_pack_weights, BF16 NHWC y [b][ho][wo][kn] =
 * relu?(acc*scale + shift) (scale/shift may be NULL); bn = output channels per
 * tile (64, 128 or 256; 0 = chosen from kn), e.g. from the autotuner. */
typedef struct {
    convgemm_shape_t shape;
    const void *x;
    const void *w;
    void *y;
    const float *scale;
    const float *shift;
    int relu;
    int bn;
} convgemm_group_conv_t;

/* Packed weights of a grouped-launch convolution: [kn][taps * c64], c64 = c rounded up to 64. */
size_t convgemm_group_weights_size(const convgemm_shape_t *shape);
convgemm_status_t convgemm_group_pack_weights(convgemm_layout_t layout, const convgemm_shape_t *shape,
                                              const float *weights, void *packed, void *stream);

/* Bytes of the device problem table of n convolutions (64-byte aligned memory). */
size_t convgemm_group_table_size(int n);

/* Encodes the tensor maps of n convolutions into the device table (synchronous
 * copy; do it once, outside any stream capture) and returns the tile count. */
convgemm_status_t convgemm_group_prepare(int n, const convgemm_group_conv_t *convs, void *table, size_t table_bytes,
                                         int *total_tiles);

/* All n convolutions in one persistent launch (capturable in a CUDA graph). */
convgemm_status_t convgemm_group_launch(const void *table, int n, int total_tiles, void *stream);

/* The weight gradient's current plan for a shape (after any convgemm_tune_set
 * entry): tile width of its N side, pixel splits, and the largest useful split
 * count (the number of 64-pixel chunks).  Any pointer may be NULL. */
convgemm_status_t convgemm_wgrad_bf16_plan(const convgemm_shape_t *shape, int *bn, int *splits, int *max_splits);

/* Input gradient followed by the backward of the ReLU that produced the layer's
 * input x: dx = dgrad(dy, w) where x > 0, else 0 (x: the BF16 NHWC input of the
 * forward pass, [b][h][w][c]).  The masking is fused into the kernel's epilogue. */
convgemm_status_t convgemm_dgrad_bf16_relu(const convgemm_shape_t *shape, const void *dy, const void *wpacked, void *dx,
                                           const void *x, void *stream);

/* Input gradient with the reference's accumulate semantics: sconvGemmNHWC_back
 * adds into dx (beta = 1, src/convGemm.c:94-95; NCHW twin 142-143).  accumulate != 0:
 * dx = dx + dgrad(dy, w), the old BF16 value read in the epilogue and added in FP32
 * before one rounding; accumulate == 0: dx overwritten, as convgemm_dgrad_bf16.
 * relu_x (optional, as for convgemm_dgrad_bf16_relu): the result is then zeroed
 * where relu_x <= 0, after the sum.  dx must be 16-byte aligned when accumulating. */
convgemm_status_t convgemm_dgrad_bf16_ex(const convgemm_shape_t *shape, const void *dy, const void *wpacked, void *dx,
                                         const void *relu_x, int accumulate, void *stream);

/* Input gradient with the bias gradient of the previous layer fused into its epilogue (the
 * training step of a conv + bias + ReLU layer): dx as convgemm_dgrad_bf16_ex (relu_x masks it,
 * or NULL; overwritten), and db[ci] = sum over all pixels of the masked dx, taken from the
 * FP32 accumulators and reduced in a fixed order (bit-reproducible).  dx is the gradient at
 * the previous layer's pre-activation output, so db is that layer's bias gradient (the
 * reference has no bias gradient: its epilogue is inference-only, src/im2row_nhwc.c:269-285).
 * workspace: convgemm_dgrad_bf16_bias_grad_workspace_size bytes, 16-byte aligned.  Needs
 * c % 8 == 0. */
size_t convgemm_dgrad_bf16_bias_grad_workspace_size(const convgemm_shape_t *shape);
convgemm_status_t convgemm_dgrad_bf16_bias_grad(const convgemm_shape_t *shape, const void *dy, const void *wpacked,
                                                void *dx, const void *relu_x, float *db, void *workspace,
                                                size_t workspace_bytes, void *stream);

/* Bias gradient of the convolution: db[co] = sum over the b*ho*wo output pixels of
 * dy[p][co] (dy BF16 NHWC with kn rounded up to 8 channels, as for
 * convgemm_wgrad_bf16), FP32 in a fixed order (bit-reproducible). */
size_t convgemm_bias_grad_bf16_workspace_size(const convgemm_shape_t *shape);
convgemm_status_t convgemm_bias_grad_bf16(const convgemm_shape_t *shape, const void *dy, float *db, void *workspace,
                                          size_t workspace_bytes, void *stream);

/* ------------------------------------------ training-mode batch normalisation
 * The BF16 forward with batch statistics fused into its epilogue: y as
 * convgemm_fwd_bf16, and stats (FP64, device) = [0][kn] the sums and [1][kn] the
 * sums of squares over the b*ho*wo output pixels of z = conv * scale + shift (FP32,
 * before ReLU and BF16 rounding).  Partial sums per 32 pixels go to the workspace
 * and are reduced in a fixed order (bit-reproducible).  For a training step call it
 * with relu = 0 and scale / shift = NULL (or a bias as shift), fold the statistics
 * (convgemm_bn_stats_fold) and normalise (convgemm_bn_apply_bf16). */
size_t convgemm_fwd_bf16_stats_workspace_size(const convgemm_shape_t *shape);
convgemm_status_t convgemm_fwd_bf16_stats(const convgemm_shape_t *shape, const void *x, const void *wpacked, void *y,
                                          const float *scale, const float *shift, int relu, double *stats,
                                          void *workspace, size_t workspace_bytes, void *stream);
/* scale = gamma / sqrt(var + eps), shift = beta - mean * scale from the batch mean
 * = stats[0] / count and biased variance stats[1] / count - mean^2 (FP64); gamma /
 * beta NULL = 1 / 0; batch_mean / batch_var (FP32, optional) receive mean and var. */
convgemm_status_t convgemm_bn_stats_fold(int kn, const double *stats, long long count, const float *gamma,
                                         const float *beta, float eps, float *scale, float *shift, float *batch_mean,
                                         float *batch_var, void *stream);
/* y = relu?(z * scale + shift) per channel, BF16 NHWC [npix][kn] (kn % 8 == 0;
 * z == y allowed). */
convgemm_status_t convgemm_bn_apply_bf16(long long npix, int kn, const void *z, const float *scale,
                                         const float *shift, int relu, void *y, void *stream);

/* Workspace of convgemm_wgrad_bf16 in bytes: FP32 partial tiles of the pixel splits. */
size_t convgemm_wgrad_bf16_workspace_size(const convgemm_shape_t *shape);

/* Weight gradient, BF16 tensor cores, split over pixels with a fixed-order
 * reduction (bit-reproducible): generalises sconvGemmNHWC('T') (src/convGemm.c:71-76).
 * dy: BF16 NHWC [b][ho][wo][kn8]; x: BF16 NHWC [b][h][w][c8]; dw: FP32 in the
 * reference weight layout of `layout` (NHWC API [c][kh][kw][kn], NCHW API
 * [kn][c][kh][kw]), overwritten. */
convgemm_status_t convgemm_wgrad_bf16(convgemm_layout_t layout, const convgemm_shape_t *shape, const void *dy,
                                      const void *x, float *dw, void *workspace, size_t workspace_bytes,
                                      void *stream);

/* Weight gradient like convgemm_wgrad_bf16, for callers that cannot allocate GPU
 * memory (e.g. code running inside a CUDA-graph stream capture, where cudaMalloc
 * is not allowed, or services that fix their memory footprint at start-up): it
 * takes no workspace and calls no allocator.  No counterpart in the reference.
 * Its split partials live in one file-scope device array of 16 MiB (4 Mi FP32
 * values) that every GPU loading the library keeps until exit; layers with
 * kh*kw*c8*kn above that are rejected with CONVGEMM_ERROR_NOT_SUPPORTED.  All
 * calls share the array, so calls that overlap on the GPU race.  The first call
 * on a device looks up the array's address; make it before any stream capture.
 * The same shape checks as convgemm_wgrad_bf16 apply (filters up to 49 taps); a
 * device-side wait that runs out is reported by convgemm_check_device. */
convgemm_status_t convgemm_wgrad_bf16_noalloc(convgemm_layout_t layout, const convgemm_shape_t *shape,
                                              const void *dy, const void *x, float *dw, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* CONVGEMM_GPU_H */
