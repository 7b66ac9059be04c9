/* The reference's explicit lowering helpers, on the GPU (FP32, drop-in names and
 * signatures).  Each replaces the function of the same name in the reference:
 *   im2row_nhwc, row2im_nhwc     src/im2row_nhwc.h:20-29 (bodies im2row_nhwc.c:147-229)
 *   im2col_nchw, transpose_nchw,
 *   col2im_nchw                  src/im2col_nchw.h:20-38 (bodies im2col_nchw.c:146-233, 337-359)
 * Pointers may be device or host memory (host buffers are staged through the GPU
 * and the call returns with the results in host memory).  As in the reference,
 * im2row / im2col leave the entries of padding taps untouched, row2im / col2im
 * accumulate into out (here in the reference's summation order, without atomics),
 * and ld / m / n do not change the lowered layout (rows of c*kh*kw, columns of
 * b*ho*wo), except ld of transpose_nchw.  Errors go to convgemm_get_last_error(). */
#ifndef CONVGEMM_HELPERS_H
#define CONVGEMM_HELPERS_H

#ifdef __cplusplus
extern "C" {
#endif

void im2row_nhwc(float *rows, int ld, const float *in, int batches, int height, int width, int channels,
                 int oheight, int owidth, int kheight, int kwidth, int vpadding, int hpadding,
                 int vstride, int hstride, int vdilation, int hdilation);

void row2im_nhwc(int m, int n, const float *rows, int ld, float *out, int batches, int height, int width, int channels,
                 int oheight, int owidth, int kheight, int kwidth, int vpadding, int hpadding,
                 int vstride, int hstride, int vdilation, int hdilation);

void im2col_nchw(float *cols, int ld, const float *in, int batches, int channels, int height, int width, int oheight,
                 int owidth, int kheight, int kwidth, int vpadding, int hpadding, int vstride, int hstride,
                 int vdilation, int hdilation);

void transpose_nchw(int rows, int cols, const float *in, int ld, float beta, float *out, int kn, int ho, int wo,
                    int start_row, int start_col);

void col2im_nchw(int m, int n, const float *cols, int ld, float *out, int batches, int channels, int height, int width,
                 int oheight, int owidth, int kheight, int kwidth, int vpadding, int hpadding, int vstride, int hstride,
                 int vdilation, int hdilation);

#ifdef __cplusplus
}
#endif

#endif
