/*
 * FP64 direct-convolution oracle.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the library links or calls this file;
 * tests/, the smoke check and bench.py's CPU-baseline leg use it as the checker.
 *
 * It restates, as plain loops in double precision, what convGemm's five entry
 * points compute (the index semantics come from the reference's explicit
 * lowering helpers):
 *   - K index  k = (c*kh + kx)*kw + ky        (src/im2row_nhwc.c:163, src/im2col_nchw.c:155)
 *   - P index  p = (b*ho + x)*wo + y          (src/im2row_nhwc.c:155)
 *   - input row ix = vstride*x + vdilation*kx - vpadding, column
 *     iy = hstride*y + hdilation*ky - hpadding; taps outside the image are 0
 *     (src/im2row_nhwc.c:53-58)
 *   - ho = (h + 2*vpad - vdil*(kh-1) - 1)/vstride + 1   (src/convGemm.c:60-61)
 *   - NHWC weights are [c][kh][kw][kn] (ld = kn, src/convGemm.c:66),
 *     NCHW weights are [kn][c][kh][kw] (ld = K, src/convGemm.c:117)
 *   - epilogue: +bias, then (v - mean)*inv_std*gamma + beta, then ReLU,
 *     per output channel (src/im2row_nhwc.c:269-285, src/im2col_nchw.c:424-431)
 *
 * Every routine accumulates in double and writes double results, so the
 * FP32 and BF16/FP8 paths can be measured against it.
 */
#include <stdint.h>
#include <stddef.h>
#include <string.h>
#include <math.h>

#define LAYOUT_NHWC 0
#define LAYOUT_NCHW 1

typedef struct {
    int b, h, w, c, kn, kh, kw;
    int vpad, hpad, vstr, hstr, vdil, hdil;
    int ho, wo;
} odesc;

static odesc make_desc(int b, int h, int w, int c, int kn, int kh, int kw, int vpad, int hpad,
                       int vstr, int hstr, int vdil, int hdil) {
    odesc d = {b, h, w, c, kn, kh, kw, vpad, hpad, vstr, hstr, vdil, hdil, 0, 0};
    d.ho = (h + 2 * vpad - vdil * (kh - 1) - 1) / vstr + 1;
    d.wo = (w + 2 * hpad - hdil * (kw - 1) - 1) / hstr + 1;
    return d;
}

static inline size_t x_index(int layout, const odesc *d, int b, int ix, int iy, int c) {
    if (layout == LAYOUT_NHWC) return (((size_t) b * d->h + ix) * d->w + iy) * d->c + c;
    return (((size_t) b * d->c + c) * d->h + ix) * d->w + iy;
}

static inline size_t y_index(int layout, const odesc *d, int b, int x, int y, int n) {
    if (layout == LAYOUT_NHWC) return (((size_t) b * d->ho + x) * d->wo + y) * d->kn + n;
    return (((size_t) b * d->kn + n) * d->ho + x) * d->wo + y;
}

/* weight element for (input channel c, tap kx, ky, output channel n) */
static inline size_t w_index(int layout, const odesc *d, int c, int kx, int ky, int n) {
    size_t k = ((size_t) c * d->kh + kx) * d->kw + ky;
    if (layout == LAYOUT_NHWC) return k * d->kn + n;
    return (size_t) n * ((size_t) d->c * d->kh * d->kw) + k;
}

static double fwd_point(int layout, const odesc *d, const float *wts, const float *x,
                        int b, int ox, int oy, int n) {
    double acc = 0.0;
    for (int c = 0; c < d->c; c++)
        for (int kx = 0; kx < d->kh; kx++) {
            int ix = d->vstr * ox + d->vdil * kx - d->vpad;
            if (ix < 0 || ix >= d->h) continue;
            for (int ky = 0; ky < d->kw; ky++) {
                int iy = d->hstr * oy + d->hdil * ky - d->hpad;
                if (iy < 0 || iy >= d->w) continue;
                acc += (double) x[x_index(layout, d, b, ix, iy, c)] *
                       (double) wts[w_index(layout, d, c, kx, ky, n)];
            }
        }
    return acc;
}

static double apply_epilogue(double v, int n, const float *bias, const float *mean, const float *inv_std,
                             const float *gamma, const float *beta, int relu) {
    if (bias) v += (double) bias[n];
    if (mean) v = (v - (double) mean[n]) * (double) inv_std[n] * (double) gamma[n] + (double) beta[n];
    if (relu && v < 0.0) v = 0.0;
    return v;
}

/* Forward convolution (+ optional epilogue) for every output element.
 * y has the output layout of `layout` (NHWC [b][ho][wo][kn] or NCHW [b][kn][ho][wo]). */
void oracle_fwd_f64(int layout, int b, int h, int w, int c, int kn, int kh, int kw,
                    int vpad, int hpad, int vstr, int hstr, int vdil, int hdil,
                    const float *wts, const float *x, double *y,
                    const float *bias, const float *mean, const float *inv_std,
                    const float *gamma, const float *beta, int relu) {
    odesc d = make_desc(b, h, w, c, kn, kh, kw, vpad, hpad, vstr, hstr, vdil, hdil);
    const int64_t total = (int64_t) b * d.ho * d.wo;
    #pragma omp parallel for schedule(static)
    for (int64_t p = 0; p < total; p++) {
        int oy = (int) (p % d.wo), ox = (int) ((p / d.wo) % d.ho), bb = (int) (p / ((int64_t) d.wo * d.ho));
        for (int n = 0; n < kn; n++) {
            double v = fwd_point(layout, &d, wts, x, bb, ox, oy, n);
            y[y_index(layout, &d, bb, ox, oy, n)] = apply_epilogue(v, n, bias, mean, inv_std, gamma, beta, relu);
        }
    }
}

/* Forward convolution at selected flat output indices (in the output layout). */
void oracle_fwd_points_f64(int layout, int b, int h, int w, int c, int kn, int kh, int kw,
                           int vpad, int hpad, int vstr, int hstr, int vdil, int hdil,
                           const float *wts, const float *x, const int64_t *idx, int64_t npts, double *out,
                           const float *bias, const float *mean, const float *inv_std,
                           const float *gamma, const float *beta, int relu) {
    odesc d = make_desc(b, h, w, c, kn, kh, kw, vpad, hpad, vstr, hstr, vdil, hdil);
    #pragma omp parallel for schedule(dynamic, 16)
    for (int64_t t = 0; t < npts; t++) {
        int64_t i = idx[t];
        int bb, ox, oy, n;
        if (layout == LAYOUT_NHWC) {
            n = (int) (i % kn); i /= kn;
            oy = (int) (i % d.wo); i /= d.wo;
            ox = (int) (i % d.ho); bb = (int) (i / d.ho);
        } else {
            oy = (int) (i % d.wo); i /= d.wo;
            ox = (int) (i % d.ho); i /= d.ho;
            n = (int) (i % kn); bb = (int) (i / kn);
        }
        double v = fwd_point(layout, &d, wts, x, bb, ox, oy, n);
        out[t] = apply_epilogue(v, n, bias, mean, inv_std, gamma, beta, relu);
    }
}

static double wgrad_point(int layout, const odesc *d, const float *dy, const float *x,
                          int c, int kx, int ky, int n) {
    double acc = 0.0;
    for (int b = 0; b < d->b; b++)
        for (int ox = 0; ox < d->ho; ox++) {
            int ix = d->vstr * ox + d->vdil * kx - d->vpad;
            if (ix < 0 || ix >= d->h) continue;
            for (int oy = 0; oy < d->wo; oy++) {
                int iy = d->hstr * oy + d->hdil * ky - d->hpad;
                if (iy < 0 || iy >= d->w) continue;
                acc += (double) dy[y_index(layout, d, b, ox, oy, n)] * (double) x[x_index(layout, d, b, ix, iy, c)];
            }
        }
    return acc;
}

/* Weight gradient: dw has the weight layout of `layout`. */
void oracle_wgrad_f64(int layout, int b, int h, int w, int c, int kn, int kh, int kw,
                      int vpad, int hpad, int vstr, int hstr, int vdil, int hdil,
                      const float *dy, const float *x, double *dw) {
    odesc d = make_desc(b, h, w, c, kn, kh, kw, vpad, hpad, vstr, hstr, vdil, hdil);
    const int64_t total = (int64_t) c * kh * kw * kn;
    #pragma omp parallel for schedule(dynamic, 4)
    for (int64_t t = 0; t < total; t++) {
        int n = (int) (t % kn);
        int64_t k = t / kn;
        int ky = (int) (k % kw), kx = (int) ((k / kw) % kh), cc = (int) (k / ((int64_t) kw * kh));
        dw[w_index(layout, &d, cc, kx, ky, n)] = wgrad_point(layout, &d, dy, x, cc, kx, ky, n);
    }
}

static double dgrad_point(int layout, const odesc *d, const float *wts, const float *dy,
                          int b, int ix, int iy, int c) {
    double acc = 0.0;
    for (int kx = 0; kx < d->kh; kx++) {
        int tx = ix + d->vpad - d->vdil * kx;
        if (tx < 0 || tx % d->vstr) continue;
        int ox = tx / d->vstr;
        if (ox >= d->ho) continue;
        for (int ky = 0; ky < d->kw; ky++) {
            int ty = iy + d->hpad - d->hdil * ky;
            if (ty < 0 || ty % d->hstr) continue;
            int oy = ty / d->hstr;
            if (oy >= d->wo) continue;
            for (int n = 0; n < d->kn; n++)
                acc += (double) wts[w_index(layout, d, c, kx, ky, n)] * (double) dy[y_index(layout, d, b, ox, oy, n)];
        }
    }
    return acc;
}

/* Input gradient (the col2im/row2im of W^T*dY, written in gather form):
 * dx (input layout of `layout`) receives the gradient; it is NOT accumulated
 * into existing contents. */
void oracle_dgrad_f64(int layout, int b, int h, int w, int c, int kn, int kh, int kw,
                      int vpad, int hpad, int vstr, int hstr, int vdil, int hdil,
                      const float *wts, const float *dy, double *dx) {
    odesc d = make_desc(b, h, w, c, kn, kh, kw, vpad, hpad, vstr, hstr, vdil, hdil);
    const int64_t total = (int64_t) b * h * w;
    #pragma omp parallel for schedule(static)
    for (int64_t p = 0; p < total; p++) {
        int iy = (int) (p % w), ix = (int) ((p / w) % h), bb = (int) (p / ((int64_t) w * h));
        for (int cc = 0; cc < c; cc++)
            dx[x_index(layout, &d, bb, ix, iy, cc)] = dgrad_point(layout, &d, wts, dy, bb, ix, iy, cc);
    }
}

/* Input gradient at selected flat input indices (input layout). */
void oracle_dgrad_points_f64(int layout, int b, int h, int w, int c, int kn, int kh, int kw,
                             int vpad, int hpad, int vstr, int hstr, int vdil, int hdil,
                             const float *wts, const float *dy, const int64_t *idx, int64_t npts, double *out) {
    odesc d = make_desc(b, h, w, c, kn, kh, kw, vpad, hpad, vstr, hstr, vdil, hdil);
    #pragma omp parallel for schedule(dynamic, 16)
    for (int64_t t = 0; t < npts; t++) {
        int64_t i = idx[t];
        int bb, ix, iy, cc;
        if (layout == LAYOUT_NHWC) {
            cc = (int) (i % c); i /= c;
            iy = (int) (i % w); i /= w;
            ix = (int) (i % h); bb = (int) (i / h);
        } else {
            iy = (int) (i % w); i /= w;
            ix = (int) (i % h); i /= h;
            cc = (int) (i % c); bb = (int) (i / c);
        }
        out[t] = dgrad_point(layout, &d, wts, dy, bb, ix, iy, cc);
    }
}

/* Weight gradient at selected flat weight indices (weight layout). */
void oracle_wgrad_points_f64(int layout, int b, int h, int w, int c, int kn, int kh, int kw,
                             int vpad, int hpad, int vstr, int hstr, int vdil, int hdil,
                             const float *dy, const float *x, const int64_t *idx, int64_t npts, double *out) {
    odesc d = make_desc(b, h, w, c, kn, kh, kw, vpad, hpad, vstr, hstr, vdil, hdil);
    const int64_t K = (int64_t) c * kh * kw;
    #pragma omp parallel for schedule(dynamic, 1)
    for (int64_t t = 0; t < npts; t++) {
        int64_t i = idx[t], k;
        int n;
        if (layout == LAYOUT_NHWC) { n = (int) (i % kn); k = i / kn; }
        else { k = i % K; n = (int) (i / K); }
        int ky = (int) (k % kw), kx = (int) ((k / kw) % kh), cc = (int) (k / ((int64_t) kw * kh));
        out[t] = wgrad_point(layout, &d, dy, x, cc, kx, ky, n);
    }
}

/* Batch-norm fold in double: scale = gamma*inv_std, shift = beta + (bias - mean)*scale
 * (bias and mean may be NULL).  y = acc*scale + shift reproduces the epilogue above. */
void oracle_bn_fold_f64(int kn, const float *bias, const float *mean, const float *inv_std,
                        const float *gamma, const float *beta, double *scale, double *shift) {
    for (int n = 0; n < kn; n++) {
        double s = 1.0, t = bias ? (double) bias[n] : 0.0;
        if (mean) {
            s = (double) gamma[n] * (double) inv_std[n];
            t = (double) beta[n] + (t - (double) mean[n]) * s;
        }
        scale[n] = s;
        shift[n] = t;
    }
}

/* Explicit im2row lowering (NHWC) into rows[P][K], zero for padding taps:
 * the materialised matrix the reference's tests build (src/im2row_nhwc.c:147-169). */
void oracle_im2row_nhwc(float *rows, const float *in, int b, int h, int w, int c, int kh, int kw,
                        int vpad, int hpad, int vstr, int hstr, int vdil, int hdil) {
    odesc d = make_desc(b, h, w, c, 1, kh, kw, vpad, hpad, vstr, hstr, vdil, hdil);
    const int64_t K = (int64_t) c * kh * kw, P = (int64_t) b * d.ho * d.wo;
    #pragma omp parallel for schedule(static)
    for (int64_t p = 0; p < P; p++) {
        int oy = (int) (p % d.wo), ox = (int) ((p / d.wo) % d.ho), bb = (int) (p / ((int64_t) d.wo * d.ho));
        for (int cc = 0; cc < c; cc++)
            for (int kx = 0; kx < kh; kx++)
                for (int ky = 0; ky < kw; ky++) {
                    int ix = vstr * ox + vdil * kx - vpad, iy = hstr * oy + hdil * ky - hpad;
                    int64_t k = ((int64_t) cc * kh + kx) * kw + ky;
                    rows[p * K + k] = (ix >= 0 && ix < h && iy >= 0 && iy < w)
                                      ? in[x_index(LAYOUT_NHWC, &d, bb, ix, iy, cc)] : 0.0f;
                }
    }
}

/* Explicit im2col lowering (NCHW) into cols[K][P] (src/im2col_nchw.c:146-169). */
void oracle_im2col_nchw(float *cols, const float *in, int b, int c, int h, int w, int kh, int kw,
                        int vpad, int hpad, int vstr, int hstr, int vdil, int hdil) {
    odesc d = make_desc(b, h, w, c, 1, kh, kw, vpad, hpad, vstr, hstr, vdil, hdil);
    const int64_t K = (int64_t) c * kh * kw, P = (int64_t) b * d.ho * d.wo;
    #pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < K; k++) {
        int ky = (int) (k % kw), kx = (int) ((k / kw) % kh), cc = (int) (k / ((int64_t) kw * kh));
        for (int64_t p = 0; p < P; p++) {
            int oy = (int) (p % d.wo), ox = (int) ((p / d.wo) % d.ho), bb = (int) (p / ((int64_t) d.wo * d.ho));
            int ix = vstr * ox + vdil * kx - vpad, iy = hstr * oy + hdil * ky - hpad;
            cols[k * P + p] = (ix >= 0 && ix < h && iy >= 0 && iy < w)
                              ? in[x_index(LAYOUT_NCHW, &d, bb, ix, iy, cc)] : 0.0f;
        }
    }
}
