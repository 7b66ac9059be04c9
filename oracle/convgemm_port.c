/*
 * FP32 CPU restatement of convGemm's arithmetic, in the reference's own
 * summation order.
 *
 * TEST INFRASTRUCTURE ONLY: tests/ use it as a checker and bench.py times it as
 * the CPU baseline on hosts where the reference's sources are not present.
 *
 * What "the reference's order" means (src/gemm_blis_B3A2C0_orig.c:55-64,
 * src/gemm_blis_B3A2C0.c:58-64): the reduction dimension is cut into blocks
 * of KC = 384 (slides/slides.tex:158-160); each block is one fused
 * multiply-add chain per output element, in increasing k, starting from +0
 * (the BLIS micro-kernel, gemm_blis.h:65-76); blocks are added to the running
 * result in increasing order (betaI = beta on the first block and 1 after,
 * B3A2C0_orig.c:64; sxpbyM, gemm_blis.c:147-161).  The epilogue runs on the
 * last block only: t = block + running (if any), t += bias,
 * t = (t - mean)*inv_std, t = t*gamma + beta (fused, as gcc contracts it at
 * -Ofast), ReLU (src/im2row_nhwc.c:269-285, src/im2col_nchw.c:419-432).
 *
 * Forward and weight-gradient results therefore match the reference bit for
 * bit.  The input gradient is a scatter with `omp atomic` in the reference
 * (src/im2row_nhwc.c:252, src/im2col_nchw.c:381), whose order is not
 * deterministic; the restatement below scatters in a fixed order.
 */
#include <stdint.h>
#include <stdlib.h>
#include <stdbool.h>
#include <string.h>
#include <math.h>

#define CG_KC 384
#define FWD_PT 4      /* pixels per register block */
#define FWD_NB 64     /* output channels per register block */
#define WG_KG 4       /* K indices per weight-gradient pass */

typedef struct {
    int b, h, w, c, kn, kh, kw;
    int vpad, hpad, vstr, hstr, vdil, hdil;
    int ho, wo;
} pdesc;

typedef struct {
    const float *bias, *mean, *inv_std, *gamma, *beta;
    bool relu;
    bool any;
} pepi;

static pdesc mkdesc(int b, int h, int w, int c, int kn, int kh, int kw, int vpad, int hpad,
                    int vstr, int hstr, int vdil, int hdil) {
    pdesc d = {b, h, w, c, kn, kh, kw, vpad, hpad, vstr, hstr, vdil, hdil, 0, 0};
    d.ho = (h + 2 * vpad - vdil * (kh - 1) - 1) / vstr + 1;
    d.wo = (w + 2 * hpad - hdil * (kw - 1) - 1) / hstr + 1;
    return d;
}

/* im2row/im2col element X(p, k) of the input, 0 for padding taps. */
static inline float xval(const pdesc *d, int nchw, const float *x, int b, int ox, int oy, int k) {
    int ky = k % d->kw, kx = (k / d->kw) % d->kh, c = k / (d->kw * d->kh);
    int ix = d->vstr * ox + d->vdil * kx - d->vpad;
    int iy = d->hstr * oy + d->hdil * ky - d->hpad;
    if (ix < 0 || ix >= d->h || iy < 0 || iy >= d->w) return 0.0f;
    if (nchw) return x[(((size_t) b * d->c + c) * d->h + ix) * d->w + iy];
    return x[(((size_t) b * d->h + ix) * d->w + iy) * d->c + c];
}

static inline float epilogue(float t, int n, const pepi *e) {
    if (e->bias) t = t + e->bias[n];
    if (e->mean) {
        t = (t - e->mean[n]) * e->inv_std[n];
        t = fmaf(t, e->gamma[n], e->beta[n]);
    }
    if (e->relu && t < 0.0f) t = 0.0f;
    return t;
}

/* y(p, n) = epi( sum_k X(p,k) * wt[k][n] ), wt row-major [K][kn]. */
static void fwd_core(const pdesc *d, int nchw, const float *wt, const float *x, float *y, const pepi *e) {
    const int K = d->c * d->kh * d->kw, kn = d->kn;
    const int64_t P = (int64_t) d->b * d->ho * d->wo;
    #pragma omp parallel
    {
        float *xcol = (float *) malloc(sizeof(float) * FWD_PT * (size_t) K);
        float S[FWD_PT][FWD_NB], blk[FWD_PT][FWD_NB];
        #pragma omp for schedule(dynamic, 4)
        for (int64_t p0 = 0; p0 < P; p0 += FWD_PT) {
            int pt = (P - p0 < FWD_PT) ? (int) (P - p0) : FWD_PT;
            int bs[FWD_PT], oxs[FWD_PT], oys[FWD_PT];
            for (int t = 0; t < pt; t++) {
                int64_t p = p0 + t;
                oys[t] = (int) (p % d->wo);
                oxs[t] = (int) ((p / d->wo) % d->ho);
                bs[t] = (int) (p / ((int64_t) d->wo * d->ho));
                for (int k = 0; k < K; k++) xcol[(size_t) t * K + k] = xval(d, nchw, x, bs[t], oxs[t], oys[t], k);
            }
            for (int n0 = 0; n0 < kn; n0 += FWD_NB) {
                int nb = (kn - n0 < FWD_NB) ? kn - n0 : FWD_NB;
                for (int pc = 0; pc < K; pc += CG_KC) {
                    int kc = (K - pc < CG_KC) ? K - pc : CG_KC;
                    for (int t = 0; t < FWD_PT; t++)
                        for (int n = 0; n < FWD_NB; n++) blk[t][n] = 0.0f;
                    for (int k = pc; k < pc + kc; k++) {
                        const float *wr = wt + (size_t) k * kn + n0;
                        for (int t = 0; t < pt; t++) {
                            const float xv = xcol[(size_t) t * K + k];
                            for (int n = 0; n < nb; n++) blk[t][n] = fmaf(xv, wr[n], blk[t][n]);
                        }
                    }
                    for (int t = 0; t < pt; t++)
                        for (int n = 0; n < nb; n++) S[t][n] = (pc == 0) ? blk[t][n] : blk[t][n] + S[t][n];
                }
                for (int t = 0; t < pt; t++) {
                    for (int n = 0; n < nb; n++) {
                        float v = e->any ? epilogue(S[t][n], n0 + n, e) : S[t][n];
                        size_t o = nchw ? ((((size_t) bs[t] * kn + n0 + n) * d->ho + oxs[t]) * d->wo + oys[t])
                                        : ((size_t) (p0 + t) * kn + n0 + n);
                        y[o] = v;
                    }
                }
            }
        }
        free(xcol);
    }
}

/* dW(k, n) = sum_p X(p,k) * dyt[p][n], dyt row-major [P][kn]; stored by layout. */
static void wgrad_core(const pdesc *d, int nchw, const float *dyt, const float *x, float *dw) {
    const int K = d->c * d->kh * d->kw, kn = d->kn;
    const int64_t P = (int64_t) d->b * d->ho * d->wo;
    #pragma omp parallel
    {
        float *S = (float *) malloc(sizeof(float) * WG_KG * (size_t) kn);
        float *blk = (float *) malloc(sizeof(float) * WG_KG * (size_t) kn);
        #pragma omp for schedule(dynamic, 1)
        for (int k0 = 0; k0 < K; k0 += WG_KG) {
            int kg = (K - k0 < WG_KG) ? K - k0 : WG_KG;
            for (int64_t pc = 0; pc < P; pc += CG_KC) {
                int64_t kc = (P - pc < CG_KC) ? P - pc : CG_KC;
                memset(blk, 0, sizeof(float) * WG_KG * (size_t) kn);
                for (int64_t p = pc; p < pc + kc; p++) {
                    int oy = (int) (p % d->wo), ox = (int) ((p / d->wo) % d->ho), b = (int) (p / ((int64_t) d->wo * d->ho));
                    const float *dr = dyt + (size_t) p * kn;
                    for (int g = 0; g < kg; g++) {
                        const float xv = xval(d, nchw, x, b, ox, oy, k0 + g);
                        float *br = blk + (size_t) g * kn;
                        for (int n = 0; n < kn; n++) br[n] = fmaf(dr[n], xv, br[n]);
                    }
                }
                for (int g = 0; g < kg; g++)
                    for (int n = 0; n < kn; n++)
                        S[(size_t) g * kn + n] = (pc == 0) ? blk[(size_t) g * kn + n]
                                                           : S[(size_t) g * kn + n] + blk[(size_t) g * kn + n];
            }
            for (int g = 0; g < kg; g++)
                for (int n = 0; n < kn; n++) {
                    size_t o = nchw ? ((size_t) n * K + k0 + g) : ((size_t) (k0 + g) * kn + n);
                    dw[o] = S[(size_t) g * kn + n];
                }
        }
        free(S);
        free(blk);
    }
}

/* dx += scatter_k( sum_l dyt[p][l] * wt[l][k] ), one KC block of l at a time.
 * Parallel over (image, input-channel chunk): the scatter targets of two
 * tasks never overlap, so no atomics are needed and the order is fixed. */
static void dgrad_core(const pdesc *d, int nchw, const float *wt, const float *dyt, float *dx) {
    const int K = d->c * d->kh * d->kw, kn = d->kn, T = d->kh * d->kw;
    const int cchunk = d->c < 8 ? 1 : 8;
    const int nchunks = (d->c + cchunk - 1) / cchunk;
    #pragma omp parallel
    {
        float *blk = (float *) malloc(sizeof(float) * (size_t) cchunk * T);
        #pragma omp for schedule(dynamic, 1) collapse(2)
        for (int b = 0; b < d->b; b++)
            for (int cc = 0; cc < nchunks; cc++) {
                const int c0 = cc * cchunk, c1 = (c0 + cchunk < d->c) ? c0 + cchunk : d->c;
                const int k0 = c0 * T, nk = (c1 - c0) * T;
                for (int ox = 0; ox < d->ho; ox++)
                    for (int oy = 0; oy < d->wo; oy++) {
                        int64_t p = ((int64_t) b * d->ho + ox) * d->wo + oy;
                        const float *dr = dyt + (size_t) p * kn;
                        for (int pc = 0; pc < kn; pc += CG_KC) {
                            int kc = (kn - pc < CG_KC) ? kn - pc : CG_KC;
                            for (int k = 0; k < nk; k++) blk[k] = 0.0f;
                            for (int l = pc; l < pc + kc; l++) {
                                const float dv = dr[l];
                                const float *wr = wt + (size_t) l * K + k0;
                                for (int k = 0; k < nk; k++) blk[k] = fmaf(wr[k], dv, blk[k]);
                            }
                            for (int kk = 0; kk < nk; kk++) {
                                int k = k0 + kk;
                                int ky = k % d->kw, kx = (k / d->kw) % d->kh, c = k / (d->kw * d->kh);
                                int ix = d->vstr * ox + d->vdil * kx - d->vpad;
                                int iy = d->hstr * oy + d->hdil * ky - d->hpad;
                                if (ix < 0 || ix >= d->h || iy < 0 || iy >= d->w) continue;
                                size_t o = nchw ? ((((size_t) b * d->c + c) * d->h + ix) * d->w + iy)
                                                : ((((size_t) b * d->h + ix) * d->w + iy) * d->c + c);
                                dx[o] += blk[kk];
                            }
                        }
                    }
            }
        free(blk);
    }
}

/* [rows][cols] -> [cols][rows] */
static float *transpose_copy(const float *a, int64_t rows, int64_t cols) {
    float *t = (float *) malloc(sizeof(float) * (size_t) (rows * cols));
    #pragma omp parallel for schedule(static)
    for (int64_t r = 0; r < rows; r++)
        for (int64_t c = 0; c < cols; c++) t[c * rows + r] = a[r * cols + c];
    return t;
}

/* NCHW dY [b][kn][ho][wo] -> [P][kn] */
static float *nchw_to_pk(const pdesc *d, const float *dy) {
    const int64_t hw = (int64_t) d->ho * d->wo;
    float *t = (float *) malloc(sizeof(float) * (size_t) ((int64_t) d->b * hw * d->kn));
    #pragma omp parallel for schedule(static)
    for (int b = 0; b < d->b; b++)
        for (int n = 0; n < d->kn; n++)
            for (int64_t q = 0; q < hw; q++)
                t[((int64_t) b * hw + q) * d->kn + n] = dy[((int64_t) b * d->kn + n) * hw + q];
    return t;
}

/* ---- entry points with the reference's signatures (src/convGemm.h:20-64) ---- */

int port_alloc_pack_buffs(float **Ac_pack, float **Bc_pack) {
    *Ac_pack = NULL;
    *Bc_pack = NULL;
    return 0;
}

void port_sconvGemmNHWC(char trans, int b, int h, int w, int c, int kn, int kh, int kw,
                        int vpadding, int hpadding, int vstride, int hstride, int vdilation, int hdilation,
                        const float *in, const float *x, float *out, const float *bias_vector,
                        const float *bn_running_mean, const float *bn_inv_std,
                        const float *bn_gamma, const float *bn_beta, bool relu,
                        float *ac_pack, float *bc_pack) {
    (void) ac_pack;
    (void) bc_pack;
    pdesc d = mkdesc(b, h, w, c, kn, kh, kw, vpadding, hpadding, vstride, hstride, vdilation, hdilation);
    if (trans == 'N') {
        pepi e = {bias_vector, bn_running_mean, bn_inv_std, bn_gamma, bn_beta, relu,
                  bias_vector != NULL || bn_running_mean != NULL || relu};
        fwd_core(&d, 0, in, x, out, &e);
    } else {
        wgrad_core(&d, 0, in, x, out);
    }
}

void port_sconvGemmNHWC_back(int b, int h, int w, int c, int kn, int kh, int kw,
                             int vstride, int hstride, int vpadding, int hpadding, int vdilation, int hdilation,
                             const float *weights, const float *dy, float *dx, float *ac_pack, float *bc_pack) {
    (void) ac_pack;
    (void) bc_pack;
    pdesc d = mkdesc(b, h, w, c, kn, kh, kw, vpadding, hpadding, vstride, hstride, vdilation, hdilation);
    float *wt = transpose_copy(weights, (int64_t) c * kh * kw, kn);   /* [K][kn] -> [kn][K] */
    dgrad_core(&d, 0, wt, dy, dx);
    free(wt);
}

void port_sconvGemmNCHW(char trans, int b, int c, int h, int w, int kn, int kh, int kw,
                        int vpadding, int hpadding, int vstride, int hstride, int vdilation, int hdilation,
                        const float *in, const float *x, float *out, const float *bias_vector,
                        const float *bn_running_mean, const float *bn_inv_std,
                        const float *bn_gamma, const float *bn_beta, bool relu,
                        float *ac_pack, float *bc_pack) {
    (void) ac_pack;
    (void) bc_pack;
    pdesc d = mkdesc(b, h, w, c, kn, kh, kw, vpadding, hpadding, vstride, hstride, vdilation, hdilation);
    if (trans == 'N') {
        pepi e = {bias_vector, bn_running_mean, bn_inv_std, bn_gamma, bn_beta, relu, true};
        float *wt = transpose_copy(in, kn, (int64_t) c * kh * kw);      /* [kn][K] -> [K][kn] */
        fwd_core(&d, 1, wt, x, out, &e);
        free(wt);
    } else {
        float *dyt = nchw_to_pk(&d, in);
        wgrad_core(&d, 1, dyt, x, out);
        free(dyt);
    }
}

void port_sconvGemmNCHW_back(int b, int c, int h, int w, int kn, int kh, int kw,
                             int vstride, int hstride, int vpadding, int hpadding, int vdilation, int hdilation,
                             const float *weights, const float *dy, float *dx, float *ac_pack, float *bc_pack) {
    (void) ac_pack;
    (void) bc_pack;
    pdesc d = mkdesc(b, h, w, c, kn, kh, kw, vpadding, hpadding, vstride, hstride, vdilation, hdilation);
    float *dyt = nchw_to_pk(&d, dy);
    dgrad_core(&d, 1, weights, dyt, dx);   /* OIHW weights are already [kn][K] */
    free(dyt);
}

/* ---- sampled points of the port, in the same per-element arithmetic ----
 * For layers too large to restate whole in a test: out[i] is the port's value of
 * output element idx[i] (the forward's y, or the weight gradient's dW, indexed as
 * the reference lays them out for `layout`), computed with the same KC = 384
 * blocked FMA chains, block sums and epilogue as fwd_core / wgrad_core above, so
 * each equals the corresponding element of port_sconvGemm{NHWC,NCHW} bit for bit.
 * Weights are in the reference layout of `layout` ([c][kh][kw][kn] / [kn][c][kh][kw]);
 * dy is NHWC [b][ho][wo][kn] or NCHW [b][kn][ho][wo]. */
void port_fwd_points(int layout, int b, int h, int w, int c, int kn, int kh, int kw, int vpad, int hpad,
                     int vstr, int hstr, int vdil, int hdil, const float *wts, const float *x,
                     const int64_t *idx, int64_t n, float *out, const float *bias, const float *mean,
                     const float *inv_std, const float *gamma, const float *beta, int relu) {
    pdesc d = mkdesc(b, h, w, c, kn, kh, kw, vpad, hpad, vstr, hstr, vdil, hdil);
    const int nchw = layout == 1;
    const int K = c * kh * kw;
    pepi e = {bias, mean, inv_std, gamma, beta, relu != 0, nchw || bias != NULL || mean != NULL || relu};
    #pragma omp parallel for schedule(dynamic, 16)
    for (int64_t i = 0; i < n; i++) {
        int64_t o = idx[i];
        int bb, ox, oy, co;
        if (nchw) {
            oy = (int) (o % d.wo); ox = (int) ((o / d.wo) % d.ho);
            co = (int) ((o / ((int64_t) d.wo * d.ho)) % kn); bb = (int) (o / ((int64_t) d.wo * d.ho * kn));
        } else {
            co = (int) (o % kn); oy = (int) ((o / kn) % d.wo);
            ox = (int) ((o / ((int64_t) kn * d.wo)) % d.ho); bb = (int) (o / ((int64_t) kn * d.wo * d.ho));
        }
        float S = 0.0f;
        for (int pc = 0; pc < K; pc += CG_KC) {
            int kc = (K - pc < CG_KC) ? K - pc : CG_KC;
            float blk = 0.0f;
            for (int k = pc; k < pc + kc; k++) {
                const float wv = nchw ? wts[(size_t) co * K + k] : wts[(size_t) k * kn + co];
                blk = fmaf(xval(&d, nchw, x, bb, ox, oy, k), wv, blk);
            }
            S = (pc == 0) ? blk : blk + S;
        }
        out[i] = e.any ? epilogue(S, co, &e) : S;
    }
}

void port_wgrad_points(int layout, int b, int h, int w, int c, int kn, int kh, int kw, int vpad, int hpad,
                       int vstr, int hstr, int vdil, int hdil, const float *dy, const float *x,
                       const int64_t *idx, int64_t n, float *out) {
    pdesc d = mkdesc(b, h, w, c, kn, kh, kw, vpad, hpad, vstr, hstr, vdil, hdil);
    const int nchw = layout == 1;
    const int K = c * kh * kw;
    const int64_t P = (int64_t) d.b * d.ho * d.wo, hw = (int64_t) d.ho * d.wo;
    #pragma omp parallel for schedule(dynamic, 1)
    for (int64_t i = 0; i < n; i++) {
        const int64_t o = idx[i];
        const int k = nchw ? (int) (o % K) : (int) (o / kn);
        const int co = nchw ? (int) (o / K) : (int) (o % kn);
        float S = 0.0f;
        for (int64_t pc = 0; pc < P; pc += CG_KC) {
            int64_t kc = (P - pc < CG_KC) ? P - pc : CG_KC;
            float blk = 0.0f;
            for (int64_t p = pc; p < pc + kc; p++) {
                int oy = (int) (p % d.wo), ox = (int) ((p / d.wo) % d.ho), bb = (int) (p / hw);
                const float dv = nchw ? dy[((int64_t) bb * kn + co) * hw + (int64_t) ox * d.wo + oy]
                                      : dy[(size_t) p * kn + co];
                blk = fmaf(dv, xval(&d, nchw, x, bb, ox, oy, k), blk);
            }
            S = (pc == 0) ? blk : S + blk;
        }
        out[i] = S;
    }
}
