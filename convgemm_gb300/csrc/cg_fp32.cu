// FP32 plain form of the five convGemm entry points: SIMT FFMA implicit GEMM.
//
// Each output element is one fused multiply-add chain per KC=384 block of the
// reduction, blocks added in increasing order — the arithmetic of the
// reference's loop nests with a BLIS micro-kernel (the KC loop and betaI of
// src/gemm_blis_B3A2C0_orig.c:55-64, src/gemm_blis_B3A2C0.c:64; sxpbyM at
// src/gemm_blis.c:147-161), and the
// reduction index runs in the reference's order k = (c*kh + kx)*kw + ky
// (src/im2row_nhwc.c:163).  Forward and weight gradient therefore reproduce
// the reference's values, not just its tolerance.
//
// One templated kernel serves every operation; an "op" object supplies the
// implicit operands (im2row/im2col gathers straight from the activation
// tensor, never materialised), the block boundaries of the reduction and the
// store.  Tiles are 128x128 outputs per 256-thread CTA (256x64 when the
// operation has at most 64 columns), 8x8 per thread, reduction slices of 8
// double-buffered through shared memory.  Every gather address splits into a
// row part (computed once per thread) and a reduction-index part, which the
// CTA tabulates in shared memory 256 indices at a time, so a gathered element
// costs a table read, two bounds tests and an add.  The running sum of
// completed KC blocks lives in shared memory (it is touched once per 384
// reduction steps).
//
// Operands are read in the layout where a tile's column (or a B row) is
// contiguous: k x k NHWC activations through NCHW copies, single-tap NHWC rows
// as 16-byte channel vectors, weights repacked, NCHW weight-gradient operands
// through NHWC copies (see the entry points at the end).  Strided input
// gradients group their rows by stride phase (DgradPhaseOp), so each row runs
// only the taps that reach it.  None of this changes which products are added
// to an output, or in which order.
//
// Block split: when a convolution's tiles leave SMs idle or end in a thin last wave,
// the forward and input gradient run one CTA per (tile, reduction segment): each CTA
// writes the FMA chain of one KC block (input gradient: one KC block of one tap) to a
// scratch plane, and a second kernel adds the planes in order to the same start value
// (0, or dx) and applies the epilogue: the fused form's running sum, the same additions
// in the same order, so bit for bit the same result.
#include <climits>
#include <cmath>
#include <cstdint>
#include <tuple>
#include <type_traits>
#include <map>
#include <mutex>
#include <utility>
#include "cg_common.cuh"

namespace {

constexpr int BK = 8, NT = 256;
constexpr int KC = 384;
constexpr int OUT = 1 << 29;  // an input offset that puts a gather outside every image
constexpr int SREGS = 64;  // outputs per thread
constexpr size_t S_SMEM_BYTES = sizeof(float) * SREGS * NT;

__device__ __forceinline__ bool in_range(int v, int n) { return (unsigned) v < (unsigned) n; }

// Four consecutive outputs of one row: one 16-byte store where the caller knows p is aligned
// and all four exist, else the ones below `valid`.
__device__ __forceinline__ void store4(float *p, const float (&v)[4], bool vec, int valid) {
    if (vec && valid >= 4) {
        *reinterpret_cast<float4 *>(p) = make_float4(v[0], v[1], v[2], v[3]);
    } else {
#pragma unroll
        for (int j = 0; j < 4; j++)
            if (j < valid) p[j] = v[j];
    }
}

// The forward epilogue, operation by operation as the reference does it
// (src/im2row_nhwc.c:276-282, src/im2col_nchw.c:422-431); the gamma/beta step is
// one fused multiply-add, as gcc contracts it in the reference's -Ofast build.
__device__ __forceinline__ float fwd_epilogue(float t, int n, const cg_epi &e) {
    if (e.bias) t = __fadd_rn(t, __ldg(e.bias + n));
    if (e.mean) {
        t = __fmul_rn(__fsub_rn(t, __ldg(e.mean + n)), __ldg(e.inv_std + n));
        t = __fmaf_rn(t, __ldg(e.gamma + n), __ldg(e.beta + n));
    }
    if (e.relu && t < 0.0f) t = 0.0f;
    return t;
}

// ---------------------------------------------------------------- forward
// GEMM rows m = output pixel p = (b*ho + ox)*wo + oy, columns n = output
// channel, reduction r = K index (c, kx, ky).
//
// Every gather is base(row) + delta(r) in both layouts, valid where the input
// position (ix(row) + ox(r), iy(row) + oy(r)) lies inside the image:
//   NHWC  ((b*h + ix)*w + iy)*c + ch = ((b*h + bix)*w + biy)*c + ((kx*vdil)*w + ky*hdil)*c + ch
//   NCHW  ((b*c + ch)*h + ix)*w + iy = ((b*c*h) + bix)*w + biy + (ch*h + kx*vdil)*w + ky*hdil
// The row part is computed once per thread, the r part once per CTA (the
// reduction-index table).
struct FwdOp {
    ConvGeom g;
    int nchw;        // layout of y
    int xl, wl;      // layout of the x the kernel reads (0 NHWC, 1 NCHW) and of w (0 [K][kn], 1 [kn][K])
    int ov;          // y NHWC with 16-byte aligned rows of kn % 4 == 0
    const float *w, *x;
    float *y;
    cg_epi e;
    FastDiv dwo, dho, dkw, dkh;
    float *ws;   // block split: [K blocks][P][kn] chains, else NULL

    __host__ __device__ int M() const { return (int) g.P; }
    __host__ __device__ int N() const { return g.kn; }

    struct Row { long long base; int ix, iy; };
    __device__ Row row(int m) const {
        uint32_t q, oy, ox, bb;
        dwo.divmod(m < g.P ? m : 0, q, oy);
        dho.divmod(q, bb, ox);
        Row rw;
        const int bix = (int) ox * g.vstr - g.vpad, biy = (int) oy * g.hstr - g.hpad;
        rw.base = xl ? ((long long) bb * g.c * g.h + bix) * g.w + biy
                     : (((long long) bb * g.h + bix) * g.w + biy) * g.c;
        rw.ix = m < g.P ? bix : -OUT;
        rw.iy = biy;
        return rw;
    }
    // Single-tap NHWC: the row's reduction indices are its input pixel's channels, contiguous.
    __device__ bool row_in(const Row &rw) const { return in_range(rw.ix, g.h) && in_range(rw.iy, g.w); }
    __device__ const float *asrc() const { return x; }
    __device__ const float *bsrc() const { return w; }
    struct Col { long long base; int valid; };
    __device__ Col col(int n) const { return Col{wl ? (long long) n * g.K : (long long) n, n < g.kn}; }
    struct alignas(16) REnt { int delta, ox, oy, bd; };
    __device__ REnt rent(int r, int rend) const {
        uint32_t q, ky, kx, c;
        dkw.divmod(r < rend ? r : 0, q, ky);
        dkh.divmod(q, c, kx);
        REnt t;
        const int offx = (int) kx * g.vdil;
        t.oy = (int) ky * g.hdil;
        t.delta = xl ? ((int) c * g.h + offx) * g.w + t.oy : (offx * g.w + t.oy) * g.c + (int) c;
        t.ox = r < rend ? offx : -OUT;
        t.bd = r < rend ? (wl ? r : r * g.kn) : -1;
        return t;
    }
    __device__ float a(const Row &rw, const REnt &t) const {
        return in_range(rw.ix + t.ox, g.h) && in_range(rw.iy + t.oy, g.w) ? __ldg(x + (rw.base + t.delta)) : 0.0f;
    }
    __device__ float b(const Col &cl, const REnt &t) const {
        return cl.valid && t.bd >= 0 ? __ldg(w + (cl.base + t.bd)) : 0.0f;
    }
    __host__ __device__ int segments() const { return (g.K + KC - 1) / KC; }
    __host__ __device__ long long rlen() const { return g.K; }
    __device__ void range(int m0, int z, int &rbeg, int &rend) const {
        if (ws) {
            rbeg = z * KC;
            rend = min(g.K, rbeg + KC);
        } else {
            rbeg = 0;
            rend = g.K;
        }
    }
    __device__ int next_fold(int r, int rend) const {
        int nf = (r / KC + 1) * KC;
        return nf >= rend ? INT_MAX : nf;
    }
    __device__ float s_init(int m, int n) const { return 0.0f; }
    __device__ float s_start(int m, int n) const { return 0.0f; }
    __device__ int zcount(int m, int nz) const { return nz; }
    __device__ void finish_z4(int z, int m, int n, const float (&s)[4]) const {
        if (m >= (int) g.P) return;
        if (ws) return store4(ws + ((size_t) z * g.P + m) * g.kn + n, s, g.kn % 4 == 0, g.kn - n);
        if (!ov) {
#pragma unroll
            for (int j = 0; j < 4; j++) finish(m, n + j, s[j]);
            return;
        }
        float v[4];
#pragma unroll
        for (int j = 0; j < 4; j++) v[j] = n + j < g.kn ? fwd_epilogue(s[j], n + j, e) : 0.0f;
        store4(y + (size_t) m * g.kn + n, v, true, g.kn - n);
    }
    __device__ void finish(int m, int n, float s) const {
        if (m >= (int) g.P || n >= g.kn) return;
        float v = fwd_epilogue(s, n, e);
        if (nchw) {
            uint32_t q, oy, ox, bb;
            dwo.divmod(m, q, oy);
            dho.divmod(q, bb, ox);
            y[(((size_t) bb * g.kn + n) * g.ho + ox) * g.wo + oy] = v;
        } else {
            y[(size_t) m * g.kn + n] = v;
        }
    }
};

// --------------------------------------------------------- weight gradient
// Rows m = K index, columns n = output channel, reduction r = output pixel.
// One CTA per (tile, KC block of pixels): it writes that block's partial to
// the workspace, and wgrad_reduce adds the blocks in increasing order.  The
// gather of x is the forward's with the roles swapped: the tap part comes from
// the row, the pixel part from the reduction-index table.
struct WgradOp {
    ConvGeom g;
    int xl, yl;  // layout of the x and dy the kernel reads (0 NHWC, 1 NCHW)
    const float *dy, *x;
    float *ws;   // [nblocks][K][kn]
    int ov;      // ws 16-byte aligned, kn % 4 == 0
    FastDiv dwo, dho, dkw, dkh;

    __host__ __device__ int M() const { return g.K; }
    __host__ __device__ int N() const { return g.kn; }

    struct Row { int delta, ox, oy; };
    __device__ Row row(int m) const {
        uint32_t q, ky, kx, c;
        dkw.divmod(m < g.K ? m : 0, q, ky);
        dkh.divmod(q, c, kx);
        Row rw;
        const int offx = (int) kx * g.vdil;
        rw.oy = (int) ky * g.hdil;
        rw.delta = xl ? ((int) c * g.h + offx) * g.w + rw.oy : (offx * g.w + rw.oy) * g.c + (int) c;
        rw.ox = m < g.K ? offx : -OUT;
        return rw;
    }
    struct Col { long long base; int valid; };
    __device__ Col col(int n) const {
        return Col{yl ? (long long) n * g.ho * g.wo : (long long) n, n < g.kn};
    }
    __device__ const float *bsrc() const { return dy; }
    struct alignas(16) REnt { long long base; int ix, iy; long long bd; long long pad; };
    __device__ REnt rent(int r, int rend) const {
        uint32_t q, oy, ox, bb;
        dwo.divmod(r < rend ? r : 0, q, oy);
        dho.divmod(q, bb, ox);
        REnt t;
        const int bix = (int) ox * g.vstr - g.vpad, biy = (int) oy * g.hstr - g.hpad;
        t.base = xl ? ((long long) bb * g.c * g.h + bix) * g.w + biy
                      : (((long long) bb * g.h + bix) * g.w + biy) * g.c;
        t.ix = r < rend ? bix : -OUT;
        t.iy = biy;
        const long long hw = (long long) g.ho * g.wo;
        t.bd = r < rend ? (yl ? (long long) bb * g.kn * hw + ((long long) ox * g.wo + oy) : (long long) r * g.kn)
                        : -1;
        t.pad = 0;
        return t;
    }
    __device__ float a(const Row &rw, const REnt &t) const {
        return in_range(t.ix + rw.ox, g.h) && in_range(t.iy + rw.oy, g.w) ? __ldg(x + (t.base + rw.delta)) : 0.0f;
    }
    __device__ float b(const Col &cl, const REnt &t) const {
        return cl.valid && t.bd >= 0 ? __ldg(dy + (cl.base + t.bd)) : 0.0f;
    }
    __device__ void range(int m0, int z, int &rbeg, int &rend) const {
        rbeg = z * KC;
        rend = min((long long) (z + 1) * KC, g.P);
    }
    __device__ int next_fold(int r, int rend) const { return INT_MAX; }
    __device__ float s_init(int m, int n) const { return 0.0f; }
    __device__ void finish_z4(int z, int m, int n, const float (&s)[4]) const {
        if (m < g.K) store4(ws + ((size_t) z * g.K + m) * g.kn + n, s, ov, g.kn - n);
    }
};

// ---------------------------------------------------------- input gradient
// Gather form: rows m = input pixel (b, ih, iw), columns n = input channel,
// reduction r = tap*kn + l over taps (kx, ky) and output channels l.  A tap
// contributes where (ih + vpad - kx*vdil) is a non-negative multiple of the
// stride below ho (same for iy).  Each (tap, KC block of l) partial is added
// to the running value in a fixed order; the reference adds the same partials
// with `omp atomic` in thread order (src/im2row_nhwc.c:252).
//
// With ih + vpad = vstr*xd + xm and kx*vdil = vstr*exd + exm (0 <= xm, exm < vstr),
// the tap reads output row xd - exd exactly when xm == exm, so the table holds
// (exd, exm) per r and the rows hold (xd, xm): no division per element.
struct DgradOp {
    ConvGeom g;
    int nchw, accumulate;   // layout of dx; dx += result
    int yl;                 // layout of the dy the kernel reads (0 NHWC, 1 NCHW)
    int wl;                 // layout of w: 0 NHWC [c][tap][kn], 1 NCHW [kn][c][tap], 2 packed [tap][kn][c]
    int ov;                 // dx NHWC with 16-byte aligned rows of c % 4 == 0
    const float *w, *dy;
    float *dx;
    FastDiv dw_, dh_, dkn, dkw, dvs, dhs;
    float *ws;   // block split: [segment][b*h*w][c] chains (segment = tap, KC block of kn), else NULL

    __host__ __device__ int M() const { return g.b * g.h * g.w; }
    __host__ __device__ int N() const { return g.c; }

    struct Row { long long base; int ix, iy, cls; };
    __device__ Row row(int m) const {
        const bool valid = m < M();
        uint32_t q, iw, ih, bb, xd, xm, yd, ym;
        dw_.divmod(valid ? m : 0, q, iw);
        dh_.divmod(q, bb, ih);
        dvs.divmod(ih + g.vpad, xd, xm);
        dhs.divmod(iw + g.hpad, yd, ym);
        Row rw;
        rw.base = yl ? ((long long) bb * g.kn * g.ho + xd) * g.wo + yd
                     : (((long long) bb * g.ho + xd) * g.wo + yd) * g.kn;
        rw.ix = valid ? (int) xd : -OUT;
        rw.iy = (int) yd;
        rw.cls = (int) (xm | (ym << 16));
        return rw;
    }
    // Single-tap NHWC: the row's reduction indices are its output pixel's channels, contiguous.
    __device__ bool row_in(const Row &rw) const {
        return rw.cls == 0 && in_range(rw.ix, g.ho) && in_range(rw.iy, g.wo);
    }
    __device__ const float *asrc() const { return dy; }
    __device__ const float *bsrc() const { return w; }
    struct Col { long long base; int valid; };
    __device__ Col col(int n) const {
        const long long b = wl == 2 ? n : wl == 1 ? (long long) n * g.kh * g.kw : (long long) n * g.kh * g.kw * g.kn;
        return Col{b, n < g.c};
    }
    struct alignas(16) REnt { int delta, ox, oy, cls, bd, pad0, pad1, pad2; };
    __device__ REnt rent(int r, int rend) const {
        uint32_t tap, l, kx, ky, exd, exm, eyd, eym;
        dkn.divmod(r < rend ? r : 0, tap, l);
        dkw.divmod(tap, kx, ky);
        dvs.divmod(kx * g.vdil, exd, exm);
        dhs.divmod(ky * g.hdil, eyd, eym);
        REnt t;
        t.delta = yl ? ((int) l * g.ho - (int) exd) * g.wo - (int) eyd
                     : (int) l - ((int) exd * g.wo + (int) eyd) * g.kn;
        t.ox = r < rend ? -(int) exd : -OUT;
        t.oy = -(int) eyd;
        t.cls = (int) (exm | (eym << 16));
        t.bd = r < rend ? (wl == 2 ? r * g.c : wl == 1 ? (int) l * g.K + (int) tap : r) : -1;
        t.pad0 = t.pad1 = t.pad2 = 0;
        return t;
    }
    __device__ float a(const Row &rw, const REnt &t) const {
        return rw.cls == t.cls && in_range(rw.ix + t.ox, g.ho) && in_range(rw.iy + t.oy, g.wo)
                   ? __ldg(dy + (rw.base + t.delta)) : 0.0f;
    }
    __device__ float b(const Col &cl, const REnt &t) const {
        return cl.valid && t.bd >= 0 ? __ldg(w + (cl.base + t.bd)) : 0.0f;
    }
    __host__ __device__ int segments() const { return g.kh * g.kw * ((g.kn + KC - 1) / KC); }
    __host__ __device__ long long rlen() const { return (long long) g.kh * g.kw * g.kn; }
    __device__ void range(int m0, int z, int &rbeg, int &rend) const {
        if (ws) {
            const int nch = (g.kn + KC - 1) / KC, tap = z / nch, j = z - tap * nch;
            rbeg = tap * g.kn + j * KC;
            rend = tap * g.kn + min(g.kn, (j + 1) * KC);
        } else {
            rbeg = 0;
            rend = g.kh * g.kw * g.kn;
        }
    }
    __device__ int next_fold(int r, int rend) const {
        uint32_t tap, l;
        dkn.divmod(r, tap, l);
        int nf = r - (int) l + min(g.kn, (int) (l / KC + 1) * KC);
        return nf >= rend ? INT_MAX : nf;
    }
    __device__ size_t out_index(int m, int n) const {
        if (!nchw) return (size_t) m * g.c + n;
        uint32_t q, iw, ih, bb;
        dw_.divmod(m, q, iw);
        dh_.divmod(q, bb, ih);
        return (((size_t) bb * g.c + n) * g.h + ih) * g.w + iw;
    }
    __device__ float s_init(int m, int n) const {
        if (ws || !accumulate || m >= M() || n >= g.c) return 0.0f;   // split: the reduction starts from dx
        return dx[out_index(m, n)];
    }
    __device__ float s_start(int m, int n) const {
        if (!accumulate || m >= M() || n >= g.c) return 0.0f;
        return dx[out_index(m, n)];
    }
    __device__ int zcount(int m, int nz) const { return nz; }
    __device__ void finish_z4(int z, int m, int n, const float (&s)[4]) const {
        if (m >= M()) return;
        if (ws) return store4(ws + ((size_t) z * M() + m) * g.c + n, s, g.c % 4 == 0, g.c - n);
        if (ov) return store4(dx + (size_t) m * g.c + n, s, true, g.c - n);
#pragma unroll
        for (int j = 0; j < 4; j++) finish(m, n + j, s[j]);
    }
    __device__ void finish(int m, int n, float s) const {
        if (m >= M() || n >= g.c) return;
        dx[out_index(m, n)] = s;
    }
};


// ------------------------------------------- input gradient, strided layers
// The gather form above runs every tap for every input pixel, although with strides
// (sv, sh) a pixel of stride phase (xm, ym) = ((ih + vpad) % sv, (iw + hpad) % sh) is
// reached only by the taps of the same phase.  Here the GEMM rows are the input pixels
// grouped by phase (each phase padded to a multiple of 256 rows, so no tile straddles
// two), and a phase's reduction runs over its own taps only, in increasing tap order:
// the segments (tap, KC block of kn) of a pixel are those of the gather form minus the
// ones whose products are all zero, added in the same order.
constexpr int DG_MAXCLS = 16, DG_MAXTAPS = 64;
struct DgPhase {
    int mbeg, rows;   // first (padded) GEMM row, pixels of this phase
    int ih0, iw0;     // first input row / column of this phase
    int rbeg, ntaps;  // reduction indices [rbeg, rbeg + ntaps*kn), taps tap0 .. tap0 + ntaps - 1
    int tap0;
    FastDiv dwc, dhc; // phase columns and rows per image
};
struct DgradPhaseOp {
    ConvGeom g;
    int nchw, accumulate, yl, wl, ov;   // as in DgradOp
    const float *w, *dy;
    float *dx;
    FastDiv dkn, dvs, dhs;
    int ncls, mpad, nkb;            // phases, padded rows, KC blocks per tap
    DgPhase ph[DG_MAXCLS];
    unsigned char taps[DG_MAXTAPS]; // tap indices kx*kw + ky grouped by phase
    float *ws;

    __host__ __device__ int M() const { return mpad; }
    __host__ __device__ int N() const { return g.c; }
    __device__ int phase_of_m(int m) const {
        int c = 0;
        for (int i = 1; i < ncls; i++) c = m >= ph[i].mbeg ? i : c;
        return c;
    }
    __device__ int phase_of_r(int r) const {
        int c = 0;
        for (int i = 1; i < ncls; i++) c = r >= ph[i].rbeg && ph[i].ntaps ? i : c;
        return c;
    }
    // GEMM row -> input pixel (b, ih, iw), or false for padding rows
    __device__ bool pixel(int m, uint32_t &bb, int &ih, int &iw) const {
        const DgPhase &p = ph[phase_of_m(m)];
        const int loc = m - p.mbeg;
        uint32_t q, tw, th;
        p.dwc.divmod(loc < p.rows ? loc : 0, q, tw);
        p.dhc.divmod(q, bb, th);
        ih = p.ih0 + (int) th * g.vstr;
        iw = p.iw0 + (int) tw * g.hstr;
        return loc < p.rows;
    }

    struct Row { long long base; int ix, iy; };
    __device__ Row row(int m) const {
        uint32_t bb;
        int ih, iw;
        const bool valid = pixel(m, bb, ih, iw);
        const int xd = (ih + g.vpad) / g.vstr, yd = (iw + g.hpad) / g.hstr;   // exact for this phase
        Row rw;
        rw.base = yl ? ((long long) bb * g.kn * g.ho + xd) * g.wo + yd
                     : (((long long) bb * g.ho + xd) * g.wo + yd) * g.kn;
        rw.ix = valid ? xd : -OUT;
        rw.iy = yd;
        return rw;
    }
    __device__ bool row_in(const Row &rw) const { return in_range(rw.ix, g.ho) && in_range(rw.iy, g.wo); }
    __device__ const float *asrc() const { return dy; }
    __device__ const float *bsrc() const { return w; }
    struct Col { long long base; int valid; };
    __device__ Col col(int n) const {
        const long long b = wl == 2 ? n : wl == 1 ? (long long) n * g.kh * g.kw : (long long) n * g.kh * g.kw * g.kn;
        return Col{b, n < g.c};
    }
    struct alignas(16) REnt { int delta, ox, oy, bd; };
    __device__ REnt rent(int r, int rend) const {
        const DgPhase &p = ph[phase_of_r(r)];
        uint32_t j, l;
        dkn.divmod(r < rend ? r - p.rbeg : 0, j, l);
        const int tap = p.ntaps > 0 ? taps[p.tap0 + min((int) j, p.ntaps - 1)] : 0;
        const int kx = tap / g.kw, ky = tap - kx * g.kw;
        const int exd = kx * g.vdil / g.vstr, eyd = ky * g.hdil / g.hstr;
        REnt t;
        t.delta = yl ? ((int) l * g.ho - exd) * g.wo - eyd : (int) l - (exd * g.wo + eyd) * g.kn;
        t.ox = r < rend ? -exd : -OUT;
        t.oy = -eyd;
        const int rg = tap * g.kn + (int) l;   // reduction index of the gather form
        t.bd = r < rend ? (wl == 2 ? rg * g.c : wl == 1 ? (int) l * g.K + tap : rg) : -1;
        return t;
    }
    __device__ float a(const Row &rw, const REnt &t) const {
        return in_range(rw.ix + t.ox, g.ho) && in_range(rw.iy + t.oy, g.wo) ? __ldg(dy + (rw.base + t.delta)) : 0.0f;
    }
    __device__ float b(const Col &cl, const REnt &t) const {
        return cl.valid && t.bd >= 0 ? __ldg(w + (cl.base + t.bd)) : 0.0f;
    }
    __host__ __device__ int segments() const {
        int nt = 0;
        for (int i = 0; i < ncls; i++) nt = ph[i].ntaps > nt ? ph[i].ntaps : nt;
        return nt * nkb;
    }
    __host__ __device__ long long rlen() const { return (long long) segments() * min(g.kn, KC); }
    __device__ void range(int m0, int z, int &rbeg, int &rend) const {
        const DgPhase &p = ph[phase_of_m(m0)];
        if (ws) {
            const int j = z / nkb, kb = z - j * nkb;
            if (j >= p.ntaps) {
                rbeg = rend = p.rbeg;
                return;
            }
            rbeg = p.rbeg + j * g.kn + kb * KC;
            rend = p.rbeg + j * g.kn + min(g.kn, (kb + 1) * KC);
        } else {
            rbeg = p.rbeg;
            rend = p.rbeg + p.ntaps * g.kn;
        }
    }
    __device__ int next_fold(int r, int rend) const {
        const DgPhase &p = ph[phase_of_r(r)];
        uint32_t j, l;
        dkn.divmod(r - p.rbeg, j, l);
        int nf = r - (int) l + min(g.kn, (int) (l / KC + 1) * KC);
        return nf >= rend ? INT_MAX : nf;
    }
    __device__ int zcount(int m, int nz) const { return ph[phase_of_m(m)].ntaps * nkb; }
    __device__ bool out_index(int m, int n, size_t &o) const {
        uint32_t bb;
        int ih, iw;
        if (!pixel(m, bb, ih, iw) || n >= g.c) return false;
        o = nchw ? (((size_t) bb * g.c + n) * g.h + ih) * g.w + iw : (((size_t) bb * g.h + ih) * g.w + iw) * g.c + n;
        return true;
    }
    __device__ float s_start(int m, int n) const {
        size_t o;
        return accumulate && out_index(m, n, o) ? dx[o] : 0.0f;
    }
    __device__ float s_init(int m, int n) const { return ws ? 0.0f : s_start(m, n); }
    __device__ void finish_z4(int z, int m, int n, const float (&s)[4]) const {
        if (ws) {
            if (z < zcount(m, 0)) store4(ws + ((size_t) z * mpad + m) * g.c + n, s, g.c % 4 == 0, g.c - n);
            return;
        }
        size_t o;
        if (ov && out_index(m, n, o)) return store4(dx + o, s, true, g.c - n);
#pragma unroll
        for (int j = 0; j < 4; j++) finish(m, n + j, s[j]);
    }
    __device__ void finish(int m, int n, float s) const {
        size_t o;
        if (out_index(m, n, o)) dx[o] = s;
    }
};

// Tiles of BM x BN outputs per 256-thread CTA, 8 x 8 per thread: 128 x 128, or
// 256 x 64 for operations with at most 64 columns (no padding columns computed).
template <int BM_, int BN_>
struct Tile {
    static constexpr int BM = BM_, BN = BN_;
    static constexpr int TX = BN / 8;                      // compute threads along n
    static_assert((BM / 8) * (BN / 8) == NT, "8 x 8 outputs per thread");
    static constexpr int AP = BM * BK / NT, AS = NT / BM;  // A elements per thread per slice, their r stride
    static constexpr int BP = BN * BK / NT, BS = NT / BN;
};
using TileSquare = Tile<128, 128>;
using TileTall = Tile<256, 64>;

// VEC (single-tap NHWC operations): the reduction indices of an A row are consecutive
// channels of one pixel, so each thread loads whole 4-index quads of its row as 16-byte
// vectors (two threads cover the 8 indices of a row in a slice) instead of gathering
// element by element down a column.
// BV (B read from a layout with the tile's columns contiguous, N % 4 == 0, 16-byte aligned):
// each B row of a slice is loaded as BN/4 16-byte vectors, one per thread.
template <class Op, class T, bool VEC, bool BV>
__global__ void __launch_bounds__(NT, 2) fp32_igemm_kernel(const Op op) {
    __shared__ __align__(16) float As[2][BK][T::BM];
    __shared__ __align__(16) float Bs[2][BK][T::BN];
    // Reduction-index table: the r part of every gather, for two chunks of NT
    // consecutive r; chunk c + 1 is filled while the slices of chunk c run.
    __shared__ typename Op::REnt Rt[2][NT];
    extern __shared__ float Ssm[];  // [SREGS][NT], running sum of completed KC blocks
    constexpr int SLICES = NT / BK;  // slices per table chunk

    const int tid = threadIdx.x;
    const int m0 = blockIdx.x * T::BM;
    const int n0 = blockIdx.y * T::BN;
    const int z = blockIdx.z;
    int rbeg, rend;
    op.range(m0, z, rbeg, rend);
    Rt[0][tid] = op.rent(rbeg + tid, rend);
    Rt[1][tid] = op.rent(rbeg + NT + tid, rend);

    // loader mapping: A element (ak + AS*i, am), B element (bk + BS*i, bn) of each slice;
    // VEC: A quads vq .. vq + VQ - 1 (indices 4*vq ...) of row am
    constexpr int TPR = NT / T::BM, VQ = (BK / 4) / TPR;
    static_assert(!VEC || 4 * VQ == T::AP, "a thread's A quads cover its A elements");
    const int am = VEC ? tid / TPR : tid % T::BM, ak = tid / T::BM, vq = (tid % TPR) * VQ;
    const int bn = tid % T::BN, bk = tid / T::BN;
    constexpr int QB = T::BN / 4;   // BV: 16-byte quads per B row of a slice
    const auto arow = op.row(m0 + am);
    const auto bcol = op.col(n0 + (BV ? 4 * (tid % QB) : bn));
    float ra[T::AP], rb[T::BP];
    float4 rbv = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const float *vsrc = nullptr;
    if constexpr (VEC) vsrc = op.row_in(arow) ? op.asrc() + arow.base : nullptr;

    // compute mapping: rows {ty*4+i, BM/2+ty*4+i}, columns {tx*4+j, BN/2+tx*4+j}
    const int tx = tid % T::TX, ty = tid / T::TX;
    auto mrow = [&](int i) { return m0 + (i < 4 ? ty * 4 + i : T::BM / 2 + ty * 4 + i - 4); };
    auto ncol = [&](int j) { return n0 + (j < 4 ? tx * 4 + j : T::BN / 2 + tx * 4 + j - 4); };

#pragma unroll
    for (int i = 0; i < 8; i++)
#pragma unroll
        for (int j = 0; j < 8; j++) Ssm[(i * 8 + j) * NT + tid] = op.s_init(mrow(i), ncol(j));

    float acc[8][8];
#pragma unroll
    for (int i = 0; i < 8; i++)
#pragma unroll
        for (int j = 0; j < 8; j++) acc[i][j] = 0.0f;

    auto fold = [&]() {
#pragma unroll
        for (int i = 0; i < 8; i++)
#pragma unroll
            for (int j = 0; j < 8; j++) {
                float *s = &Ssm[(i * 8 + j) * NT + tid];
                *s = __fadd_rn(*s, acc[i][j]);
                acc[i][j] = 0.0f;
            }
    };

    auto gload = [&](int t) {
        const int rr = t * BK;   // slices never straddle a chunk: NT % BK == 0
        const typename Op::REnt *rt = Rt[(rr / NT) & 1] + rr % NT;
        if constexpr (VEC) {
#pragma unroll
            for (int q = 0; q < VQ; q++) {
                const int r = rbeg + rr + 4 * (vq + q);
                float4 v = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                if (vsrc) {
                    if (r + 3 < rend) {
                        v = __ldg(reinterpret_cast<const float4 *>(vsrc + r));
                    } else {
                        if (r < rend) v.x = __ldg(vsrc + r);
                        if (r + 1 < rend) v.y = __ldg(vsrc + r + 1);
                        if (r + 2 < rend) v.z = __ldg(vsrc + r + 2);
                    }
                }
                ra[4 * q] = v.x;
                ra[4 * q + 1] = v.y;
                ra[4 * q + 2] = v.z;
                ra[4 * q + 3] = v.w;
            }
        } else {
#pragma unroll
            for (int i = 0; i < T::AP; i++) ra[i] = op.a(arow, rt[ak + T::AS * i]);
        }
        if constexpr (BV) {
            if (tid < BK * QB) {
                const long long bd = rt[tid / QB].bd;
                rbv = bcol.valid && bd >= 0 ? __ldg(reinterpret_cast<const float4 *>(op.bsrc() + (bcol.base + bd)))
                                            : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            }
        } else {
#pragma unroll
            for (int i = 0; i < T::BP; i++) rb[i] = op.b(bcol, rt[bk + T::BS * i]);
        }
    };
    auto sstore = [&](int buf) {
        if constexpr (VEC) {
#pragma unroll
            for (int q = 0; q < VQ; q++)
#pragma unroll
                for (int j = 0; j < 4; j++) As[buf][4 * (vq + q) + j][am] = ra[4 * q + j];
        } else {
#pragma unroll
            for (int i = 0; i < T::AP; i++) As[buf][ak + T::AS * i][am] = ra[i];
        }
        if constexpr (BV) {
            if (tid < BK * QB) *reinterpret_cast<float4 *>(&Bs[buf][tid / QB][4 * (tid % QB)]) = rbv;
        } else {
#pragma unroll
            for (int i = 0; i < T::BP; i++) Bs[buf][bk + T::BS * i][bn] = rb[i];
        }
    };
    auto step = [&](int buf, int kk) {
        const float4 a0 = *reinterpret_cast<const float4 *>(&As[buf][kk][ty * 4]);
        const float4 a1 = *reinterpret_cast<const float4 *>(&As[buf][kk][T::BM / 2 + ty * 4]);
        const float4 b0 = *reinterpret_cast<const float4 *>(&Bs[buf][kk][tx * 4]);
        const float4 b1 = *reinterpret_cast<const float4 *>(&Bs[buf][kk][T::BN / 2 + tx * 4]);
        const float av[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
        const float bv[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
        for (int i = 0; i < 8; i++)
#pragma unroll
            for (int j = 0; j < 8; j++) acc[i][j] = __fmaf_rn(av[i], bv[j], acc[i][j]);
    };

    const int ntiles = (rend - rbeg + BK - 1) / BK;
    int next_fold = op.next_fold(rbeg, rend);
    __syncthreads();
    gload(0);
    sstore(0);
    __syncthreads();
    for (int t = 0; t < ntiles; t++) {
        const int buf = t & 1;
        if (t > 0 && t % SLICES == 0) {
            // chunk c + 1 replaces chunk c - 1, whose last reader (slice 32c - 1's
            // loads, issued during slice 32c - 2) is behind two barriers
            const int c = t / SLICES + 1;
            Rt[c & 1][tid] = op.rent(rbeg + c * NT + tid, rend);
        }
        if (t + 1 < ntiles) gload(t + 1);
        const int r0 = rbeg + t * BK;
        if (next_fold >= r0 + BK) {
#pragma unroll
            for (int kk = 0; kk < BK; kk++) step(buf, kk);
        } else {
#pragma unroll 1
            for (int kk = 0; kk < BK; kk++) {
                if (r0 + kk == next_fold) {
                    fold();
                    next_fold = op.next_fold(r0 + kk, rend);
                }
                step(buf, kk);
            }
        }
        if (t + 1 < ntiles) sstore(buf ^ 1);
        __syncthreads();
    }
    if (ntiles > 0) fold();   // an empty range leaves the start value as it is

#pragma unroll
    for (int i = 0; i < 8; i++)
#pragma unroll
        for (int q = 0; q < 2; q++) {   // columns ncol(4q) .. ncol(4q) + 3 are consecutive
            float v[4];
#pragma unroll
            for (int j = 0; j < 4; j++) v[j] = Ssm[(i * 8 + q * 4 + j) * NT + tid];
            op.finish_z4(z, mrow(i), ncol(4 * q), v);
        }
}

// Block split: out(m, n) = finish(((start + ws[0]) + ws[1]) + ...), the planes in segment order
// (start: 0, or dx for the accumulating input gradient).
template <class Op>
__global__ void fp32_split_reduce_kernel(const Op op, const float *__restrict__ ws, int nz, int M, int N) {
    const long long total = (long long) M * N;
    for (long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < total;
         i += (long long) gridDim.x * blockDim.x) {
        const int m = (int) (i / N), n = (int) (i % N);
        float s = op.s_start(m, n);
        const int nzr = op.zcount(m, nz);
        int z = 0;
        for (; z + 8 <= nzr; z += 8) {
            float v[8];
#pragma unroll
            for (int j = 0; j < 8; j++) v[j] = ws[(size_t) (z + j) * total + i];
#pragma unroll
            for (int j = 0; j < 8; j++) s = __fadd_rn(s, v[j]);
        }
        for (; z < nzr; z++) s = __fadd_rn(s, ws[(size_t) z * total + i]);
        op.finish(m, n, s);
    }
}

// dW(m, n) = ((ws[0] + ws[1]) + ws[2]) + ... : the reference's block order.
__global__ void wgrad_reduce_kernel(const float *__restrict__ ws, float *__restrict__ dw, int K, int kn,
                                    int nblocks, int nchw) {
    const long long total = (long long) K * kn;
    for (long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < total;
         i += (long long) gridDim.x * blockDim.x) {
        // loads eight blocks ahead, adds strictly in block order
        float s = ws[i];
        int z = 1;
        for (; z + 8 <= nblocks; z += 8) {
            float v[8];
#pragma unroll
            for (int j = 0; j < 8; j++) v[j] = ws[(size_t) (z + j) * total + i];
#pragma unroll
            for (int j = 0; j < 8; j++) s = __fadd_rn(s, v[j]);
        }
        for (; z < nblocks; z++) s = __fadd_rn(s, ws[(size_t) z * total + i]);
        const int m = (int) (i / kn), n = (int) (i % kn);
        dw[nchw ? ((size_t) n * K + m) : (size_t) i] = s;
    }
}

template <class Op, class T, bool VEC, bool BV>
cudaError_t launch_tile(const Op &op, int gz, cudaStream_t st) {
    static bool attr_set = false;  // per template instance; harmless if set twice
    if (!attr_set) {
        cudaError_t e = cudaFuncSetAttribute(fp32_igemm_kernel<Op, T, VEC, BV>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int) S_SMEM_BYTES);
        if (e != cudaSuccess) return e;
        attr_set = true;
    }
    dim3 grid((op.M() + T::BM - 1) / T::BM, (op.N() + T::BN - 1) / T::BN, gz);
    if (grid.x == 0 || grid.y == 0) return cudaSuccess;
    fp32_igemm_kernel<Op, T, VEC, BV><<<grid, NT, S_SMEM_BYTES, st>>>(op); cg_note_launch();
    return cudaGetLastError();
}

// 256 x 64 tiles where a 128-wide tile would compute padding columns.
inline bool tall_tiles(int N) { return N <= 64; }

template <class Op, bool VEC, bool BV>
cudaError_t launch_shape(const Op &op, int gz, cudaStream_t st) {
    return tall_tiles(op.N()) ? launch_tile<Op, TileTall, VEC, BV>(op, gz, st)
                              : launch_tile<Op, TileSquare, VEC, BV>(op, gz, st);
}

template <class Op, bool VEC>
cudaError_t launch_bv(const Op &op, int gz, bool bv, cudaStream_t st) {
    return bv ? launch_shape<Op, VEC, true>(op, gz, st) : launch_shape<Op, VEC, false>(op, gz, st);
}

// vec: A rows as channel vectors (single-tap NHWC forward / input gradient), taken together
// with bv (B rows as 16-byte vectors), which the same layouts allow.
template <class Op>
cudaError_t launch(const Op &op, int gz, bool vec, bool bv, cudaStream_t st) {
    if constexpr (!std::is_same<Op, WgradOp>::value) {
        if (vec && bv) return launch_shape<Op, true, true>(op, gz, st);
    }
    return launch_bv<Op, false>(op, gz, bv, st);
}

// Gathers add 32-bit offsets within one image and within the weights.
inline bool offsets_fit(const ConvGeom &g) {
    const long long lim = INT_MAX / 2;
    return (long long) g.c * g.h * g.w < lim && (long long) g.kn * g.ho * g.wo < lim &&
           (long long) g.K * g.kn < lim;
}

// Library-owned scratch, one grow-only buffer per (device, stream, purpose): a CUDA graph
// that captured a buffer keeps using it, so buffers are never freed or reused for another
// stream.  Purposes: the block split's planes, an operand copy in the kernel's gather layout
// (activation; a second one where a call copies two), a repacked weight tensor.
enum { SLOT_SPLIT = 0, SLOT_ACT = 1, SLOT_WGT = 2, SLOT_ACT2 = 3 };
constexpr size_t SLOT_MAX[4] = {(size_t) 256 << 20, (size_t) 4 << 30, (size_t) 256 << 20, (size_t) 4 << 30};
std::mutex g_scratch_mu;
std::map<std::tuple<int, cudaStream_t, int>, std::pair<float *, size_t>> g_scratch;

float *scratch(int slot, size_t bytes, cudaStream_t st) {
    if (bytes == 0 || bytes > SLOT_MAX[slot]) return nullptr;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    auto &e = g_scratch[std::make_tuple(dev, st, slot)];
    if (e.second >= bytes) return e.first;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) {
        cudaGetLastError();
        return nullptr;   // no allocation under capture: the form without scratch runs instead
    }
    size_t want = e.second ? e.second : ((size_t) 32 << 20);
    while (want < bytes) want *= 2;
    if (want > SLOT_MAX[slot]) want = SLOT_MAX[slot];
    float *p = nullptr;
    if (cudaMalloc(&p, want) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    e = {p, want};   // the previous buffer stays allocated for graphs that captured it
    return p;
}

// dst[b][c][r] = src[b][r][c] through 32 x 33 shared-memory tiles (both sides coalesced).
__global__ void transpose_kernel(const float *__restrict__ src, float *__restrict__ dst, int R, int C) {
    __shared__ float t[32][33];
    const size_t off = (size_t) blockIdx.z * R * C;
    const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
    for (int i = threadIdx.y; i < 32; i += 8) {
        const int r = r0 + i, c = c0 + threadIdx.x;
        if (r < R && c < C) t[i][threadIdx.x] = src[off + (size_t) r * C + c];
    }
    __syncthreads();
    for (int i = threadIdx.y; i < 32; i += 8) {
        const int c = c0 + i, r = r0 + threadIdx.x;
        if (r < R && c < C) dst[off + (size_t) c * R + r] = t[threadIdx.x][i];
    }
}

// A transposed copy of src ([batch][R][C] -> [batch][C][R]) in the given scratch slot, or NULL
// when there is no room (or the grid would not fit); the caller then reads src as it is.
const float *transposed(int slot, const float *src, long long batch, long long R, long long C, cudaStream_t st) {
    const long long gy = (R + 31) / 32, gx = (C + 31) / 32;
    if (batch < 1 || batch > 65535 || gy > 65535 || gx > INT_MAX) return nullptr;
    float *dst = scratch(slot, sizeof(float) * (size_t) (batch * R * C), st);
    if (!dst) return nullptr;
    transpose_kernel<<<dim3((unsigned) gx, (unsigned) gy, (unsigned) batch), dim3(32, 8), 0, st>>>(src, dst, (int) R,
                                                                                                   (int) C);
    cg_note_launch();
    if (cudaGetLastError() != cudaSuccess) return nullptr;
    return dst;
}

inline bool aligned16(const void *p) { return ((uintptr_t) p & 15) == 0; }

// The block split pays when the fused grid leaves SMs idle or ends in a thin last wave (two
// CTAs fit per SM), weighed against the planes it writes and reads back.  Model: the kernel's
// rate at full waves (about 35 TFLOP/s) scaled by the fraction of CTA slots its waves fill,
// plus the planes' bytes at about 4 TB/s.
template <class Op>
cudaError_t launch_split_or_fused(Op op, int M, int N, bool vec, bool bv, cudaStream_t st) {
    const int bm = tall_tiles(N) ? TileTall::BM : TileSquare::BM, bn = tall_tiles(N) ? TileTall::BN : TileSquare::BN;
    const long long tiles = (long long) ((M + bm - 1) / bm) * ((N + bn - 1) / bn);
    const int nz = op.segments();
    int sms = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    op.ws = nullptr;
    if (nz > 1 && tiles > 0) {
        const double slots = 2.0 * sms;
        auto filled = [&](double n) { return n / (std::ceil(n / slots) * slots); };
        const size_t bytes = sizeof(float) * (size_t) nz * (size_t) M * (size_t) N;
        const double flops = 2.0 * M * N * (double) op.rlen(), rate = 35e12;
        const double t_fused = flops / (rate * filled((double) tiles));
        const double t_split = flops / (rate * filled((double) tiles * nz)) + 2.0 * (double) bytes / 4e12;
        if (t_split < t_fused) op.ws = scratch(SLOT_SPLIT, bytes, st);
    }
    if (!op.ws) return launch(op, 1, vec, bv, st);
    cudaError_t e = launch(op, nz, vec, bv, st);
    if (e != cudaSuccess) return e;
    const long long total = (long long) M * N;
    const int blocks = (int) std::min<long long>((total + 255) / 256, (long long) sms * 16);
    float *ws = op.ws;
    fp32_split_reduce_kernel<Op><<<blocks, 256, 0, st>>>(op, ws, nz, M, N); cg_note_launch();
    return cudaGetLastError();
}

// A call's launches (operand copies, the kernel, the plane reduction) are enqueued under one
// lock: the copies live in per-stream scratch, so two host threads enqueueing on the same
// stream must not interleave one call's copy between another call's copy and its kernel.
std::mutex g_call_mu;

}  // namespace

// Operand layouts the kernel reads (the arithmetic and its order do not depend on them):
// a k x k NHWC forward reads x from an NCHW copy (a column of A, 128 output pixels at one
// reduction index, is then 128 consecutive floats instead of 128 pixels c floats apart);
// a single-tap NHWC forward reads x rows as 16-byte channel vectors; an NCHW forward reads
// its weights as [K][kn] (a row of B contiguous).
cudaError_t cg_fp32_fwd(int nchw, const cg_shape &s, const float *w, const float *x, float *y,
                        const cg_epi &e, cudaStream_t st) {
    std::lock_guard<std::mutex> call_lock(g_call_mu);
    FwdOp op;
    op.g = make_geom(s);
    if (!offsets_fit(op.g)) return cudaErrorNotSupported;
    op.nchw = nchw;
    op.xl = op.wl = nchw;
    op.w = w;
    op.x = x;
    op.y = y;
    op.e = e;
    op.dwo = FastDiv(op.g.wo);
    op.dho = FastDiv(op.g.ho);
    op.dkw = FastDiv(s.kw);
    op.dkh = FastDiv(s.kh);
    op.ws = nullptr;
    bool vec = false;
    if (!nchw) {
        if (s.kh == 1 && s.kw == 1) {
            vec = s.c % 4 == 0 && aligned16(x);
        } else if (const float *xt = transposed(SLOT_ACT, x, s.b, (long long) s.h * s.w, s.c, st)) {
            op.x = xt;
            op.xl = 1;
        }
    } else if (const float *wt = transposed(SLOT_WGT, w, 1, s.kn, op.g.K, st)) {
        op.w = wt;
        op.wl = 0;
    }
    op.ov = !nchw && s.kn % 4 == 0 && aligned16(y);
    const bool bv = op.wl == 0 && s.kn % 4 == 0 && aligned16(op.w);
    return launch_split_or_fused(op, (int) op.g.P, op.g.kn, vec, bv, st);
}

size_t cg_fp32_wgrad_ws_bytes(const cg_shape &s) {
    ConvGeom g = make_geom(s);
    long long nblocks = (g.P + KC - 1) / KC;
    return sizeof(float) * (size_t) nblocks * (size_t) g.K * (size_t) g.kn;
}

cudaError_t cg_fp32_wgrad(int nchw, const cg_shape &s, const float *dy, const float *x, float *dw, float *ws,
                          cudaStream_t st) {
    std::lock_guard<std::mutex> call_lock(g_call_mu);
    WgradOp op;
    op.g = make_geom(s);
    if (!offsets_fit(op.g)) return cudaErrorNotSupported;
    op.xl = op.yl = nchw;
    op.dy = dy;
    op.x = x;
    op.ws = ws;
    op.dwo = FastDiv(op.g.wo);
    op.dho = FastDiv(op.g.ho);
    op.dkw = FastDiv(s.kw);
    op.dkh = FastDiv(s.kh);
    if (nchw) {
        // NCHW dy strides the tile's columns (output channels) by ho*wo: read an NHWC copy, and
        // for a single tap, whose rows are input channels, an NHWC copy of x as well
        if (const float *t = transposed(SLOT_ACT, dy, s.b, s.kn, (long long) op.g.ho * op.g.wo, st)) {
            op.dy = t;
            op.yl = 0;
        }
        if (s.kh * s.kw == 1)
            if (const float *t = transposed(SLOT_ACT2, x, s.b, s.c, (long long) s.h * s.w, st)) {
                op.x = t;
                op.xl = 0;
            }
    }
    const int nblocks = (int) ((op.g.P + KC - 1) / KC);
    op.ov = s.kn % 4 == 0 && aligned16(ws);
    cudaError_t e = launch(op, nblocks, false, op.yl == 0 && s.kn % 4 == 0 && aligned16(op.dy), st);
    if (e != cudaSuccess) return e;
    const long long total = (long long) op.g.K * op.g.kn;
    int blocks = (int) std::min<long long>((total + 255) / 256, 152LL * 16);
    wgrad_reduce_kernel<<<blocks, 256, 0, st>>>(ws, dw, op.g.K, op.g.kn, nblocks, nchw); cg_note_launch();
    return cudaGetLastError();
}

// Operand layouts as in the forward: a k x k NHWC input gradient reads dy from an NCHW copy,
// a single-tap NHWC one reads dy rows as channel vectors, and the weights are read as
// [tap][kn][c] (a row of B, consecutive input channels at one (tap, output channel), contiguous).
cudaError_t cg_fp32_dgrad(int nchw, const cg_shape &s, const float *w, const float *dy, float *dx, int accumulate,
                          cudaStream_t st) {
    std::lock_guard<std::mutex> call_lock(g_call_mu);
    DgradOp op;
    op.g = make_geom(s);
    if (!offsets_fit(op.g)) return cudaErrorNotSupported;
    op.nchw = nchw;
    op.accumulate = accumulate;
    op.yl = op.wl = nchw;
    op.w = w;
    op.dy = dy;
    op.dx = dx;
    op.dw_ = FastDiv(s.w);
    op.dh_ = FastDiv(s.h);
    op.dkn = FastDiv(s.kn);
    op.dkw = FastDiv(s.kw);
    op.dvs = FastDiv(s.vstride);
    op.dhs = FastDiv(s.hstride);
    op.ws = nullptr;
    const int taps = s.kh * s.kw;
    const bool phased = (s.vstride > 1 || s.hstride > 1) && s.vstride * s.hstride <= DG_MAXCLS && taps <= DG_MAXTAPS;
    bool vec = false;
    if (!nchw) {
        if (taps == 1) {
            vec = s.kn % 4 == 0 && aligned16(dy);
        } else if (const float *t = transposed(SLOT_ACT, dy, s.b, (long long) op.g.ho * op.g.wo, s.kn, st)) {
            op.dy = t;
            op.yl = 1;
        }
    }
    // NHWC w is [c][tap*kn], NCHW w is [kn*c][tap]; both transpose to [tap][kn][c]
    const float *wt = nullptr;
    if (!nchw) wt = transposed(SLOT_WGT, w, 1, s.c, (long long) taps * s.kn, st);
    else if (taps > 1) wt = transposed(SLOT_WGT, w, 1, (long long) s.kn * s.c, taps, st);
    if (wt) {
        op.w = wt;
        op.wl = 2;
    } else if (nchw && taps == 1) {
        op.wl = 2;   // [kn][c] is [tap][kn][c] already
    }
    op.ov = !nchw && s.c % 4 == 0 && aligned16(dx);
    const bool bv = op.wl == 2 && s.c % 4 == 0 && aligned16(op.w);
    if (!phased) return launch_split_or_fused(op, op.M(), op.g.c, vec, bv, st);

    DgradPhaseOp po;
    po.g = op.g;
    po.nchw = nchw;
    po.accumulate = accumulate;
    po.yl = op.yl;
    po.wl = op.wl;
    po.ov = op.ov;
    po.w = op.w;
    po.dy = op.dy;
    po.dx = dx;
    po.dkn = FastDiv(s.kn);
    po.nkb = (s.kn + KC - 1) / KC;
    po.ws = nullptr;
    long long m = 0;
    int r = 0, t0 = 0, c = 0;
    for (int xm = 0; xm < s.vstride; xm++)
        for (int ym = 0; ym < s.hstride; ym++, c++) {
            DgPhase &p = po.ph[c];
            p.ih0 = ((xm - s.vpad) % s.vstride + s.vstride) % s.vstride;
            p.iw0 = ((ym - s.hpad) % s.hstride + s.hstride) % s.hstride;
            const int hc = p.ih0 < s.h ? (s.h - p.ih0 + s.vstride - 1) / s.vstride : 0;
            const int wc = p.iw0 < s.w ? (s.w - p.iw0 + s.hstride - 1) / s.hstride : 0;
            p.rows = s.b * hc * wc;
            p.dhc = FastDiv(hc > 0 ? hc : 1);
            p.dwc = FastDiv(wc > 0 ? wc : 1);
            p.mbeg = (int) m;
            p.rbeg = r;
            p.tap0 = t0;
            p.ntaps = 0;
            for (int kx = 0; kx < s.kh; kx++)
                for (int ky = 0; ky < s.kw; ky++)
                    if ((kx * s.vdil) % s.vstride == xm && (ky * s.hdil) % s.hstride == ym)
                        po.taps[t0 + p.ntaps++] = (unsigned char) (kx * s.kw + ky);
            t0 += p.ntaps;
            r += p.ntaps * s.kn;
            m += ((long long) p.rows + 255) / 256 * 256;
        }
    if (m > INT_MAX / 2) return cudaErrorNotSupported;
    po.ncls = c;
    po.mpad = (int) m;
    return launch_split_or_fused(po, po.mpad, s.c, vec && taps == 1, bv, st);
}
