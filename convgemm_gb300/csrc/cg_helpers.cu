// The reference's explicit lowering helpers on the GPU (FP32), with the
// reference's semantics (src/im2row_nhwc.c:147-229, src/im2col_nchw.c:146-233, 337-359):
//   im2row_nhwc    rows[(b,x,y)][(c,kx,ky)] = in[b][ix][iy][c]; entries whose tap
//                  falls in the padding are left as they are;
//   row2im_nhwc    out[b][ix][iy][c] += rows[...]: here a gather per output element
//                  that adds its contributions in the reference's loop order
//                  (increasing output pixel), so the sums are bit-identical;
//   im2col_nchw    cols[(c,kx,ky)][(b,x,y)] = in[b][c][ix][iy] (padding left as is);
//   col2im_nchw    out[b][c][ix][iy] += cols[...], contributions in increasing (kx, ky);
//   transpose_nchw out[b][k][x][y] = in[k][(b,x,y)] (+ beta * out when beta != 0).
// As in the reference, the ld / m / n arguments of the helpers do not change the
// layout (rows are K = c*kh*kw wide, cols P = b*ho*wo wide), except ld of transpose_nchw.
#include "cg_common.cuh"
#include "cg_internal.h"

namespace {

struct HGeom {
    int b, h, w, c, ho, wo, kh, kw, vpad, hpad, vstr, hstr, vdil, hdil;
};

inline unsigned hgrid(long long n) {
    long long g = (n + 255) / 256;
    return (unsigned) (g > 152 * 64 ? 152 * 64 : (g < 1 ? 1 : g));
}

__global__ void im2row_kernel(float *__restrict__ rows, const float *__restrict__ in, HGeom g) {
    const long long K = (long long) g.c * g.kh * g.kw, total = (long long) g.b * g.ho * g.wo * K;
    for (long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < total; i += (long long) gridDim.x * blockDim.x) {
        const long long row = i / K;
        const int col = (int) (i % K);
        const int c = col / (g.kh * g.kw), r = col % (g.kh * g.kw), kx = r / g.kw, ky = r % g.kw;
        const int y = (int) (row % g.wo), x = (int) ((row / g.wo) % g.ho), b = (int) (row / ((long long) g.wo * g.ho));
        const int ix = g.vstr * x + g.vdil * kx - g.vpad, iy = g.hstr * y + g.hdil * ky - g.hpad;
        if (0 <= ix && ix < g.h && 0 <= iy && iy < g.w) rows[i] = in[(((long long) b * g.h + ix) * g.w + iy) * g.c + c];
    }
}

__global__ void row2im_kernel(const float *__restrict__ rows, float *__restrict__ out, HGeom g) {
    const long long K = (long long) g.c * g.kh * g.kw, total = (long long) g.b * g.h * g.w * g.c;
    for (long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < total; i += (long long) gridDim.x * blockDim.x) {
        const int c = (int) (i % g.c);
        const long long pix = i / g.c;
        const int iy = (int) (pix % g.w), ix = (int) ((pix / g.w) % g.h), b = (int) (pix / ((long long) g.w * g.h));
        float acc = out[i];
        // increasing x = decreasing kx; for each x increasing y = decreasing ky
        for (int kx = g.kh - 1; kx >= 0; kx--) {
            const int t = ix + g.vpad - g.vdil * kx;
            if (t < 0 || t % g.vstr) continue;
            const int x = t / g.vstr;
            if (x >= g.ho) continue;
            for (int ky = g.kw - 1; ky >= 0; ky--) {
                const int u = iy + g.hpad - g.hdil * ky;
                if (u < 0 || u % g.hstr) continue;
                const int y = u / g.hstr;
                if (y >= g.wo) continue;
                acc = __fadd_rn(acc, rows[(((long long) b * g.ho + x) * g.wo + y) * K + (c * g.kh + kx) * g.kw + ky]);
            }
        }
        out[i] = acc;
    }
}

__global__ void im2col_kernel(float *__restrict__ cols, const float *__restrict__ in, HGeom g) {
    const long long P = (long long) g.b * g.ho * g.wo, total = P * g.c * g.kh * g.kw;
    for (long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < total; i += (long long) gridDim.x * blockDim.x) {
        const long long col = i % P;
        const int row = (int) (i / P);
        const int c = row / (g.kh * g.kw), r = row % (g.kh * g.kw), kx = r / g.kw, ky = r % g.kw;
        const int y = (int) (col % g.wo), x = (int) ((col / g.wo) % g.ho), b = (int) (col / ((long long) g.wo * g.ho));
        const int ix = g.vstr * x + g.vdil * kx - g.vpad, iy = g.hstr * y + g.hdil * ky - g.hpad;
        if (0 <= ix && ix < g.h && 0 <= iy && iy < g.w) cols[i] = in[(((long long) b * g.c + c) * g.h + ix) * g.w + iy];
    }
}

__global__ void col2im_kernel(const float *__restrict__ cols, float *__restrict__ out, HGeom g) {
    const long long P = (long long) g.b * g.ho * g.wo, total = (long long) g.b * g.c * g.h * g.w;
    for (long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < total; i += (long long) gridDim.x * blockDim.x) {
        const int iy = (int) (i % g.w), ix = (int) ((i / g.w) % g.h);
        const long long bc = i / ((long long) g.w * g.h);
        const int c = (int) (bc % g.c), b = (int) (bc / g.c);
        float acc = out[i];
        for (int kx = 0; kx < g.kh; kx++) {
            const int t = ix + g.vpad - g.vdil * kx;
            if (t < 0 || t % g.vstr) continue;
            const int x = t / g.vstr;
            if (x >= g.ho) continue;
            for (int ky = 0; ky < g.kw; ky++) {
                const int u = iy + g.hpad - g.hdil * ky;
                if (u < 0 || u % g.hstr) continue;
                const int y = u / g.hstr;
                if (y >= g.wo) continue;
                acc = __fadd_rn(acc, cols[(long long) ((c * g.kh + kx) * g.kw + ky) * P + ((long long) b * g.ho + x) * g.wo + y]);
            }
        }
        out[i] = acc;
    }
}

__global__ void transpose_kernel(int rows, int cols, const float *__restrict__ in, int ld, float beta,
                                 float *__restrict__ out, int kn, int ho, int wo, int start_row, int start_col) {
    const long long total = (long long) rows * cols;
    for (long long t = blockIdx.x * (long long) blockDim.x + threadIdx.x; t < total; t += (long long) gridDim.x * blockDim.x) {
        const int j = (int) (t / rows), i = (int) (t % rows);
        const long long r = (long long) start_row + i;
        const int y = (int) (r % wo), x = (int) ((r / wo) % ho);
        const long long b = r / ((long long) wo * ho);
        const long long idx = ((b * kn + start_col + j) * ho + x) * wo + y;
        const float v = in[(long long) j * ld + i];
        out[idx] = beta == 0.0f ? v : fmaf(beta, out[idx], v);
    }
}

}  // namespace

static HGeom hgeom(int b, int h, int w, int c, int ho, int wo, int kh, int kw, int vpad, int hpad, int vstr, int hstr,
                   int vdil, int hdil) {
    HGeom g = {b, h, w, c, ho, wo, kh, kw, vpad, hpad, vstr, hstr, vdil, hdil};
    return g;
}

cudaError_t cg_helper_im2row(float *rows, const float *in, int b, int h, int w, int c, int ho, int wo, int kh, int kw,
                             int vpad, int hpad, int vstr, int hstr, int vdil, int hdil, cudaStream_t st) {
    const HGeom g = hgeom(b, h, w, c, ho, wo, kh, kw, vpad, hpad, vstr, hstr, vdil, hdil);
    im2row_kernel<<<hgrid((long long) b * ho * wo * c * kh * kw), 256, 0, st>>>(rows, in, g); cg_note_launch();
    return cudaGetLastError();
}
cudaError_t cg_helper_row2im(const float *rows, float *out, int b, int h, int w, int c, int ho, int wo, int kh, int kw,
                             int vpad, int hpad, int vstr, int hstr, int vdil, int hdil, cudaStream_t st) {
    const HGeom g = hgeom(b, h, w, c, ho, wo, kh, kw, vpad, hpad, vstr, hstr, vdil, hdil);
    row2im_kernel<<<hgrid((long long) b * h * w * c), 256, 0, st>>>(rows, out, g); cg_note_launch();
    return cudaGetLastError();
}
cudaError_t cg_helper_im2col(float *cols, const float *in, int b, int c, int h, int w, int ho, int wo, int kh, int kw,
                             int vpad, int hpad, int vstr, int hstr, int vdil, int hdil, cudaStream_t st) {
    const HGeom g = hgeom(b, h, w, c, ho, wo, kh, kw, vpad, hpad, vstr, hstr, vdil, hdil);
    im2col_kernel<<<hgrid((long long) b * ho * wo * c * kh * kw), 256, 0, st>>>(cols, in, g); cg_note_launch();
    return cudaGetLastError();
}
cudaError_t cg_helper_col2im(const float *cols, float *out, int b, int c, int h, int w, int ho, int wo, int kh, int kw,
                             int vpad, int hpad, int vstr, int hstr, int vdil, int hdil, cudaStream_t st) {
    const HGeom g = hgeom(b, h, w, c, ho, wo, kh, kw, vpad, hpad, vstr, hstr, vdil, hdil);
    col2im_kernel<<<hgrid((long long) b * c * h * w), 256, 0, st>>>(cols, out, g); cg_note_launch();
    return cudaGetLastError();
}
cudaError_t cg_helper_transpose(int rows, int cols, const float *in, int ld, float beta, float *out, int kn, int ho,
                                int wo, int start_row, int start_col, cudaStream_t st) {
    transpose_kernel<<<hgrid((long long) rows * cols), 256, 0, st>>>(rows, cols, in, ld, beta, out, kn, ho, wo,
                                                                      start_row, start_col); cg_note_launch();
    return cudaGetLastError();
}
