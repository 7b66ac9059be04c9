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
// store.  Tiles are 128x128 outputs per 256-thread CTA, 8x8 per thread,
// reduction slices of 8 double-buffered through shared memory.  The running
// sum of completed KC blocks lives in shared memory (it is touched once per
// 384 reduction steps).
//
// Block split: when a convolution's tiles fill less than the GPU (the 14x14 and 7x7
// layers), the forward and input gradient run one CTA per (tile, reduction segment):
// each CTA writes the FMA chain of one KC block (input gradient: one KC block of one
// tap) to a scratch plane, and a second kernel adds the planes in order and applies
// the epilogue.  The chains start from +0 and so are never -0, hence 0 + chain ==
// chain and the ordered sum of the planes equals the running sum of the fused form
// bit for bit.
#include <climits>
#include <type_traits>
#include <map>
#include <mutex>
#include <utility>
#include <vector>
#include "cg_common.cuh"

namespace {

constexpr int BM = 128, BN = 128, BK = 8, NT = 256;
constexpr int KC = 384;
constexpr int SREGS = 64;  // outputs per thread
constexpr size_t S_SMEM_BYTES = sizeof(float) * SREGS * NT;

__device__ __forceinline__ bool in_range(int v, int n) { return (unsigned) v < (unsigned) n; }

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
struct FwdOp {
    ConvGeom g;
    int nchw;
    const float *w, *x;
    float *y;
    cg_epi e;
    FastDiv dwo, dho, dkw, dkh;
    float *ws;   // block split: [K blocks][P][kn] chains, else NULL

    __host__ __device__ int M() const { return (int) g.P; }
    __host__ __device__ int N() const { return g.kn; }

    struct Row { int valid, bb, bix, biy; };
    __device__ Row row(int m) const {
        Row rw;
        rw.valid = m < (int) g.P;
        uint32_t q, oy, ox, bb;
        dwo.divmod(rw.valid ? m : 0, q, oy);
        dho.divmod(q, bb, ox);
        rw.bb = bb;
        rw.bix = ox * g.vstr - g.vpad;
        rw.biy = oy * g.hstr - g.hpad;
        return rw;
    }
    struct Col { int valid, n; };
    __device__ Col col(int n) const { return Col{n < g.kn, n}; }
    struct RI { int valid, c, offx, offy, r; };
    __device__ RI rinfo(int r, int rend) const {
        RI ri;
        ri.valid = r < rend;
        ri.r = r;
        uint32_t t, ky, kx, c;
        dkw.divmod(ri.valid ? r : 0, t, ky);
        dkh.divmod(t, c, kx);
        ri.c = c;
        ri.offx = kx * g.vdil;
        ri.offy = ky * g.hdil;
        return ri;
    }
    __device__ float a(const Row &rw, const RI &ri) const {
        int ix = rw.bix + ri.offx, iy = rw.biy + ri.offy;
        if (!(rw.valid && ri.valid && in_range(ix, g.h) && in_range(iy, g.w))) return 0.0f;
        size_t o = nchw ? ((((size_t) rw.bb * g.c + ri.c) * g.h + ix) * g.w + iy)
                        : ((((size_t) rw.bb * g.h + ix) * g.w + iy) * g.c + ri.c);
        return __ldg(x + o);
    }
    __device__ float b(const Col &cl, const RI &ri) const {
        if (!(cl.valid && ri.valid)) return 0.0f;
        size_t o = nchw ? ((size_t) cl.n * g.K + ri.r) : ((size_t) ri.r * g.kn + cl.n);
        return __ldg(w + o);
    }
    __host__ __device__ int segments() const { return (g.K + KC - 1) / KC; }
    __device__ void range(int z, int &rbeg, int &rend) const {
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
    __device__ void finish_z(int z, int m, int n, float s) const {
        if (!ws) return finish(m, n, s);
        if (m < (int) g.P && n < g.kn) ws[((size_t) z * g.P + m) * g.kn + n] = s;
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
// the workspace, and wgrad_reduce adds the blocks in increasing order.
struct WgradOp {
    ConvGeom g;
    int nchw;
    const float *dy, *x;
    float *ws;   // [nblocks][K][kn]
    FastDiv dwo, dho, dkw, dkh, dhw;

    __host__ __device__ int M() const { return g.K; }
    __host__ __device__ int N() const { return g.kn; }

    struct Row { int valid, c, offx, offy; };
    __device__ Row row(int m) const {
        Row rw;
        rw.valid = m < g.K;
        uint32_t t, ky, kx, c;
        dkw.divmod(rw.valid ? m : 0, t, ky);
        dkh.divmod(t, c, kx);
        rw.c = c;
        rw.offx = kx * g.vdil;
        rw.offy = ky * g.hdil;
        return rw;
    }
    struct Col { int valid, n; };
    __device__ Col col(int n) const { return Col{n < g.kn, n}; }
    struct RI { int valid, bb, bix, biy, q, r; };
    __device__ RI rinfo(int r, int rend) const {
        RI ri;
        ri.valid = r < rend;
        ri.r = r;
        uint32_t q, oy, ox, bb;
        dwo.divmod(ri.valid ? r : 0, q, oy);
        dho.divmod(q, bb, ox);
        ri.bb = bb;
        ri.q = ox * g.wo + oy;
        ri.bix = ox * g.vstr - g.vpad;
        ri.biy = oy * g.hstr - g.hpad;
        return ri;
    }
    __device__ float a(const Row &rw, const RI &ri) const {
        int ix = ri.bix + rw.offx, iy = ri.biy + rw.offy;
        if (!(rw.valid && ri.valid && in_range(ix, g.h) && in_range(iy, g.w))) return 0.0f;
        size_t o = nchw ? ((((size_t) ri.bb * g.c + rw.c) * g.h + ix) * g.w + iy)
                        : ((((size_t) ri.bb * g.h + ix) * g.w + iy) * g.c + rw.c);
        return __ldg(x + o);
    }
    __device__ float b(const Col &cl, const RI &ri) const {
        if (!(cl.valid && ri.valid)) return 0.0f;
        size_t o = nchw ? (((size_t) ri.bb * g.kn + cl.n) * ((size_t) g.ho * g.wo) + ri.q)
                        : ((size_t) ri.r * g.kn + cl.n);
        return __ldg(dy + o);
    }
    __device__ void range(int z, int &rbeg, int &rend) const {
        rbeg = z * KC;
        rend = min((long long) (z + 1) * KC, g.P);
    }
    __device__ int next_fold(int r, int rend) const { return INT_MAX; }
    __device__ float s_init(int m, int n) const { return 0.0f; }
    __device__ void finish_z(int z, int m, int n, float s) const {
        if (m >= g.K || n >= g.kn) return;
        ws[((size_t) z * g.K + m) * g.kn + n] = s;
    }
};

// ---------------------------------------------------------- input gradient
// Gather form: rows m = input pixel (b, ih, iw), columns n = input channel,
// reduction r = tap*kn + l over taps (kx, ky) and output channels l.  A tap
// contributes where (ih + vpad - kx*vdil) is a non-negative multiple of the
// stride below ho (same for iy).  Each (tap, KC block of l) partial is added
// to the running value in a fixed order; the reference adds the same partials
// with `omp atomic` in thread order (src/im2row_nhwc.c:252).
struct DgradOp {
    ConvGeom g;
    int nchw, accumulate;
    const float *w, *dy;
    float *dx;
    FastDiv dw_, dh_, dkn, dkw, dvs, dhs;
    float *ws;   // block split: [segment][b*h*w][c] chains (segment = tap, KC block of kn), else NULL

    __host__ __device__ int M() const { return g.b * g.h * g.w; }
    __host__ __device__ int N() const { return g.c; }

    struct Row { int valid, bb, tx0, ty0; };
    __device__ Row row(int m) const {
        Row rw;
        rw.valid = m < g.b * g.h * g.w;
        uint32_t q, iw, ih, bb;
        dw_.divmod(rw.valid ? m : 0, q, iw);
        dh_.divmod(q, bb, ih);
        rw.bb = bb;
        rw.tx0 = ih + g.vpad;
        rw.ty0 = iw + g.hpad;
        return rw;
    }
    struct Col { int valid, n; };
    __device__ Col col(int n) const { return Col{n < g.c, n}; }
    struct RI { int valid, l, kx, ky; };
    __device__ RI rinfo(int r, int rend) const {
        RI ri;
        ri.valid = r < rend;
        uint32_t tap, l, kx, ky;
        dkn.divmod(ri.valid ? r : 0, tap, l);
        dkw.divmod(tap, kx, ky);
        ri.l = l;
        ri.kx = kx;
        ri.ky = ky;
        return ri;
    }
    __device__ float a(const Row &rw, const RI &ri) const {
        int tx = rw.tx0 - ri.kx * g.vdil, ty = rw.ty0 - ri.ky * g.hdil;
        if (!(rw.valid && ri.valid) || tx < 0 || ty < 0) return 0.0f;
        uint32_t ox, rx, oy, ry;
        dvs.divmod(tx, ox, rx);
        dhs.divmod(ty, oy, ry);
        if (rx || ry || (int) ox >= g.ho || (int) oy >= g.wo) return 0.0f;
        size_t o = nchw ? ((((size_t) rw.bb * g.kn + ri.l) * g.ho + ox) * g.wo + oy)
                        : ((((size_t) rw.bb * g.ho + ox) * g.wo + oy) * g.kn + ri.l);
        return __ldg(dy + o);
    }
    __device__ float b(const Col &cl, const RI &ri) const {
        if (!(cl.valid && ri.valid)) return 0.0f;
        size_t k = ((size_t) cl.n * g.kh + ri.kx) * g.kw + ri.ky;
        size_t o = nchw ? ((size_t) ri.l * g.K + k) : (k * g.kn + ri.l);
        return __ldg(w + o);
    }
    __host__ __device__ int segments() const { return g.kh * g.kw * ((g.kn + KC - 1) / KC); }
    __device__ void range(int z, int &rbeg, int &rend) const {
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
    __device__ void finish_z(int z, int m, int n, float s) const {
        if (!ws) return finish(m, n, s);
        if (m < M() && n < g.c) ws[((size_t) z * M() + m) * g.c + n] = s;
    }
    __device__ void finish(int m, int n, float s) const {
        if (m >= M() || n >= g.c) return;
        dx[out_index(m, n)] = s;
    }
};


template <class Op>
__global__ void __launch_bounds__(NT) fp32_igemm_kernel(const Op op) {
    __shared__ __align__(16) float As[2][BK][BM];
    __shared__ __align__(16) float Bs[2][BK][BN];
    extern __shared__ float Ssm[];  // [SREGS][NT], running sum of completed KC blocks

    const int tid = threadIdx.x;
    const int m0 = blockIdx.x * BM;
    const int n0 = blockIdx.y * BN;
    const int z = blockIdx.z;
    int rbeg, rend;
    op.range(z, rbeg, rend);

    // loader mapping: element (lk + 2i, lm) of each 8x128 slice
    const int lm = tid & 127, lk = tid >> 7;
    const auto arow = op.row(m0 + lm);
    const auto bcol = op.col(n0 + lm);
    float ra[4], rb[4];

    // compute mapping: rows {ty*4+i, 64+ty*4+i}, columns {tx*4+j, 64+tx*4+j}
    const int tx = tid & 15, ty = tid >> 4;
    auto mrow = [&](int i) { return m0 + (i < 4 ? ty * 4 + i : 64 + ty * 4 + i - 4); };
    auto ncol = [&](int j) { return n0 + (j < 4 ? tx * 4 + j : 64 + tx * 4 + j - 4); };

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

    auto gload = [&](int r0) {
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const auto ri = op.rinfo(r0 + lk + 2 * i, rend);
            ra[i] = op.a(arow, ri);
            rb[i] = op.b(bcol, ri);
        }
    };
    auto sstore = [&](int buf) {
#pragma unroll
        for (int i = 0; i < 4; i++) {
            As[buf][lk + 2 * i][lm] = ra[i];
            Bs[buf][lk + 2 * i][lm] = rb[i];
        }
    };

    const int ntiles = (rend - rbeg + BK - 1) / BK;
    int next_fold = op.next_fold(rbeg, rend);
    gload(rbeg);
    sstore(0);
    __syncthreads();
    for (int t = 0; t < ntiles; t++) {
        const int buf = t & 1;
        if (t + 1 < ntiles) gload(rbeg + (t + 1) * BK);
#pragma unroll
        for (int kk = 0; kk < BK; kk++) {
            const int r = rbeg + t * BK + kk;
            if (r == next_fold) {
                fold();
                next_fold = op.next_fold(r, rend);
            }
            const float4 a0 = *reinterpret_cast<const float4 *>(&As[buf][kk][ty * 4]);
            const float4 a1 = *reinterpret_cast<const float4 *>(&As[buf][kk][64 + ty * 4]);
            const float4 b0 = *reinterpret_cast<const float4 *>(&Bs[buf][kk][tx * 4]);
            const float4 b1 = *reinterpret_cast<const float4 *>(&Bs[buf][kk][64 + tx * 4]);
            const float av[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
            const float bv[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
            for (int i = 0; i < 8; i++)
#pragma unroll
                for (int j = 0; j < 8; j++) acc[i][j] = __fmaf_rn(av[i], bv[j], acc[i][j]);
        }
        if (t + 1 < ntiles) sstore(buf ^ 1);
        __syncthreads();
    }
    fold();

#pragma unroll
    for (int i = 0; i < 8; i++)
#pragma unroll
        for (int j = 0; j < 8; j++) {
            const float s = Ssm[(i * 8 + j) * NT + tid];
            op.finish_z(z, mrow(i), ncol(j), s);
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
        float s;
        if constexpr (std::is_same<Op, DgradOp>::value) s = op.s_start(m, n);
        else s = 0.0f;
        int z = 0;
        for (; z + 8 <= nz; z += 8) {
            float v[8];
#pragma unroll
            for (int j = 0; j < 8; j++) v[j] = ws[(size_t) (z + j) * total + i];
#pragma unroll
            for (int j = 0; j < 8; j++) s = __fadd_rn(s, v[j]);
        }
        for (; z < nz; z++) s = __fadd_rn(s, ws[(size_t) z * total + i]);
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

template <class Op>
cudaError_t launch(const Op &op, int gz, cudaStream_t st) {
    static bool attr_set = false;  // per template instance; harmless if set twice
    if (!attr_set) {
        cudaError_t e = cudaFuncSetAttribute(fp32_igemm_kernel<Op>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int) S_SMEM_BYTES);
        if (e != cudaSuccess) return e;
        attr_set = true;
    }
    dim3 grid((op.M() + BM - 1) / BM, (op.N() + BN - 1) / BN, gz);
    if (grid.x == 0 || grid.y == 0) return cudaSuccess;
    fp32_igemm_kernel<Op><<<grid, NT, S_SMEM_BYTES, st>>>(op); cg_note_launch();
    return cudaGetLastError();
}

// Scratch planes of the block split, one grow-only buffer per (device, stream): a CUDA graph
// that captured a buffer keeps using it, so buffers are never freed or reused for another stream.
std::mutex g_split_mu;
std::map<std::pair<int, cudaStream_t>, std::pair<float *, size_t>> g_split_ws;
constexpr size_t SPLIT_WS_MAX = (size_t) 256 << 20;

float *split_scratch(size_t bytes, cudaStream_t st) {
    if (bytes > SPLIT_WS_MAX) return nullptr;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
    std::lock_guard<std::mutex> lk(g_split_mu);
    auto &e = g_split_ws[{dev, st}];
    if (e.second >= bytes) return e.first;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) {
        cudaGetLastError();
        return nullptr;   // no allocation under capture: the fused form runs instead
    }
    size_t want = e.second ? e.second : ((size_t) 32 << 20);
    while (want < bytes) want *= 2;
    if (want > SPLIT_WS_MAX) want = SPLIT_WS_MAX;
    float *p = nullptr;
    if (cudaMalloc(&p, want) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    e = {p, want};   // the previous buffer stays allocated for graphs that captured it
    return p;
}

// The block split pays when the fused grid leaves SMs idle (two 128x128 CTAs fit per SM).
template <class Op>
cudaError_t launch_split_or_fused(Op op, int M, int N, cudaStream_t st) {
    const long long tiles = (long long) ((M + BM - 1) / BM) * ((N + BN - 1) / BN);
    const int nz = op.segments();
    int sms = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    op.ws = nullptr;
    if (nz > 1 && tiles < 2LL * sms) {
        const size_t bytes = sizeof(float) * (size_t) nz * (size_t) M * (size_t) N;
        op.ws = split_scratch(bytes, st);
    }
    if (!op.ws) return launch(op, 1, st);
    cudaError_t e = launch(op, nz, st);
    if (e != cudaSuccess) return e;
    const long long total = (long long) M * N;
    const int blocks = (int) std::min<long long>((total + 255) / 256, (long long) sms * 16);
    float *ws = op.ws;
    fp32_split_reduce_kernel<Op><<<blocks, 256, 0, st>>>(op, ws, nz, M, N); cg_note_launch();
    return cudaGetLastError();
}

}  // namespace

cudaError_t cg_fp32_fwd(int nchw, const cg_shape &s, const float *w, const float *x, float *y,
                        const cg_epi &e, cudaStream_t st) {
    FwdOp op;
    op.g = make_geom(s);
    op.nchw = nchw;
    op.w = w;
    op.x = x;
    op.y = y;
    op.e = e;
    op.dwo = FastDiv(op.g.wo);
    op.dho = FastDiv(op.g.ho);
    op.dkw = FastDiv(s.kw);
    op.dkh = FastDiv(s.kh);
    op.ws = nullptr;
    return launch_split_or_fused(op, (int) op.g.P, op.g.kn, st);
}

size_t cg_fp32_wgrad_ws_bytes(const cg_shape &s) {
    ConvGeom g = make_geom(s);
    long long nblocks = (g.P + KC - 1) / KC;
    return sizeof(float) * (size_t) nblocks * (size_t) g.K * (size_t) g.kn;
}

cudaError_t cg_fp32_wgrad(int nchw, const cg_shape &s, const float *dy, const float *x, float *dw, float *ws,
                          cudaStream_t st) {
    WgradOp op;
    op.g = make_geom(s);
    op.nchw = nchw;
    op.dy = dy;
    op.x = x;
    op.ws = ws;
    op.dwo = FastDiv(op.g.wo);
    op.dho = FastDiv(op.g.ho);
    op.dkw = FastDiv(s.kw);
    op.dkh = FastDiv(s.kh);
    op.dhw = FastDiv(op.g.ho * op.g.wo);
    const int nblocks = (int) ((op.g.P + KC - 1) / KC);
    cudaError_t e = launch(op, nblocks, st);
    if (e != cudaSuccess) return e;
    const long long total = (long long) op.g.K * op.g.kn;
    int blocks = (int) std::min<long long>((total + 255) / 256, 152LL * 16);
    wgrad_reduce_kernel<<<blocks, 256, 0, st>>>(ws, dw, op.g.K, op.g.kn, nblocks, nchw); cg_note_launch();
    return cudaGetLastError();
}

cudaError_t cg_fp32_dgrad(int nchw, const cg_shape &s, const float *w, const float *dy, float *dx, int accumulate,
                          cudaStream_t st) {
    DgradOp op;
    op.g = make_geom(s);
    op.nchw = nchw;
    op.accumulate = accumulate;
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
    return launch_split_or_fused(op, op.M(), op.g.c, st);
}
