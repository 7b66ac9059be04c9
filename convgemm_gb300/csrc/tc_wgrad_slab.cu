// BF16 weight gradient of stride-1 convolutions with 128-channel input blocks from input
// slabs: the transposed GEMM of sconvGemmNHWC('T') (src/convGemm.c:71-76) for those shapes,
//     dW[tap][ci][co] = sum over output pixels p of X[p + shift(tap)][ci] * dY[p][co].
//
// The general weight-gradient kernel loads one im2col box per tap and 64 pixels, so each
// input pixel crosses L2 -> shared memory kh*kw times per output-channel tile, and its MMAs
// wait on those loads.  Here a CTA owns one kernel row dy, a pair of 64-channel input blocks
// and one tile of BN output channels, and walks bands of R whole output rows:
//   * per band, one TMA load per input block brings the R input rows that kernel row dy
//     reads, Wp = wo + (kw - 1) * hdil columns wide (the padding columns and rows outside the
//     image are zero fill), one 128-byte swizzled row per pixel: slab row i * Wp + j;
//   * one TMA load per 64 output channels brings dY of the band with the same pitch Wp: its
//     columns j >= wo lie outside dY and arrive as zeros, so they add nothing;
//   * the tap (dy, dx) operand is the slab read from row dx * hdil on: an MN-major SW128
//     operand (channels along M, pixels along K) whose two 64-channel atoms are the two input
//     blocks (descriptor LBO = the distance between the two slabs).  The swizzle is
//     address-based, so a start at any whole row reads the right data;
//   * kw accumulators of 128 x BN FP32 in TMEM, one per dx: per 16-pixel step, kw MMAs share
//     the dY operand;
//   * rows past the band's R * Wp up to the last 16-row step (and the dx overreach of the
//     slab) are zero: TMA never writes them and the kernel clears them once.
// Each input pixel crosses L2 -> shared memory kh times per output-channel tile and each dY
// pixel kh * (input blocks / 2) times, in a few large boxes per band.  Each CTA writes one
// FP32 partial of its (dy, input-block pair, output-channel tile) to the workspace in the
// general kernel's dY-on-A layout [split][co][tap * Cp + ci] (a warp's lanes hold consecutive
// input channels, so each column is one 128-byte store), and the general kernel's fixed-order
// reduction adds the splits (with one split the CTA writes dW itself).
#include <cstring>

#include <cuda_bf16.h>

#include "cg_common.cuh"
#include "tc_host.h"
#include "tc_ptx.cuh"
#include "tc_wgrad.h"

namespace {

constexpr int WS_MAXST = 8;
constexpr size_t WS_SMEM_MAX = 232448;   // the per-block opt-in maximum

struct WsParams {
    float *ws;                 // partials [split][kn][Nx] (the dY-on-A layout of the general kernel)
    float *dw;                 // direct (one split): dW in the reference layout `layout`
    int direct, layout, C;
    int kn, Cp, Nx, kh, kw, hdil, vdil, padh, padw;
    int R, Wp, bands_per_img, total_bands, bands_per_split;
    int ncp, nct;              // input-block pairs, output-channel tiles
    int ksteps;                // 16-row K steps per band
    int stages;
    int niss;                  // MMA-issuing threads (lane 0 of warps 1..niss), min(kw, 3)
    uint32_t x_bytes, dy_bytes, stage_bytes;   // one slab / one dY atom buffer, one stage
    uint32_t x_box_rows;       // rows one TMA box writes (R * Wp)
    int *err;
};

template <int BN>
__global__ void __launch_bounds__(128, 2)
    tc_wgrad_slab_kernel(const __grid_constant__ WsParams p, const __grid_constant__ CUtensorMap xmap,
                         const __grid_constant__ CUtensorMap dymap) {
    constexpr int DYA = BN / 64;   // dY atoms
    extern __shared__ uint8_t smem_raw[];
    uint8_t *base = (uint8_t *) (((uintptr_t) smem_raw + 1023) & ~(uintptr_t) 1023);
    uint64_t *full = (uint64_t *) (base + (size_t) p.stages * p.stage_bytes);
    uint64_t *empty = full + WS_MAXST;
    uint64_t *accum = empty + WS_MAXST;
    uint32_t *tmem_holder = (uint32_t *) (accum + 1);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    // unit: (kernel row dy, input-block pair cp, output-channel tile ct); split: a band range
    const int unit = blockIdx.x;
    const int ct = unit % p.nct, cp = (unit / p.nct) % p.ncp, dy = unit / (p.nct * p.ncp);
    const int band0 = blockIdx.y * p.bands_per_split;
    const int nb = min(p.bands_per_split, p.total_bands - band0);

    // rows that TMA never writes but the MMAs read: zero once (generic writes, then the fence
    // that makes them visible to the tensor core's async proxy)
    {
        const uint32_t box_bytes = p.x_box_rows * 128;
        for (int s = 0; s < p.stages; s++) {
            uint8_t *st = base + (size_t) s * p.stage_bytes;
            for (int a = 0; a < 2 + DYA; a++) {
                uint8_t *buf = a < 2 ? st + a * p.x_bytes : st + 2 * p.x_bytes + (a - 2) * p.dy_bytes;
                const uint32_t len = a < 2 ? p.x_bytes : p.dy_bytes;
                for (uint32_t o = box_bytes + 16 * threadIdx.x; o < len; o += 16 * 128)
                    *reinterpret_cast<uint4 *>(buf + o) = make_uint4(0, 0, 0, 0);
            }
        }
        tc::fence_proxy_async_smem();
    }
    if (threadIdx.x == 0) {
        for (int s = 0; s < p.stages; s++) {
            tc::mbar_init(&full[s], 1);
            tc::mbar_init(&empty[s], p.niss);
        }
        tc::mbar_init(accum, p.niss);
        tc::fence_mbar_init();
        tc::prefetch_tmap(&xmap);
        tc::prefetch_tmap(&dymap);
    }
    uint32_t tcols = 32;   // kw accumulators of BN columns (kw * BN <= 512), a power of two
    while (tcols < (uint32_t) (p.kw * BN)) tcols <<= 1;
    if (warp == 2) {
        tc::tmem_alloc(tmem_holder, tcols);
        tc::tmem_relinquish();
    }
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tmem = *tmem_holder;
    bool ok = true;

    if (warp == 0 && lane == 0) {
        // producer: per band two input slabs and DYA dY atoms
        const uint32_t tx = 2 * p.x_box_rows * 128 + DYA * p.x_box_rows * 128;
        for (int i = 0; i < nb; i++) {
            const int s = i % p.stages;
            const uint32_t ph = (i / p.stages) & 1;
            if (i >= p.stages && !(ok = tc::mbar_wait(&empty[s], ph ^ 1, p.err, 41))) break;
            const int band = band0 + i;
            const int b = band / p.bands_per_img, oy0 = (band % p.bands_per_img) * p.R;
            const uint32_t st = tc::smem_u32(base + (size_t) s * p.stage_bytes);
            tc::mbar_arrive_expect_tx(&full[s], tx);
#pragma unroll
            for (int a = 0; a < 2; a++)
                tc::tma_load_4d(st + a * p.x_bytes, &xmap, cp * 128 + 64 * a, -p.padw, oy0 + dy * p.vdil - p.padh, b,
                                &full[s]);
#pragma unroll
            for (int a = 0; a < DYA; a++)
                tc::tma_load_4d(st + 2 * p.x_bytes + a * p.dy_bytes, &dymap, ct * BN + 64 * a, 0, oy0, b, &full[s]);
        }
    } else if (warp >= 1 && warp <= p.niss && lane == 0) {
        // MMA issuers (warps 1..niss): issuer j takes the accumulators dx = j, j + niss, ...;
        // each waits for the band, issues its MMAs and commits once to the band's empty barrier
        // (count niss).  One thread's tcgen05 issue, barrier wait and commit cost tens of cycles
        // each, so a single issuer cannot keep kw accumulators of short bands busy.
        constexpr uint32_t idesc = tc::idesc_bf16(128, BN, 1, 1);
        const int j = warp - 1;
        for (int i = 0; i < nb; i++) {
            const int s = i % p.stages;
            const uint32_t ph = (i / p.stages) & 1;
            if (!(ok = tc::mbar_wait(&full[s], ph, p.err, 42))) break;
            tc::tc_fence_after();
            const uint32_t st = tc::smem_u32(base + (size_t) s * p.stage_bytes);
            const uint64_t a0 = tc::sw128_desc(st, p.x_bytes, 1024);
            const uint64_t b0 = tc::sw128_desc(st + 2 * p.x_bytes, p.dy_bytes, 1024);
            for (int k = 0; k < p.ksteps; k++) {
                // 16 rows of 128 B = 2048 B = 128 units of the descriptor's start field
                const uint64_t bd = b0 + (uint64_t) (128 * k);
                for (int dx = j; dx < p.kw; dx += p.niss)
                    tc::mma_f16(tmem + (uint32_t) (dx * BN), a0 + (uint64_t) (128 * k + 8 * dx * p.hdil), bd, idesc,
                                (i | k) != 0);
            }
            tc::mma_commit(&empty[s]);
        }
        tc::mma_commit(&accum[0]);
    }
    __syncwarp();

    // epilogue: all four warps; warp w holds TMEM lanes 32w..32w+31 = input channels
    if (ok) ok = tc::mbar_wait(accum, 0, p.err, 43);
    tc::tc_fence_after();
    if (ok && nb > 0) {
        const int ci = cp * 128 + warp * 32 + lane;   // < Cp (Cp is a multiple of 128)
        const int khw = p.kh * p.kw;
        for (int dx = 0; dx < p.kw; dx++) {
            const int tap = dy * p.kw + dx;
            const int n = tap * p.Cp + ci;
#pragma unroll 1
            for (int c0 = 0; c0 < BN; c0 += 32) {
                uint32_t v[32];
                tc::tmem_ld_32x32b_x32(tmem + ((uint32_t) (warp * 32) << 16) + (uint32_t) (dx * BN + c0), v);
                tc::tmem_ld_wait();
                const int co0 = ct * BN + c0;
                if (co0 >= p.kn) continue;
                if (p.direct) {
                    if (ci >= p.C) continue;
#pragma unroll
                    for (int j = 0; j < 32; j++) {
                        const int co = co0 + j;
                        const size_t o = p.layout == 0 ? ((size_t) ci * khw + tap) * p.kn + co
                                                       : ((size_t) co * p.C + ci) * khw + tap;
                        if (co < p.kn) p.dw[o] = __uint_as_float(v[j]);
                    }
                } else {
                    // partial [split][co][n]: for each column the warp's 32 lanes write 32 consecutive n
                    float *col = p.ws + ((size_t) blockIdx.y * p.kn + co0) * p.Nx + n;
#pragma unroll
                    for (int j = 0; j < 32; j++)
                        if (co0 + j < p.kn) col[(size_t) j * p.Nx] = __uint_as_float(v[j]);
                }
            }
        }
    }
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    if (warp == 2) tc::tmem_dealloc(tmem, tcols);
}

struct WsGeom {
    int bn, R, Wp, bands_per_img, ksteps, stages, ncp, nct, units, splits, bands_per_split, total_bands;
    uint32_t x_bytes, dy_bytes, stage_bytes;
    size_t smem;
};

inline uint32_t up1024(uint32_t v) { return (v + 1023) / 1024 * 1024; }

// The band height R (whole output rows) that wastes the fewest MMA rows -- the dY columns past
// wo, the padding of each band to whole 16-row steps and the rows past the image in the last
// band -- with at least three ring stages in shared memory (two when no band fits three),
// preferring bands of at least four 16-row steps; between bands that waste the same, the
// smallest (the most stages in flight).  With 64-wide
// output tiles (three accumulators fit 256 TMEM columns) the ring is sized for two CTAs per SM.
bool ws_geom(const cg_shape &s, int want_splits, int want_bn, WsGeom &w) {
    if (s.vstride != 1 || s.hstride != 1) return false;
    const int Cp = (s.c + 7) / 8 * 8;
    if (Cp % 128 || s.kh < 1 || s.kw < 2 || s.kn < 64) return false;
    const ConvGeom g = make_geom(s);
    if (g.ho < 1 || g.wo < 1) return false;
    w.bn = want_bn == 64 || want_bn == 128 ? want_bn : (s.kn <= 64 ? 64 : 128);
    if (s.kw * w.bn > 512) return false;
    w.Wp = g.wo + (s.kw - 1) * s.hdil;
    if (w.Wp > 256) return false;
    const int dya = w.bn / 64;
    double best = 0.0;
    w.R = 0;
    for (int min_st = 3; min_st >= 2 && !w.R; min_st--) {
        for (int R = 1; R <= 64 && R <= g.ho; R++) {
            const int rows = R * w.Wp;
            const int ks = (rows + 15) / 16;
            const uint32_t xb = up1024((uint32_t) (ks * 16 + (s.kw - 1) * s.hdil) * 128);
            const uint32_t db = (uint32_t) ks * 16 * 128;
            const uint32_t sb = 2 * xb + dya * db;
            const size_t smem = 1024 + (size_t) min_st * sb + 256;
            if (smem > WS_SMEM_MAX || rows > 256 * 256) continue;
            const int bpi = (g.ho + R - 1) / R;
            // MMA rows that carry output pixels, less 3% for bands of fewer than 4 K steps (each
            // band costs every issuer a barrier wait and a commit); between equal ones the first
            // (smallest) band, which leaves the most stages in flight
            const double eff = (double) g.ho * g.wo / ((double) bpi * ks * 16) - (ks < 4 ? 0.03 : 0.0);
            if (eff > best + 1e-6) {
                best = eff;
                w.R = R;
                w.ksteps = ks;
                w.x_bytes = xb;
                w.dy_bytes = db;
                w.stage_bytes = sb;
                w.bands_per_img = bpi;
            }
        }
    }
    if (!w.R) return false;
    const size_t budget = (w.bn == 64 && s.kw * 64 <= 256) ? WS_SMEM_MAX / 2 - 1024 : WS_SMEM_MAX;
    w.stages = (int) ((budget - 1024 - 256) / w.stage_bytes);
    if (w.stages < 2) w.stages = (int) ((WS_SMEM_MAX - 1024 - 256) / w.stage_bytes);
    if (w.stages > WS_MAXST) w.stages = WS_MAXST;
    w.smem = 1024 + (size_t) w.stages * w.stage_bytes + 256;
    w.ncp = Cp / 128;
    w.nct = (s.kn + w.bn - 1) / w.bn;
    w.units = s.kh * w.ncp * w.nct;
    w.total_bands = s.b * w.bands_per_img;
    int splits = want_splits;
    if (splits <= 0) {
        // one wave of CTAs (two per SM with 64-wide tiles), at least two bands per split
        const size_t smem1 = 1024 + (size_t) w.stages * w.stage_bytes + 256;
        splits = tc_num_sms() * (2 * smem1 <= WS_SMEM_MAX && w.bn * s.kw <= 256 ? 2 : 1) / w.units;
        if (splits > w.total_bands / 2) splits = w.total_bands / 2;
    }
    if (splits > w.total_bands) splits = w.total_bands;
    if (splits < 1) splits = 1;
    w.bands_per_split = (w.total_bands + splits - 1) / splits;
    w.splits = (w.total_bands + w.bands_per_split - 1) / w.bands_per_split;
    return true;
}

}  // namespace

int tc_wgrad_slab_splits(const cg_shape &s, int want_splits, int want_bn) {
    WsGeom w;
    return ws_geom(s, want_splits, want_bn, w) ? w.splits : 0;
}

int tc_wgrad_slab_bn(const cg_shape &s, int want_bn) {
    WsGeom w;
    return ws_geom(s, 0, want_bn, w) ? w.bn : 0;
}

convgemm_status_t tc_wgrad_slab_run(const cg_shape &s, int want_splits, int want_bn, const void *dy, const void *x,
                                    float *ws, float *dw, int layout, cudaStream_t st) {
    WsGeom w;
    if (!ws_geom(s, want_splits, want_bn, w))
        return cg_set_error(CONVGEMM_ERROR_NOT_SUPPORTED, "slab weight gradient: shape");
    const ConvGeom g = make_geom(s);
    const int Cp = (s.c + 7) / 8 * 8, kn8 = (s.kn + 7) / 8 * 8;
    WsParams p;
    memset(&p, 0, sizeof(p));
    p.ws = ws;
    p.dw = dw;
    p.direct = w.splits == 1;
    p.layout = layout;
    p.C = s.c;
    p.kn = s.kn;
    p.Cp = Cp;
    p.Nx = s.kh * s.kw * Cp;
    p.kh = s.kh;
    p.kw = s.kw;
    p.hdil = s.hdil;
    p.vdil = s.vdil;
    p.padh = s.vpad;
    p.padw = s.hpad;
    p.R = w.R;
    p.Wp = w.Wp;
    p.bands_per_img = w.bands_per_img;
    p.total_bands = w.total_bands;
    p.bands_per_split = w.bands_per_split;
    p.ncp = w.ncp;
    p.nct = w.nct;
    p.ksteps = w.ksteps;
    p.stages = w.stages;
    p.niss = s.kw < 3 ? s.kw : 3;
    p.x_bytes = w.x_bytes;
    p.dy_bytes = w.dy_bytes;
    p.stage_bytes = w.stage_bytes;
    p.x_box_rows = (uint32_t) (w.R * w.Wp);
    p.err = cg_device_error_word();
    if (!p.err) return cg_set_error(CONVGEMM_ERROR_CUDA, "device error word unavailable");
    CUtensorMap xmap, dymap;
    {   // x [B][H][W][Cp]: box {64 channels, Wp columns, R rows, 1 image}
        const unsigned long long dims[4] = {(unsigned long long) Cp, (unsigned long long) s.w,
                                            (unsigned long long) s.h, (unsigned long long) s.b};
        const unsigned long long str[3] = {2ull * Cp, 2ull * Cp * s.w, 2ull * Cp * s.w * s.h};
        const unsigned box[4] = {64, (unsigned) w.Wp, (unsigned) w.R, 1};
        const unsigned estr[4] = {1, 1, 1, 1};
        if (convgemm_status_t e = tc_make_map_nd(&xmap, 4, x, dims, str, box, estr, 1)) return e;
    }
    {   // dY [B][Ho][Wo][kn8]: box {64 channels, Wp columns (past Wo: zero), R rows, 1 image}
        const unsigned long long dims[4] = {(unsigned long long) kn8, (unsigned long long) g.wo,
                                            (unsigned long long) g.ho, (unsigned long long) s.b};
        const unsigned long long str[3] = {2ull * kn8, 2ull * kn8 * g.wo, 2ull * kn8 * g.wo * g.ho};
        const unsigned box[4] = {64, (unsigned) w.Wp, (unsigned) w.R, 1};
        const unsigned estr[4] = {1, 1, 1, 1};
        if (convgemm_status_t e = tc_make_map_nd(&dymap, 4, dy, dims, str, box, estr, 1)) return e;
    }
    const dim3 grid((unsigned) w.units, (unsigned) w.splits);
    cudaError_t e;
    if (w.bn == 64) {
        static bool attr64 = false;
        if (!attr64) {
            if ((e = cudaFuncSetAttribute(tc_wgrad_slab_kernel<64>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int) WS_SMEM_MAX)))
                return cg_cuda_check(e, "slab weight-gradient attribute");
            attr64 = true;
        }
        e = cg_launch_ex(CG_PDL_OFF, tc_wgrad_slab_kernel<64>, grid, dim3(128), w.smem, st, p, xmap, dymap);
    } else {
        static bool attr128 = false;
        if (!attr128) {
            if ((e = cudaFuncSetAttribute(tc_wgrad_slab_kernel<128>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int) WS_SMEM_MAX)))
                return cg_cuda_check(e, "slab weight-gradient attribute");
            attr128 = true;
        }
        e = cg_launch_ex(CG_PDL_OFF, tc_wgrad_slab_kernel<128>, grid, dim3(128), w.smem, st, p, xmap, dymap);
    }
    if (convgemm_status_t ce = cg_cuda_check(e, "slab weight-gradient launch")) return ce;
    if (p.direct) return CONVGEMM_SUCCESS;
    return cg_cuda_check(tc_wgrad_reduce(ws, dw, w.splits, 0, p.Nx, s.kn, s.c, Cp, s.kh, s.kw, layout, st),
                         "slab weight-gradient reduction");
}
