// BF16 weight gradient of stride-2 convolutions with at most 8 input channels and 64
// output channels (the 7x7/s2 ResNet stem on 224x224 input): the transposed GEMM of
// sconvGemmNHWC('T') (src/convGemm.c:71-76),
//     dW[co][n] = sum over output pixels p of dY[p][co] * X_im2row[p][n],  n = tap*8 + ci,
// for that shape class.
//
// With the channels padded to 8, one tap of one pixel is 16 bytes, and gathering them
// (16-byte cp.async per pixel and tap) bounds the general kernel.  Here the tensor core
// reads its A operand (M = n, K = pixels, MN-major) straight out of input slabs:
//   * a CTA takes bands of SW_R output rows of one image; for every input row of the band
//     (2*(SW_R-1) + kh of them) and each of two column streams, one TMA load with traversal
//     stride 2 brings the slab row
//         S[2*y + st][s] = x[b][2*oy0 - pad_h + y][col0[st] + 2*s][0..7],  s < Wpad + npairs - 1,
//     col0[0] = 1 - pad_w (taps kx = 2m+1), col0[1] = -pad_w (taps kx = 2m), so that tap
//     pair m at output column ox reads entry s = ox + m of both streams;
//   * for output row r of the band, the 16 core matrices (8 kernel rows x 2 streams,
//     8 channels x 8 pixels each, no swizzle) of pair m start at slab row 4*r and are one
//     slab row apart (SBO = the row pitch), 8-pixel K groups 128 bytes apart (LBO): one
//     M=128 MMA per pair and 16-pixel K step, four TMEM accumulators of 64 columns;
//   * slab stages are double-buffered across bands; one MMA-issuing thread per tap pair
//     (one thread's loop overhead between MMAs bounds its issue rate);
//   * dY arrives per output row (64 channels x Wpad pixels, 128-byte swizzle, pixels past
//     Wo zero-filled) through a ring of SW_DYB buffers filled by a second producer warp;
//   * kernel rows >= kh (their slab rows are not loaded: stale data) and taps kx >= kw
//     are computed and dropped;
//   * each CTA writes its FP32 partial [n][co] to the workspace; the fixed-order split
//     reduction of the general kernel adds the partials in CTA order and writes dW.
#include <cstring>

#include <cuda_bf16.h>

#include "cg_common.cuh"
#include "tc_host.h"
#include "tc_ptx.cuh"
#include "tc_wgrad.h"

namespace {

constexpr int SW_R = 8;                          // output rows per band
constexpr int SW_NY = 2 * SW_R + 6;              // slab rows per stream and stage (kernel rows 0..7)
constexpr int SW_MAXPAIRS = 4;                   // kw <= 8
constexpr uint32_t SW_SLAB_MAX = 83 * 1024;      // 2 * SW_NY slab rows of one stage
constexpr int SW_DYB = 3;                        // dY row buffers
constexpr uint32_t SW_DY_MAX = 16 * 1024;        // one output row of dY: Wpad pixels x 128 B
constexpr size_t SW_SMEM = 1024 + 2 * (size_t) SW_SLAB_MAX + SW_DYB * (size_t) SW_DY_MAX + 256;
static_assert(SW_SMEM <= 232448, "shared memory");

struct StemWgParams {
    float *ws;                 // [gridDim.x][Nx][64] FP32 partials, Nx = kh * kw * 8
    int Ho, kh, kw, pad_h, npairs, nks, wpad, nyl;   // nyl: input rows loaded per band
    int bands_per_img, total_bands;
    int col0[2];               // input column of slab entry 0 of stream 0 / 1
    uint32_t pitch;            // bytes per slab row (entries * 16, rounded up to 128)
    uint32_t tx;               // bytes the slab loads of one stage deliver
    int *err;
};

__global__ void __launch_bounds__(320, 1)
    tc_stem_wgrad_kernel(const __grid_constant__ StemWgParams p, const __grid_constant__ CUtensorMap xmap,
                         const __grid_constant__ CUtensorMap dymap) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t *base = (uint8_t *) (((uintptr_t) smem_raw + 1023) & ~(uintptr_t) 1023);
    uint8_t *dyb = base + 2 * SW_SLAB_MAX;   // SW_DYB buffers of SW_DY_MAX (1024-aligned)
    uint64_t *full = (uint64_t *) (dyb + SW_DYB * SW_DY_MAX);
    uint64_t *empty = full + 2;
    uint64_t *dy_full = empty + 2;
    uint64_t *dy_empty = dy_full + SW_DYB;
    uint64_t *accum = dy_empty + SW_DYB;
    uint32_t *tmem_holder = (uint32_t *) (accum + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        // one MMA issuer per tap pair (warps 1, 7, 8, 9) commits to every consumer barrier
        for (int s = 0; s < 2; s++) {
            tc::mbar_init(&full[s], 1);
            tc::mbar_init(&empty[s], SW_MAXPAIRS);
        }
        for (int d = 0; d < SW_DYB; d++) {
            tc::mbar_init(&dy_full[d], 1);
            tc::mbar_init(&dy_empty[d], SW_MAXPAIRS);
        }
        tc::mbar_init(accum, SW_MAXPAIRS);
        tc::fence_mbar_init();
        tc::prefetch_tmap(&xmap);
        tc::prefetch_tmap(&dymap);
    }
    if (warp == 1) {
        tc::tmem_alloc(tmem_holder, 64 * SW_MAXPAIRS);
        tc::tmem_relinquish();
    }
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tmem = *tmem_holder;
    // bands blockIdx.x, blockIdx.x + gridDim.x, ...; the host launches at most total_bands CTAs
    const int nb = (p.total_bands - 1 - (int) blockIdx.x) / (int) gridDim.x + 1;
    bool ok = true;

    if (warp == 0) {
        // ------------------------------------------------ producer: the slab rows of each band
        if (lane == 0) {
            for (int k = 0; k < nb; k++) {
                const int s = k & 1;
                if (k >= 2 && !(ok = tc::mbar_wait(&empty[s], ((k >> 1) + 1) & 1, p.err, 61))) break;
                const int band = (int) blockIdx.x + k * (int) gridDim.x;
                const int b = band / p.bands_per_img, oy0 = (band - b * p.bands_per_img) * SW_R;
                const uint32_t st = tc::smem_u32(base + s * SW_SLAB_MAX);
                tc::mbar_arrive_expect_tx(&full[s], p.tx);
                for (int y = 0; y < p.nyl; y++)
#pragma unroll
                    for (int sm = 0; sm < 2; sm++)
                        tc::tma_load_4d(st + (2 * y + sm) * p.pitch, &xmap, 0, p.col0[sm], 2 * oy0 - p.pad_h + y, b,
                                        &full[s]);
            }
        }
        __syncwarp();
    } else if (warp == 6) {
        // ------------------------------------------------ producer: dY, one output row per buffer
        if (lane == 0) {
            int dq = 0;
            for (int k = 0; k < nb && ok; k++) {
                const int band = (int) blockIdx.x + k * (int) gridDim.x;
                const int b = band / p.bands_per_img, oy0 = (band - b * p.bands_per_img) * SW_R;
                const int rows = min(SW_R, p.Ho - oy0);
                for (int r = 0; r < rows; r++, dq++) {
                    const int d = dq % SW_DYB;
                    if (dq >= SW_DYB && !(ok = tc::mbar_wait(&dy_empty[d], ((dq / SW_DYB) + 1) & 1, p.err, 64)))
                        break;
                    tc::mbar_arrive_expect_tx(&dy_full[d], (uint32_t) p.wpad * 128);
                    tc::tma_load_3d(tc::smem_u32(dyb + d * SW_DY_MAX), &dymap, 0, 0, b * p.Ho + oy0 + r, &dy_full[d]);
                }
            }
        }
        __syncwarp();
    } else if (warp == 1 || warp >= 7) {
        // ------------------------------------------------ MMA issuers: one per tap pair, warp 1 pair 0,
        // warps 7-9 pairs 1-3 (one thread's loop overhead between MMAs bounds its issue rate)
        if (lane == 0) {
            const int m = warp == 1 ? 0 : warp - 6;
            constexpr uint32_t idesc = tc::idesc_bf16(128, 64, 1, 1);
            int dq = 0;
            for (int k = 0; k < nb && ok; k++) {
                const int s = k & 1;
                if (!(ok = tc::mbar_wait(&full[s], (k >> 1) & 1, p.err, 62))) break;
                tc::tc_fence_after();
                const int band = (int) blockIdx.x + k * (int) gridDim.x;
                const int b = band / p.bands_per_img, oy0 = (band - b * p.bands_per_img) * SW_R;
                const int rows = min(SW_R, p.Ho - oy0);
                const uint32_t sa = tc::smem_u32(base + s * SW_SLAB_MAX);
                // A: 16 core matrices one slab row apart, 8-pixel K groups 128 B apart;
                // B: a dY row of Wpad pixels x 128 B, 128-byte swizzle, a 16-pixel K step is 2048 B
                const uint64_t a0 = tc::mn_interleave_desc(sa, 128, p.pitch);
                for (int r = 0; r < rows; r++, dq++) {
                    const int d = dq % SW_DYB;
                    if (!(ok = tc::mbar_wait(&dy_full[d], (dq / SW_DYB) & 1, p.err, 65))) break;
                    tc::tc_fence_after();
                    const uint64_t b0 = tc::sw128_desc(tc::smem_u32(dyb + d * SW_DY_MAX), 8192, 1024);
                    for (int ks = 0; ks < p.nks; ks++) {
                        const uint64_t bd = b0 + (uint64_t) (ks * 128);
                        const uint64_t ar = a0 + (uint64_t) ((4 * r * p.pitch + 256 * ks) >> 4);
                        if (m < p.npairs)
                            tc::mma_f16(tmem + (uint32_t) (64 * m), ar + (uint64_t) m, bd, idesc, (k | r | ks) != 0);
                    }
                    tc::mma_commit(&dy_empty[d]);
                }
                tc::mma_commit(&empty[s]);
            }
            tc::mma_commit(accum);
        }
        __syncwarp();
    } else if (warp < 6) {
        // ------------------------------------------------ epilogue: the CTA's partial dW
        // D row L = 8 * (2 * ky + stream) + ci; pair m's columns 64m .. 64m + 63 are co
        if (ok) ok = tc::mbar_wait(accum, 0, p.err, 63);
        tc::tc_fence_after();
        const int q = warp & 3, L = q * 32 + lane;
        const int ky = L >> 4, sm = (L >> 3) & 1, ci = L & 7;
        const int Nx = p.kh * p.kw * 8;
        float *part = p.ws + (size_t) blockIdx.x * Nx * 64;
        for (int m = 0; m < p.npairs; m++) {
            uint32_t v0[32], v1[32];
            const uint32_t ta = tmem + ((uint32_t) (q * 32) << 16) + (uint32_t) (64 * m);
            tc::tmem_ld_32x32b_x32(ta, v0);
            tc::tmem_ld_32x32b_x32(ta + 32, v1);
            tc::tmem_ld_wait();
            const int kx = sm == 0 ? 2 * m + 1 : 2 * m;
            if (!ok || ky >= p.kh || kx >= p.kw) continue;
            float4 *dst = reinterpret_cast<float4 *>(part + (size_t) ((ky * p.kw + kx) * 8 + ci) * 64);
#pragma unroll
            for (int j = 0; j < 8; j++)
                dst[j] = make_float4(__uint_as_float(v0[4 * j]), __uint_as_float(v0[4 * j + 1]),
                                     __uint_as_float(v0[4 * j + 2]), __uint_as_float(v0[4 * j + 3]));
#pragma unroll
            for (int j = 0; j < 8; j++)
                dst[8 + j] = make_float4(__uint_as_float(v1[4 * j]), __uint_as_float(v1[4 * j + 1]),
                                         __uint_as_float(v1[4 * j + 2]), __uint_as_float(v1[4 * j + 3]));
        }
    }
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    if (warp == 1) tc::tmem_dealloc(tmem, 64 * SW_MAXPAIRS);
}

struct StemWgGeom {
    int wpad, npairs, ent, bands_per_img, total_bands, grid;
    uint32_t pitch;
};

bool stem_wgrad_geom(const cg_shape &s, StemWgGeom &sg) {
    if (s.c > 8 || s.kn != 64 || s.vstride != 2 || s.hstride != 2 || s.vdil != 1 || s.hdil != 1 || s.kh > 8 ||
        s.kw > 8)
        return false;
    const ConvGeom g = make_geom(s);
    if (g.ho < 1 || g.wo < 1 || (long long) s.b * g.ho * g.wo >= (1LL << 31)) return false;
    sg.wpad = (g.wo + 15) / 16 * 16;
    sg.npairs = (s.kw + 1) / 2;
    sg.ent = sg.wpad + sg.npairs - 1;   // slab entries s = ox + m
    sg.pitch = (uint32_t) (sg.ent * 16 + 127) / 128 * 128;   // TMA destinations 128-byte aligned
    sg.bands_per_img = (g.ho + SW_R - 1) / SW_R;
    sg.total_bands = s.b * sg.bands_per_img;
    const int sms = tc_num_sms();
    sg.grid = sg.total_bands < sms ? sg.total_bands : sms;
    return 2 * sg.ent <= 256 && 2 * SW_NY * sg.pitch <= SW_SLAB_MAX && (uint32_t) sg.wpad * 128 <= SW_DY_MAX;
}

}  // namespace

bool tc_stem_wgrad_applicable(const cg_shape &s) {
    StemWgGeom sg;
    return stem_wgrad_geom(s, sg);
}

int tc_stem_wgrad_splits(const cg_shape &s) {
    StemWgGeom sg;
    return stem_wgrad_geom(s, sg) ? sg.grid : 0;
}

convgemm_status_t tc_stem_wgrad_run(const cg_shape &s, const void *dy, const void *x, float *ws, float *dw,
                                    int layout, cudaStream_t st) {
    StemWgGeom sg;
    if (!stem_wgrad_geom(s, sg)) return cg_set_error(CONVGEMM_ERROR_NOT_SUPPORTED, "small-channel weight gradient: shape");
    const ConvGeom g = make_geom(s);
    StemWgParams p;
    memset(&p, 0, sizeof(p));
    p.ws = ws;
    p.Ho = g.ho;
    p.kh = s.kh;
    p.kw = s.kw;
    p.pad_h = s.vpad;
    p.npairs = sg.npairs;
    p.nks = sg.wpad / 16;
    p.wpad = sg.wpad;
    p.bands_per_img = sg.bands_per_img;
    p.total_bands = sg.total_bands;
    p.col0[0] = 1 - s.hpad;
    p.col0[1] = -s.hpad;
    p.pitch = sg.pitch;
    p.nyl = 2 * (SW_R - 1) + s.kh;
    p.tx = 2 * (uint32_t) p.nyl * sg.ent * 16;
    p.err = cg_device_error_word();
    if (!p.err) return cg_set_error(CONVGEMM_ERROR_CUDA, "device error word unavailable");
    CUtensorMap xmap, dymap;
    {   // input [B][H][W][8]: box {8, 2 * ent (traversal stride 2: ent pixels), 1 row, 1 image}
        const unsigned long long dims[4] = {8, (unsigned long long) s.w, (unsigned long long) s.h,
                                            (unsigned long long) s.b};
        const unsigned long long str[3] = {16, 16ull * s.w, 16ull * s.w * s.h};
        const unsigned box[4] = {8, (unsigned) (2 * sg.ent), 1, 1};
        const unsigned estr[4] = {1, 2, 1, 1};
        if (convgemm_status_t e = tc_make_map_nd(&xmap, 4, x, dims, str, box, estr, 0)) return e;
    }
    {   // dY [B*Ho][Wo][64]: box {64 channels, Wpad pixels, 1 row}, 128-byte swizzle
        const unsigned long long dims[3] = {64, (unsigned long long) g.wo, (unsigned long long) s.b * g.ho};
        const unsigned long long str[2] = {128, 128ull * g.wo};
        const unsigned box[3] = {64, (unsigned) sg.wpad, 1};
        const unsigned estr[3] = {1, 1, 1};
        if (convgemm_status_t e = tc_make_map_nd(&dymap, 3, dy, dims, str, box, estr, 1)) return e;
    }
    static bool attr = false;
    if (!attr) {
        if (cudaError_t e = cudaFuncSetAttribute(tc_stem_wgrad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 (int) SW_SMEM))
            return cg_cuda_check(e, "small-channel weight-gradient attribute");
        attr = true;
    }
    if (convgemm_status_t e = cg_cuda_check(cg_launch_ex(CG_PDL_OFF, tc_stem_wgrad_kernel, dim3(sg.grid), dim3(320),
                                                         SW_SMEM, st, p, xmap, dymap),
                                            "small-channel weight-gradient launch"))
        return e;
    const int Cp = 8, Nx = s.kh * s.kw * Cp;
    return cg_cuda_check(tc_wgrad_reduce(ws, dw, sg.grid, 1, Nx, s.kn, s.c, Cp, s.kh, s.kw, layout, st),
                         "small-channel weight-gradient reduction");
}
