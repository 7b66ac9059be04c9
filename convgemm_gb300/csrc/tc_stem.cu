// BF16 forward of convolutions with at most 8 input channels (the 7x7/s2 ResNet
// stem on 224x224 input, the first layer of VGG-like networks):
// sconvGemmNHWC('N') (src/convGemm.c:65-70) for c <= 8.
//
// With c padded to 8 one tap of one pixel is 16 bytes: too narrow for im2col-mode
// TMA (one 16-byte request per pixel and tap) and, copied into 128-byte-swizzled
// A tiles by threads, bound by shared-memory copies.  Here the tensor core reads
// its A operand straight out of input slabs:
//   * a tile is a chunk of up to 128 output pixels of one output row (b, oy,
//     columns 128*wc ..);
//   * for each residue rho of the input column modulo the horizontal stride sw,
//     one TMA load (traversal stride sw along W) brings the slab
//     S_rho[i][j] = x[b][oy*sh - pad_h + i][sw*(128*wc + qmin + j) + rho][0..7]
//     for i < Hbox = (kh-1)*dh + 1 input rows: tap (ky, kx), whose input column
//     for output column ox is sw*(ox + q) + rho with kx*dw - pad_w = sw*q + rho,
//     reads rows j = r + q - qmin of S_rho[ky*dh] for the tile's pixels r -- 128
//     consecutive 16-byte rows, i.e. a K-major operand of 8 K elements in the
//     no-swizzle core-matrix layout (8 rows x 16 bytes, 8-row groups 128 bytes
//     apart);
//   * one kind::f16 MMA (K = 16) takes two taps: the descriptor's leading-dimension
//     byte offset (the K-direction core-matrix stride) is the distance between the
//     two taps' slab rows, so taps are paired in address order; an odd last tap is
//     paired with a 2 KB zero region behind each slab buffer (which also absorbs
//     the reads of rows past the chunk's valid pixels);
//   * the packed weights of the single N tile are resident in shared memory in the
//     same pair order: pair p holds [BN][8] BF16 for its first tap, then for its
//     second (zero for the zero region);
//   * slab buffers are double-buffered across tiles: the MMA commit of a tile frees
//     its slab, the next-but-one tile's TMA loads refill it;
//   * the epilogue applies scale / shift / ReLU and stores through per-warp TMA
//     stores of a 3-D output map [B*Ho][Wo][kn] (rows past Wo are clipped).
// There is no K pipeline: the whole reduction of a tile (kh*kw*8 <= 512 deep) is
// one slab.
#include <algorithm>
#include <cstring>

#include <cuda_bf16.h>

#include "cg_common.cuh"
#include "tc_epi.cuh"
#include "tc_host.h"
#include "tc_ptx.cuh"

namespace {

constexpr int STEM_MAXTAPS = 64;
constexpr int STEM_MAXPAIRS = STEM_MAXTAPS / 2;
constexpr uint32_t STEM_SLAB_MAX = 48 * 1024;    // the residue slabs of one buffer
constexpr uint32_t STEM_ZERO = 2048;             // zero region behind each slab buffer: 128 rows x 16 B
constexpr uint32_t STEM_W_MAX = 64 * 1024;       // resident weights
constexpr uint32_t STEM_EPI = 4 * 4096;          // per-warp output staging, 32 rows x 128 B

struct StemParams {
    const __nv_bfloat16 *w;   // packed weights [kn][Kpad], K = tap * 8 + channel
    const float *scale, *shift;
    int relu, B, Ho, Wo, kn, Kpad, nwc, total, sh, sw, pad_h, qmin, npairs;
    uint32_t buf_bytes;       // one slab buffer: sw residue slabs (rho_bytes apart) + the zero region
    uint32_t rho_bytes;       // one residue slab, 1024-aligned
    uint32_t slab_tx;         // bytes the TMA loads of one tile deliver
    int *err;
    float *stats;             // per (tile, epilogue warp) group g: [g][0][kn] sum, [g][1][kn] sum of squares, or NULL
    uint32_t aoff[STEM_MAXPAIRS];   // byte offset of the pair's first tap rows within a slab buffer
    uint32_t alead[STEM_MAXPAIRS];  // bytes from the first to the second tap's rows (or to the zero region)
    int16_t wtap[2 * STEM_MAXPAIRS];   // the pair's taps (ky * kw + kx) in the packed weights; -1 = zero
};

template <int BN>
struct StemCfg {
    static constexpr uint32_t PAIR_W = 2 * BN * 16;   // one pair of taps of the resident weights
    static constexpr size_t SMEM = 1024 + (size_t) STEM_W_MAX + 2 * ((size_t) STEM_SLAB_MAX + STEM_ZERO) +
                                   2 * STEM_EPI + 256 + 2 * BN * 4 + 2 * STEM_MAXPAIRS * 4;
    static_assert(SMEM <= 232448, "shared memory");
};

// No-swizzle K-major descriptor: core matrices of 8 rows x 16 bytes; `lead` = bytes
// between the core matrices of K elements 0-7 and 8-15, 8-row groups 128 bytes apart.
__device__ __forceinline__ uint64_t kmajor_desc(uint32_t saddr, uint32_t lead) {
    uint64_t d = 0;
    d |= (uint64_t) ((saddr & 0x3FFFF) >> 4);
    d |= (uint64_t) ((lead >> 4) & 0x3FFF) << 16;
    d |= (uint64_t) (128 >> 4) << 32;
    d |= (uint64_t) 1 << 46;   // descriptor version for tcgen05; layout bits 61-63 = 0: no swizzle
    return d;
}

__device__ __forceinline__ void tma_store_3d(const CUtensorMap *map, uint32_t src, int c0, int c1, int c2) {
    asm volatile("cp.async.bulk.tensor.3d.global.shared::cta.bulk_group [%0, {%2, %3, %4}], [%1];" ::"l"(
                     (uint64_t) map),
                 "r"(src), "r"(c0), "r"(c1), "r"(c2)
                 : "memory");
    asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}

template <int N>
__device__ __forceinline__ void bulk_wait_read() {
    asm volatile("cp.async.bulk.wait_group.read %0;" ::"n"(N) : "memory");
}

template <int BN>
__global__ void __launch_bounds__(288, 1)
    tc_stem_kernel(const __grid_constant__ StemParams p, const __grid_constant__ CUtensorMap xmap,
                   const __grid_constant__ CUtensorMap omap) {
    using C = StemCfg<BN>;
    tc::pdl_wait();   // weights and input may come from the previous kernel; pdl_trigger: producer's last tile
    extern __shared__ uint8_t smem_raw[];
    uint8_t *base = (uint8_t *) (((uintptr_t) smem_raw + 1023) & ~(uintptr_t) 1023);
    uint8_t *wres = base;                                   // resident weights, pair p at p * PAIR_W
    uint8_t *slab = wres + STEM_W_MAX;                      // two buffers of p.buf_bytes (1024-aligned)
    uint8_t *epi = slab + 2 * (STEM_SLAB_MAX + STEM_ZERO);  // 2 x 4 warps x 4 KB of output staging
    uint64_t *slab_full = (uint64_t *) (epi + 2 * STEM_EPI);
    uint64_t *slab_free = slab_full + 2;
    uint64_t *acc_full = slab_free + 2;
    uint64_t *acc_empty = acc_full + 2;
    uint32_t *tmem_holder = (uint32_t *) (acc_empty + 2);
    float *sc_tab = (float *) (epi + 2 * STEM_EPI + 256);
    float *sh_tab = sc_tab + BN;
    uint32_t *aoff_tab = (uint32_t *) (sh_tab + BN);
    uint32_t *alead_tab = aoff_tab + STEM_MAXPAIRS;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        for (int b = 0; b < 2; b++) {
            tc::mbar_init(&slab_full[b], 1);
            tc::mbar_init(&slab_free[b], 1);   // the MMA commit of the tile that read the buffer
            tc::mbar_init(&acc_full[b], 1);
            tc::mbar_init(&acc_empty[b], 128);
        }
        tc::fence_mbar_init();
        tc::prefetch_tmap(&xmap);
        tc::prefetch_tmap(&omap);
    }
    if (warp < 4) {
        // the resident weights in pair order, and the zero regions
        const int t = threadIdx.x;
        const int nrow = p.npairs * 2 * BN;   // 16-byte rows
        for (int i = t; i < nrow; i += 128) {
            const int half = i / BN, n = i % BN;   // half = 2 * pair + (second tap)
            const int tap = p.wtap[half];
            uint4 v = make_uint4(0, 0, 0, 0);
            if (tap >= 0 && n < p.kn)
                v = __ldg(reinterpret_cast<const uint4 *>(p.w + (size_t) n * p.Kpad + tap * 8));
            *reinterpret_cast<uint4 *>(wres + (size_t) i * 16) = v;
        }
        for (int b = 0; b < 2; b++)
            for (int i = t; i < (int) (STEM_ZERO / 16); i += 128)
                *reinterpret_cast<uint4 *>(slab + b * p.buf_bytes + p.sw * p.rho_bytes + i * 16) =
                    make_uint4(0, 0, 0, 0);
        tc::fence_proxy_async_smem();
    } else if (warp < 8) {
        const int et = threadIdx.x - 128;
        for (int n = et; n < BN; n += 128) {
            const int nn = min(n, p.kn - 1);
            sc_tab[n] = p.scale ? __ldg(p.scale + nn) : 1.0f;
            sh_tab[n] = p.shift ? __ldg(p.shift + nn) : 0.0f;
        }
        for (int i = et; i < p.npairs; i += 128) {
            aoff_tab[i] = p.aoff[i];
            alead_tab[i] = p.alead[i];
        }
    } else {
        tc::tmem_alloc(tmem_holder, 2 * BN);
        tc::tmem_relinquish();
    }
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tmem = *tmem_holder;
    bool ok = true;

    if (warp == 0) {
        // ------------------------------------------------ producer: the slab TMA loads of each tile
        if (lane == 0) {
            uint32_t lt = 0;
            for (int tile = blockIdx.x; tile < p.total && ok; tile += gridDim.x, lt++) {
                if (tile + (int) gridDim.x >= p.total) tc::pdl_trigger();   // this CTA's last tile
                const int sb = lt & 1;
                if (lt >= 2 && !(ok = tc::mbar_wait(&slab_free[sb], ((lt >> 1) + 1) & 1, p.err, 41))) break;
                const int row = tile / p.nwc, wc = tile % p.nwc;
                const int b = row / p.Ho, oy = row % p.Ho;
                const uint32_t dst = tc::smem_u32(slab + sb * p.buf_bytes);
                tc::mbar_arrive_expect_tx(&slab_full[sb], p.slab_tx);
                for (int rho = 0; rho < p.sw; rho++)
                    tc::tma_load_4d(dst + rho * p.rho_bytes, &xmap, 0, p.sw * (128 * wc + p.qmin) + rho,
                                oy * p.sh - p.pad_h, b, &slab_full[sb]);
            }
        }
        __syncwarp();
    } else if (warp >= 4 && warp < 8) {
        // ------------------------------------------------ epilogue
        const int ew = warp - 4;
        uint8_t *stg_warp = epi + ew * 4096;
        uint32_t lt = 0;
        int ebuf = 0;
        for (int tile = blockIdx.x; tile < p.total && ok; tile += gridDim.x, lt++) {
            const int row = tile / p.nwc, wc = tile % p.nwc;
            const int buf = lt & 1;
            if (!(ok = tc::mbar_wait(&acc_full[buf], (lt >> 1) & 1, p.err, 43))) break;
            tc::tc_fence_after();
            for (int c0 = 0; c0 < BN; c0 += 64) {
                uint32_t v0[32], v1[32];
                const uint32_t ta = tmem + ((uint32_t) (ew * 32) << 16) + (uint32_t) (buf * BN + c0);
                tc::tmem_ld_32x32b_x32(ta, v0);
                tc::tmem_ld_32x32b_x32(ta + 32, v1);
                tc::tmem_ld_wait();
                if (c0 + 64 >= BN) {
                    tc::tc_fence_before();
                    tc::mbar_arrive(&acc_empty[buf]);
                }
                if (p.stats) {
                    // batch-norm statistics of the 64 columns over this warp's 32 pixels
                    float *part = p.stats + ((size_t) tile * 4 + ew) * 2 * p.kn;
                    const bool valid = 128 * wc + ew * 32 + lane < p.Wo;
#pragma unroll
                    for (int h = 0; h < 2; h++) {
                        float sum, sq;
                        tc::stats_cols32(h ? v1 : v0, sc_tab + c0 + 32 * h, sh_tab + c0 + 32 * h, valid, sum, sq);
                        const int col = c0 + 32 * h + lane;
                        if (col < p.kn) {
                            part[col] = sum;
                            part[p.kn + col] = sq;
                        }
                    }
                }
                uint32_t pk[32];
                if (p.relu)
                    tc::epi_bf16_64<true>(v0, v1, sc_tab + c0, sh_tab + c0, pk);
                else
                    tc::epi_bf16_64<false>(v0, v1, sc_tab + c0, sh_tab + c0, pk);
                if (lane == 0) bulk_wait_read<1>();   // the store that last read this staging buffer
                __syncwarp();
                uint8_t *stg = stg_warp + ebuf * STEM_EPI;
#pragma unroll
                for (int q = 0; q < 8; q++) {
                    const uint4 u = make_uint4(pk[4 * q], pk[4 * q + 1], pk[4 * q + 2], pk[4 * q + 3]);
                    *reinterpret_cast<uint4 *>(stg + lane * 128 + ((q ^ (lane & 7)) << 4)) = u;
                }
                tc::fence_proxy_async_smem();
                __syncwarp();
                const int ox0 = 128 * wc + ew * 32;
                if (lane == 0 && ox0 < p.Wo && c0 < p.kn) tma_store_3d(&omap, tc::smem_u32(stg), c0, ox0, row);
                ebuf ^= 1;
            }
        }
        if (lane == 0) asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
    } else if (warp == 8) {
        // ------------------------------------------------ MMA issuer
        if (lane == 0) {
            constexpr uint32_t idesc = tc::idesc_bf16(128, BN, 0, 0);
            const uint32_t wbase = tc::smem_u32(wres);
            // the low descriptor words of every pair's A operand (start within a slab buffer,
            // lead) in registers: table loads between the MMAs would queue behind the TMA and
            // tensor-core shared-memory traffic
            uint32_t alo[STEM_MAXPAIRS];
#pragma unroll
            for (int q = 0; q < STEM_MAXPAIRS; q++)
                alo[q] = q < p.npairs ? (uint32_t) kmajor_desc(aoff_tab[q], alead_tab[q]) : 0u;
            const uint64_t dhi = kmajor_desc(0, 0) & 0xFFFFFFFF00000000ull;   // SBO, version, layout
            uint32_t lt = 0;
            for (int tile = blockIdx.x; tile < p.total && ok; tile += gridDim.x, lt++) {
                const int sb = lt & 1, buf = lt & 1;
                if (lt >= 2) {
                    if (!(ok = tc::mbar_wait(&acc_empty[buf], ((lt >> 1) + 1) & 1, p.err, 44))) break;
                    tc::tc_fence_after();
                }
                if (!(ok = tc::mbar_wait(&slab_full[sb], (lt >> 1) & 1, p.err, 45))) break;
                tc::tc_fence_after();
                const uint32_t a0 = tc::smem_u32(slab + sb * p.buf_bytes);
                const uint32_t dt = tmem + (uint32_t) (buf * BN);
#pragma unroll
                for (int q = 0; q < STEM_MAXPAIRS; q++)
                    if (q < p.npairs)
                        tc::mma_f16(dt, dhi | (uint64_t) (alo[q] + ((a0 & 0x3FFFF) >> 4)),
                                    kmajor_desc(wbase + q * C::PAIR_W, BN * 16), idesc, q > 0);
                tc::mma_commit(&slab_free[sb]);
                tc::mma_commit(&acc_full[buf]);
            }
        }
        __syncwarp();
    }
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    if (warp == 8) tc::tmem_dealloc(tmem, 2 * BN);
}

template <int BN>
cudaError_t launch_stem(const StemParams &p, const CUtensorMap &x, const CUtensorMap &o, int grid, cudaStream_t st) {
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(tc_stem_kernel<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int) StemCfg<BN>::SMEM);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    return cg_launch_pdl(tc_stem_kernel<BN>, dim3(grid), dim3(288), StemCfg<BN>::SMEM, st, p, x, o);
}

int floor_div(int a, int b) { return a >= 0 ? a / b : -((-a + b - 1) / b); }

// The slab geometry of a shape; false when the path does not apply.
struct StemGeom {
    int bn, wc, qmin, qmax, nj, hbox, npairs;
    uint32_t rho_bytes, buf_bytes;
};

bool stem_geom(const cg_shape &s, StemGeom &sg) {
    // kn >= 64: the output store box is 64 channels wide
    if (s.c > 8 || s.kn % 8 || s.kn < 64 || s.kn > 128 || s.kh * s.kw > STEM_MAXTAPS || s.hstride > 8) return false;
    const ConvGeom g = make_geom(s);
    if ((long long) s.b * g.ho * g.wo >= (1LL << 31)) return false;
    sg.bn = s.kn > 64 ? 128 : 64;
    sg.qmin = 1 << 30;
    sg.qmax = -(1 << 30);
    for (int kx = 0; kx < s.kw; kx++) {
        const int q = floor_div(kx * s.hdil - s.hpad, s.hstride);
        sg.qmin = std::min(sg.qmin, q);
        sg.qmax = std::max(sg.qmax, q);
    }
    sg.wc = std::min(g.wo, 128);
    sg.nj = sg.wc + sg.qmax - sg.qmin;
    sg.hbox = (s.kh - 1) * s.vdil + 1;
    sg.npairs = (s.kh * s.kw + 1) / 2;
    sg.rho_bytes = (uint32_t) ((sg.hbox * sg.nj * 16 + 1023) / 1024 * 1024);
    sg.buf_bytes = (uint32_t) s.hstride * sg.rho_bytes + STEM_ZERO;
    return sg.nj * s.hstride <= 256 && sg.hbox <= 256 && (uint32_t) s.hstride * sg.rho_bytes <= STEM_SLAB_MAX &&
           (uint32_t) sg.npairs * 2 * sg.bn * 16 <= STEM_W_MAX;
}

}  // namespace

bool tc_stem_applicable(const cg_shape &s) {
    StemGeom sg;
    return stem_geom(s, sg);
}

int tc_stem_stat_groups(const cg_shape &s) {
    const ConvGeom g = make_geom(s);
    return s.b * g.ho * ((g.wo + 127) / 128) * 4;
}

convgemm_status_t tc_stem_run(const cg_shape &s, const void *x, const void *wpacked, int Kpad, void *y,
                              const float *scale, const float *shift, int relu, cudaStream_t st, float *stats) {
    StemGeom sg;
    if (!stem_geom(s, sg)) return cg_set_error(CONVGEMM_ERROR_NOT_SUPPORTED, "small-channel forward: shape");
    const ConvGeom g = make_geom(s);
    const int ntaps = s.kh * s.kw;
    if (((ntaps + 7) / 8) * 64 > Kpad) return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "small-channel forward: packed K");
    StemParams p;
    memset(&p, 0, sizeof(p));
    p.w = (const __nv_bfloat16 *) wpacked;
    p.scale = scale;
    p.shift = shift;
    p.relu = relu;
    p.B = s.b;
    p.Ho = g.ho;
    p.Wo = g.wo;
    p.kn = s.kn;
    p.Kpad = Kpad;
    p.nwc = (g.wo + 127) / 128;
    p.total = s.b * g.ho * p.nwc;
    p.sh = s.vstride;
    p.sw = s.hstride;
    p.pad_h = s.vpad;
    p.qmin = sg.qmin;
    p.npairs = sg.npairs;
    p.rho_bytes = sg.rho_bytes;
    p.buf_bytes = sg.buf_bytes;
    p.slab_tx = (uint32_t) s.hstride * sg.hbox * sg.nj * 16;
    p.err = cg_device_error_word();
    if (!p.err) return cg_set_error(CONVGEMM_ERROR_CUDA, "device error word unavailable");
    p.stats = stats;
    // every tap's rows in a slab buffer, sorted by address and paired
    struct TapAt {
        uint32_t off;
        int tap;
    } taps[STEM_MAXTAPS];
    for (int ky = 0; ky < s.kh; ky++)
        for (int kx = 0; kx < s.kw; kx++) {
            const int off = kx * s.hdil - s.hpad;
            const int q = floor_div(off, s.hstride), rho = off - q * s.hstride;
            taps[ky * s.kw + kx] = {(uint32_t) rho * sg.rho_bytes + (uint32_t) (ky * s.vdil * sg.nj + q - sg.qmin) * 16,
                                    ky * s.kw + kx};
        }
    std::sort(taps, taps + ntaps, [](const TapAt &a, const TapAt &b) { return a.off < b.off; });
    const uint32_t zero_off = (uint32_t) s.hstride * sg.rho_bytes;
    for (int q = 0; q < sg.npairs; q++) {
        const TapAt &t1 = taps[2 * q];
        p.aoff[q] = t1.off;
        p.wtap[2 * q] = (int16_t) t1.tap;
        if (2 * q + 1 < ntaps) {
            p.alead[q] = taps[2 * q + 1].off - t1.off;
            p.wtap[2 * q + 1] = (int16_t) taps[2 * q + 1].tap;
        } else {
            p.alead[q] = zero_off - t1.off;
            p.wtap[2 * q + 1] = -1;
        }
    }
    // input [B][H][W][8]: box {8, nj * sw (traversal stride sw: nj pixels), hbox rows, 1 image}
    CUtensorMap xmap, omap;
    {
        const unsigned long long dims[4] = {8, (unsigned long long) s.w, (unsigned long long) s.h,
                                            (unsigned long long) s.b};
        const unsigned long long str[3] = {16, 16ull * s.w, 16ull * s.w * s.h};
        const unsigned box[4] = {8, (unsigned) (sg.nj * s.hstride), (unsigned) sg.hbox, 1};
        const unsigned estr[4] = {1, (unsigned) s.hstride, 1, 1};
        if (convgemm_status_t e = tc_make_map_nd(&xmap, 4, x, dims, str, box, estr, 0)) return e;
    }
    // output [B*Ho][Wo][kn]: box {64 channels, 32 pixels, 1 row}, 128-byte swizzle
    {
        const unsigned long long dims[3] = {(unsigned long long) s.kn, (unsigned long long) g.wo,
                                            (unsigned long long) s.b * g.ho};
        const unsigned long long str[2] = {2ull * s.kn, 2ull * s.kn * g.wo};
        const unsigned box[3] = {64, 32, 1};
        const unsigned estr[3] = {1, 1, 1};
        if (convgemm_status_t e = tc_make_map_nd(&omap, 3, y, dims, str, box, estr, 1)) return e;
    }
    const int sms = tc_num_sms();
    const int grid = p.total < sms ? p.total : sms;
    return cg_cuda_check(sg.bn == 64 ? launch_stem<64>(p, xmap, omap, grid, st) : launch_stem<128>(p, xmap, omap, grid, st),
                         "small-channel forward launch");
}
