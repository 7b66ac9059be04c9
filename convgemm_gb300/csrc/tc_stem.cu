// BF16 forward of convolutions with at most 8 input channels whose output rows
// fit one 128-row tile (the 7x7/s2 ResNet stem on 224x224 input, the first
// layers of VGG-like networks): sconvGemmNHWC('N') (src/convGemm.c:65-70) for c <= 8.
//
// With c padded to 8 one tap of one pixel is 16 bytes, and the general kernel's
// im2row gather issues one 16-byte cp.async per (pixel, tap): the load-store
// unit, not memory, bounds it.  Here a tile is one output row (b, oy) of up to
// 128 pixels:
//   * one TMA load brings the input slab the row needs -- Hbox = (kh-1)*dh + 1
//     input rows x Wbox = (wo-1)*sw + (kw-1)*dw + 1 pixels x 8 channels, zero
//     outside the image -- into shared memory (double-buffered across tiles);
//   * the 128 producer threads build each 64-deep K block (8 taps x 8 channels)
//     of the 128-byte-swizzled K-major A tile from the slab with 16-byte
//     shared-memory copies (taps past kh*kw and rows past wo are zero);
//   * the packed weights of the (single) N tile are loaded once per CTA and stay
//     resident; a pipeline stage carries two K blocks of A;
//   * tcgen05.mma accumulates in TMEM, and the epilogue applies scale / shift /
//     ReLU and stores each valid row directly.
#include <cstring>

#include <cuda_bf16.h>

#include "cg_common.cuh"
#include "tc_epi.cuh"
#include "tc_host.h"
#include "tc_ptx.cuh"

namespace {

constexpr int STEM_STAGES = 3;
constexpr int STEM_KB = 2;                       // K blocks per stage
constexpr uint32_t STEM_A = 128 * 128;           // one K block: 128 rows x 64 BF16 K
constexpr uint32_t STEM_SLAB_MAX = 27 * 1024;   // input slab bytes per buffer
constexpr uint32_t STEM_W_MAX = 64 * 1024;      // resident packed weights (every K block of the N tile)
constexpr int STEM_MAXTAPS = 64;

struct StemParams {
    __nv_bfloat16 *out;
    const float *scale, *shift;
    int relu, B, Ho, Wo, kn, ntaps, ktiles, ntn, total, sw, Wbox, Hbox, pad_h, pad_w, sh;
    int *err;
    int32_t tapoff[STEM_MAXTAPS];   // slab pixel offset of each tap for output column 0
};

template <int BN>
struct StemCfg {
    static constexpr uint32_t B_BYTES = BN * 128;   // one K block of weights
    static constexpr uint32_t STAGE = STEM_KB * STEM_A;
    static constexpr size_t SMEM = 1024 + (size_t) STEM_STAGES * STAGE + STEM_W_MAX + 2 * (size_t) STEM_SLAB_MAX + 256 +
                                   2 * BN * 4 + STEM_MAXTAPS * 4;   // 256: the mbarriers
    static_assert(SMEM <= 232448, "shared memory");
};


__device__ __forceinline__ void tma_load_4d(uint32_t dst, const CUtensorMap *map, int c0, int c1, int c2, int c3,
                                            uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
        "[%6];" ::"r"(dst),
        "l"((uint64_t) map), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(tc::smem_u32(bar))
        : "memory");
}

template <int BN>
__global__ void __launch_bounds__(288, 1)
    tc_stem_kernel(const __grid_constant__ StemParams p, const __grid_constant__ CUtensorMap xmap,
                   const __grid_constant__ CUtensorMap wmap) {
    using C = StemCfg<BN>;
    tc::pdl_wait();   // the weights are loaded in the prologue; pdl_trigger: in the producer loop
    extern __shared__ uint8_t smem_raw[];
    uint8_t *base = (uint8_t *) (((uintptr_t) smem_raw + 1023) & ~(uintptr_t) 1023);
    uint8_t *wres = base + STEM_STAGES * C::STAGE;   // resident weights: K block j at j * B_BYTES
    uint8_t *slab = wres + STEM_W_MAX;                // two buffers of STEM_SLAB_MAX (1024-aligned)
    uint64_t *full = (uint64_t *) (slab + 2 * STEM_SLAB_MAX);
    uint64_t *empty = full + STEM_STAGES;
    uint64_t *slab_full = empty + STEM_STAGES;
    uint64_t *slab_free = slab_full + 2;
    uint64_t *acc_full = slab_free + 2;
    uint64_t *acc_empty = acc_full + 2;
    uint64_t *wfull = acc_empty + 2;
    uint32_t *tmem_holder = (uint32_t *) (wfull + 1);
    float *sc_tab = (float *) (slab + 2 * STEM_SLAB_MAX + 256);
    float *sh_tab = sc_tab + BN;
    int32_t *tap_tab = (int32_t *) (sh_tab + BN);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t slab_bytes = (uint32_t) p.Hbox * p.Wbox * 16;
    if (threadIdx.x == 0) {
        for (int s = 0; s < STEM_STAGES; s++) {
            tc::mbar_init(&full[s], 4);   // the 4 A-builder warps
            tc::mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; b++) {
            tc::mbar_init(&slab_full[b], 1);
            tc::mbar_init(&slab_free[b], 4);   // every producer warp done reading the buffer
            tc::mbar_init(&acc_full[b], 1);
            tc::mbar_init(&acc_empty[b], 128);
        }
        tc::mbar_init(wfull, 1);
        tc::fence_mbar_init();
        tc::prefetch_tmap(&xmap);
        // the whole N tile of packed weights (the path takes one N tile), loaded once
        tc::mbar_arrive_expect_tx(wfull, p.ktiles * C::B_BYTES);
        for (int j = 0; j < p.ktiles; j++)
            tc::tma_load_2d(tc::smem_u32(wres + j * C::B_BYTES), &wmap, j * 64, 0, wfull);
    }
    for (int i = threadIdx.x; i < STEM_MAXTAPS; i += blockDim.x) tap_tab[i] = i < p.ntaps ? p.tapoff[i] : 0;
    if (warp == 8) {
        tc::tmem_alloc(tmem_holder, 2 * BN);
        tc::tmem_relinquish();
    }
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tmem = *tmem_holder;
    bool ok = true;

    if (warp < 4) {
        // ------------------------------------------------ producers: slab TMA, A builds, weights TMA
        const int t = threadIdx.x;
        const int tt = t & 7, r0 = t >> 3;   // this thread's tap within a K block; rows r0 + 16*i
        uint32_t it = 0, lt = 0;
        int tile = blockIdx.x;
        if (t == 0 && tile < p.total) {
            const int row = tile / p.ntn, b = row / p.Ho, oy = row % p.Ho;
            tc::mbar_arrive_expect_tx(&slab_full[0], slab_bytes);
            tma_load_4d(tc::smem_u32(slab), &xmap, 0, -p.pad_w, oy * p.sh - p.pad_h, b, &slab_full[0]);
        }
        for (; tile < p.total && ok; tile += gridDim.x, lt++) {
            if (t == 0 && tile + (int) gridDim.x >= p.total) tc::pdl_trigger();   // this CTA's last tile
            const int sb = lt & 1;
            // the next tile's slab goes to the other buffer once every producer has read it (tile lt - 1)
            const int nxt = tile + gridDim.x;
            if (t == 0 && nxt < p.total) {
                if (lt >= 1 && !(ok = tc::mbar_wait(&slab_free[sb ^ 1], ((lt - 1) >> 1) & 1, p.err, 46))) break;
                const int nrow = nxt / p.ntn, nb = nrow / p.Ho, noy = nrow % p.Ho;
                tc::mbar_arrive_expect_tx(&slab_full[sb ^ 1], slab_bytes);
                tma_load_4d(tc::smem_u32(slab + (sb ^ 1) * STEM_SLAB_MAX), &xmap, 0, -p.pad_w, noy * p.sh - p.pad_h,
                            nb, &slab_full[sb ^ 1]);
            }
            if (!(ok = tc::mbar_wait(&slab_full[sb], (lt >> 1) & 1, p.err, 41))) break;
            const uint8_t *sl = slab + sb * STEM_SLAB_MAX;
            for (int j0 = 0; j0 < p.ktiles; j0 += STEM_KB, it++) {
                const int s = it % STEM_STAGES;
                const uint32_t ph = (it / STEM_STAGES) & 1;
                if (it >= (uint32_t) STEM_STAGES && !(ok = tc::mbar_wait(&empty[s], ph ^ 1, p.err, 42))) break;
                for (int kb = 0; kb < STEM_KB && j0 + kb < p.ktiles; kb++) {
                    uint8_t *A = base + s * C::STAGE + kb * STEM_A;
                    const int tap = (j0 + kb) * 8 + tt;
                    const bool tap_ok = tap < p.ntaps;
                    const int toff = tap_ok ? tap_tab[tap] : 0;
#pragma unroll
                    for (int i = 0; i < 8; i++) {
                        const int r = r0 + 16 * i;
                        uint4 v = make_uint4(0, 0, 0, 0);
                        if (tap_ok && r < p.Wo) v = *reinterpret_cast<const uint4 *>(sl + (size_t) (toff + r * p.sw) * 16);
                        *reinterpret_cast<uint4 *>(A + r * 128 + ((tt ^ (r & 7)) << 4)) = v;
                    }
                }
                tc::fence_proxy_async_smem();
                __syncwarp();
                if (lane == 0) tc::mbar_arrive(&full[s]);   // one arrival per warp: its 32 rows are written
            }
            __syncwarp();
            if (lane == 0) tc::mbar_arrive(&slab_free[sb]);   // the warp's reads of the slab are done
        }
    } else if (warp < 8) {
        // ------------------------------------------------ epilogue: direct stores of the valid rows
        const int ew = warp - 4, r = ew * 32 + lane, et = threadIdx.x - 128;
        uint32_t lt = 0;
        for (int tile = blockIdx.x; tile < p.total && ok; tile += gridDim.x, lt++) {
            const int row = tile / p.ntn, n0 = (tile % p.ntn) * BN;
            asm volatile("bar.sync 1, 128;" ::: "memory");   // the previous tile's table readers are done
            for (int jj = et; jj < BN; jj += 128) {
                const int n = min(n0 + jj, p.kn - 1);
                sc_tab[jj] = p.scale ? __ldg(p.scale + n) : 1.0f;
                sh_tab[jj] = p.shift ? __ldg(p.shift + n) : 0.0f;
            }
            const int buf = lt & 1;
            const bool mine = tc::mbar_wait(&acc_full[buf], (lt >> 1) & 1, p.err, 43);
            // tables written, and every epilogue thread agrees whether to go on
            uint32_t all_ok;
            asm volatile(
                "{\n\t.reg .pred pi, po;\n\tsetp.ne.u32 pi, %1, 0;\n\t"
                "bar.red.and.pred po, 1, 128, pi;\n\tselp.u32 %0, 1, 0, po;\n\t}"
                : "=r"(all_ok)
                : "r"((uint32_t) mine)
                : "memory");
            if (!(ok = all_ok != 0)) break;
            tc::tc_fence_after();
            __nv_bfloat16 *orow = p.out + ((size_t) row * p.Wo + r) * p.kn;
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
                uint32_t pk[32];
                if (p.relu)
                    tc::epi_bf16_64<true>(v0, v1, sc_tab + c0, sh_tab + c0, pk);
                else
                    tc::epi_bf16_64<false>(v0, v1, sc_tab + c0, sh_tab + c0, pk);
                const int nb = n0 + c0;
                if (r >= p.Wo || nb >= p.kn) continue;
                if (nb + 64 <= p.kn) {
                    uint4 *dst = reinterpret_cast<uint4 *>(orow + nb);
#pragma unroll
                    for (int q = 0; q < 8; q++) dst[q] = make_uint4(pk[4 * q], pk[4 * q + 1], pk[4 * q + 2], pk[4 * q + 3]);
                } else {
                    uint32_t *dst = reinterpret_cast<uint32_t *>(orow + nb);
#pragma unroll
                    for (int q = 0; q < 32; q++)
                        if (2 * q < p.kn - nb) dst[q] = pk[q];
                }
            }
        }
    } else {
        // ------------------------------------------------ MMA issuer
        if (lane == 0) {
            constexpr uint32_t idesc = tc::idesc_bf16(128, BN, 0, 0);
            uint32_t it = 0, lt = 0;
            ok = tc::mbar_wait(wfull, 0, p.err, 47);
            for (int tile = blockIdx.x; tile < p.total && ok; tile += gridDim.x, lt++) {
                const int buf = lt & 1;
                if (lt >= 2) {
                    ok = tc::mbar_wait(&acc_empty[buf], ((lt >> 1) - 1) & 1, p.err, 44);
                    if (!ok) break;
                    tc::tc_fence_after();
                }
                const uint32_t dt = tmem + (uint32_t) (buf * BN);
                for (int j0 = 0; j0 < p.ktiles; j0 += STEM_KB, it++) {
                    const int s = it % STEM_STAGES;
                    if (!tc::mbar_wait(&full[s], (it / STEM_STAGES) & 1, p.err, 45)) {
                        ok = false;
                        break;
                    }
                    tc::tc_fence_after();
                    for (int kb = 0; kb < STEM_KB && j0 + kb < p.ktiles; kb++) {
                        const uint32_t a0 = tc::smem_u32(base + s * C::STAGE + kb * STEM_A);
                        const uint32_t b0 = tc::smem_u32(wres + (j0 + kb) * C::B_BYTES);
#pragma unroll
                        for (int k = 0; k < 4; k++)
                            tc::mma_f16(dt, tc::sw128_desc(a0 + k * 32, 16, 1024),
                                        tc::sw128_desc(b0 + k * 32, 16, 1024), idesc, (j0 | kb | k) != 0);
                    }
                    tc::mma_commit(&empty[s]);
                }
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
cudaError_t launch_stem(const StemParams &p, const CUtensorMap &x, const CUtensorMap &w, int grid, cudaStream_t st) {
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(tc_stem_kernel<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int) StemCfg<BN>::SMEM);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    return cg_launch_pdl(tc_stem_kernel<BN>, dim3(grid), dim3(288), StemCfg<BN>::SMEM, st, p, x, w);
}

}  // namespace

bool tc_stem_applicable(const cg_shape &s) {
    const ConvGeom g = make_geom(s);
    const long long wbox = (long long) (g.wo - 1) * s.hstride + (long long) (s.kw - 1) * s.hdil + 1;
    const long long hbox = (long long) (s.kh - 1) * s.vdil + 1;
    const int bn = s.kn > 64 ? 128 : 64;
    const long long wbytes = (long long) ((s.kh * s.kw + 7) / 8) * bn * 128;
    return s.c <= 8 && g.wo <= 128 && s.kh * s.kw <= STEM_MAXTAPS && s.kn % 8 == 0 && s.kn <= 128 &&
           wbytes <= STEM_W_MAX && wbox <= 256 && hbox <= 256 && hbox * wbox * 16 <= STEM_SLAB_MAX &&
           (long long) s.b * g.ho * g.wo < (1LL << 31);
}

convgemm_status_t tc_stem_run(const cg_shape &s, const void *x, const void *wpacked, int Kpad, void *y,
                              const float *scale, const float *shift, int relu, cudaStream_t st) {
    const ConvGeom g = make_geom(s);
    StemParams p;
    memset(&p, 0, sizeof(p));
    p.out = (__nv_bfloat16 *) y;
    p.scale = scale;
    p.shift = shift;
    p.relu = relu;
    p.B = s.b;
    p.Ho = g.ho;
    p.Wo = g.wo;
    p.kn = s.kn;
    p.ntaps = s.kh * s.kw;
    p.ktiles = (p.ntaps + 7) / 8;
    const int bn = s.kn > 64 ? 128 : 64;
    p.ntn = (s.kn + bn - 1) / bn;
    p.total = s.b * g.ho * p.ntn;
    p.sw = s.hstride;
    p.sh = s.vstride;
    p.pad_h = s.vpad;
    p.pad_w = s.hpad;
    p.Wbox = (g.wo - 1) * s.hstride + (s.kw - 1) * s.hdil + 1;
    p.Hbox = (s.kh - 1) * s.vdil + 1;
    p.err = cg_device_error_word();
    if (!p.err) return cg_set_error(CONVGEMM_ERROR_CUDA, "device error word unavailable");
    if (p.ktiles * 64 > Kpad) return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "small-channel forward: packed K");
    for (int kx = 0; kx < s.kh; kx++)
        for (int ky = 0; ky < s.kw; ky++) p.tapoff[kx * s.kw + ky] = kx * s.vdil * p.Wbox + ky * s.hdil;
    CUtensorMap xmap, wmap;
    if (convgemm_status_t e = tc_make_map_4d_box(&xmap, x, s.b, s.h, s.w, 8, p.Hbox, p.Wbox)) return e;
    if (convgemm_status_t e = tc_make_map_2d(&wmap, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, wpacked, s.kn, Kpad, 64, bn))
        return e;
    const int sms = tc_num_sms();
    const int grid = p.total < sms ? p.total : sms;
    return cg_cuda_check(bn == 64 ? launch_stem<64>(p, xmap, wmap, grid, st) : launch_stem<128>(p, xmap, wmap, grid, st),
                         "small-channel forward launch");
}
