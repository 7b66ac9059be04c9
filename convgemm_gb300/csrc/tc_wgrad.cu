// BF16 tensor-core weight gradient (sm_103a): the transposed GEMM of
// sconvGemmNHWC('T') (src/convGemm.c:71-76),
//     dW[co][n] = sum_p dY[p][co] * X_im2row[p][n],  n = tap*Cp + ci,
// whose reduction runs over all b*ho*wo output pixels.  The pixels are cut
// into 64-pixel chunks and the chunks into `splits` contiguous ranges, one per
// blockIdx.z; each CTA writes its FP32 partial tile to a workspace and
// the reduction adds the splits in a fixed order (in increasing split order,
// or, with many splits, in fixed contiguous groups whose sums are then added in
// group order), so the result is bit-reproducible run to run (no float atomics).
//
// Both operands reach the tensor core MN-major (the pixel index is the slow,
// K dimension in memory):
//   dY side: TMA boxes of 64 channels x 64 pixels from dY viewed as [P][kn8];
//   X side:  im2col-mode TMA boxes of 64 channels of one tap x 64 pixels when the
//            channels are multiples of 64 (tiled boxes of the [P][Cp] matrix for a
//            1x1 stride-1 unpadded convolution), else 16-byte cp.async gathers of
//            8 channels of one tap for each pixel, zero-filled for padding, written
//            in the 128-byte-swizzled layout.
// The X side is the 128-row A operand when kn < 128 (template XA), else dY is,
// so narrow layers do not waste half of each MMA; a tuned configuration may put
// the X side on A for wide layers too (measured faster on 3x3 layers at the same
// tile shape and traffic).
#include <cuda_bf16.h>

#include <mutex>

#include "cg_common.cuh"
#include "tc_ptx.cuh"
#include "tc_wgrad.h"

namespace {

using bf16 = __nv_bfloat16;

// FP32 TMA store of one 32 x 1 x 32 box of dW, coordinates (co, tap, ci).
__device__ __forceinline__ void wg_store_3d(const CUtensorMap *map, uint32_t src, int co, int tap, int ci) {
    asm volatile("cp.async.bulk.tensor.3d.global.shared::cta.bulk_group [%0, {%2, %3, %4}], [%1];" ::"l"((uint64_t) map),
                 "r"(src), "r"(co), "r"(tap), "r"(ci)
                 : "memory");
}
__device__ __forceinline__ void wg_bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void wg_bulk_wait_read() {
    asm volatile("cp.async.bulk.wait_group.read %0;" ::"n"(N) : "memory");
}
__device__ __forceinline__ void wg_bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }
// Bulk copy of `bytes` (a multiple of 16, both addresses 16-byte aligned) shared -> global.
__device__ __forceinline__ void wg_bulk_store(void *dst, uint32_t src, uint32_t bytes) {
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(src), "r"(bytes) : "memory");
}
// FP32 TMA store of one 32 x 32 x 1 box of the split partials (n, m, split).
__device__ __forceinline__ void wg_store_part(const CUtensorMap *map, uint32_t src, int n, int m, int z) {
    asm volatile("cp.async.bulk.tensor.3d.global.shared::cta.bulk_group [%0, {%2, %3, %4}], [%1];" ::"l"((uint64_t) map),
                 "r"(src), "r"(n), "r"(m), "r"(z)
                 : "memory");
}
// Bulk copy of `bytes` (a multiple of 16, both addresses 16-byte aligned) global -> shared.
__device__ __forceinline__ void wg_bulk_load(uint32_t dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(tc::smem_u32(bar))
                 : "memory");
}

// One 32 x 32 FP32 block into a 4 KB staging buffer laid out as a dW box: 32 rows (K indices
// n = tap*Cp + ci) of 32 output channels, 16-byte chunk q of row r at chunk q ^ (r & 7) (the
// 128-byte swizzle of the store's tensor map; conflict-free shared-memory stores).  The thread
// holds row `lane` of the block, v[j] = column j.  With X on the A side the block's rows are K
// indices; otherwise they are output channels and the block is transposed on the way in.
template <bool XA>
__device__ __forceinline__ void wg_stage_block(uint32_t buf, int lane, const uint32_t (&v)[32]) {
    if constexpr (XA) {
#pragma unroll
        for (int q = 0; q < 8; q++)
            asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(buf + lane * 128 + ((q ^ (lane & 7)) << 4)),
                         "r"(v[4 * q]), "r"(v[4 * q + 1]), "r"(v[4 * q + 2]), "r"(v[4 * q + 3])
                         : "memory");
    } else {
#pragma unroll
        for (int j = 0; j < 32; j++)
            asm volatile("st.shared.b32 [%0], %1;" ::"r"(buf + j * 128 + (((lane >> 2) ^ (j & 7)) << 4) + ((lane & 3) << 2)),
                         "r"(v[j])
                         : "memory");
    }
}

// KB chunks of BK pixels per pipeline stage: one full barrier and one MMA commit
// cover KB chunks (the barrier round trip, not the loads or the MMAs, bounds a
// one-chunk stage).
// PAIR: a CTA pair shares 256 x BN tiles (cta_group::2 MMAs): each CTA holds its 128 A rows and
// half of the BN B columns.
template <int BN, int STAGES, bool XA, int KB = 1, int BKP = 64, bool PAIR = false>
struct WgCfg {
    static constexpr int BM = 128, BK = BKP;  // BK pixels per chunk (64, or 128: each TMA box twice as large)
    static constexpr int BNL = PAIR ? BN / 2 : BN;   // B columns in this CTA's shared memory
    static constexpr uint32_t ATOM_BYTES = (uint32_t) BK * 128;   // 64 channels x BK pixels
    static constexpr uint32_t A_BYTES = BM * BK * 2;
    static constexpr uint32_t B_BYTES = BNL * BK * 2;
    static constexpr uint32_t CHUNK_BYTES = A_BYTES + B_BYTES;
    static constexpr uint32_t STAGE_BYTES = KB * CHUNK_BYTES;
    static constexpr int X_ATOMS = (XA ? BM : BNL) / 64;    // 64-channel atoms gathered from X
    static constexpr int DY_ATOMS = (XA ? BNL : BM) / 64;   // 64-channel atoms loaded from dY
    static constexpr uint32_t DY_BYTES = DY_ATOMS * ATOM_BYTES;
    static constexpr int LAG = STAGES / 2;  // half the ring in flight, half queued for the MMA
    static constexpr size_t SMEM = 1024 + (size_t) STAGES * STAGE_BYTES + 256;
};

// Warps: the gather warps (one TMA-issuing thread on the im2col path; eight warps of
// cp.async gathers otherwise, whose issue rate bounds that path), then the MMA warp;
// warps 0-3 run the epilogue.
// ISS2: a second MMA-issuing warp (warp GW + 1).  Each issuer takes alternate chunks of every
// two-chunk stage into its own accumulator and the epilogue adds the two: one thread's tcgen05
// issue, barrier wait and commit cost tens of cycles each, which bounds a single issuer of the
// eight 128-wide MMAs of a stage.
template <bool IM2C, bool ISS2 = false>
struct WgWarps {
    static constexpr int GW = IM2C ? 4 : 8, THREADS = 32 * (GW + 1 + (ISS2 ? 1 : 0));
};

// PAIR: clusters of two CTAs (x) share 256-row tiles through cta_group::2 MMAs issued by the even
// CTA; each CTA loads its own A rows and half of the B columns (the odd CTA's loads complete on the
// even CTA's barriers) and writes its own 128 rows of dW.
template <int BN, int STAGES, bool XA, bool IM2C, int KB, bool ISS2 = false, int BKP = 64, bool PAIR = false>
__global__ void __launch_bounds__(WgWarps<IM2C, ISS2>::THREADS, 1)
    tc_wgrad_kernel(const __grid_constant__ TcWgradParams p, const __grid_constant__ CUtensorMap dymap,
                    const __grid_constant__ CUtensorMap xmap) {
    using C = WgCfg<BN, STAGES, XA, KB, BKP, PAIR>;
    static_assert(!PAIR || (IM2C && KB == 1 && !ISS2 && BKP == 128 && BN >= 128), "CTA pairs: 128-pixel chunks, 256 x 128 / 256");
    static_assert(BKP == 64 || (IM2C && KB == 1 && !ISS2), "128-pixel chunks: im2col path, one chunk per stage");
    static_assert(IM2C || KB == 1, "the cp.async gather fills one chunk per stage");
    static_assert(!ISS2 || (IM2C && KB == 2), "two issuers: alternate chunks of two-chunk stages");
    constexpr uint32_t NISS = ISS2 ? 2 : 1;
    constexpr uint32_t TCOLS = ISS2 ? 2 * BN : BN;
    extern __shared__ uint8_t smem_raw[];
    uint8_t *base = (uint8_t *) (((uintptr_t) smem_raw + 1023) & ~(uintptr_t) 1023);
    uint64_t *full = (uint64_t *) (base + STAGES * C::STAGE_BYTES);
    uint64_t *empty = full + STAGES;
    uint64_t *accum = empty + STAGES;
    uint32_t *tmem_holder = (uint32_t *) (accum + 1);
    uint64_t *xbar = accum + 2;   // four: the epilogue warps' copies of the exchanged blocks

    constexpr int GW = WgWarps<IM2C>::GW;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; s++) {
            tc::mbar_init(&full[s], IM2C ? 1 : 32 * GW + 1);
            tc::mbar_init(&empty[s], NISS);
        }
        tc::mbar_init(accum, NISS);
        for (int i = 0; i < 4; i++) tc::mbar_init(&xbar[i], 1);
        tc::fence_mbar_init();
        tc::prefetch_tmap(&dymap);
        if (IM2C) tc::prefetch_tmap(&xmap);
    }
    uint32_t prank = 0;   // rank in the CTA pair (0: the MMA-issuing CTA)
    if constexpr (PAIR) {
        asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(prank));
        prank &= 1;
    }
    if (warp == GW) {
        if constexpr (PAIR) {
            tc::tmem_alloc_pair(tmem_holder, TCOLS);
            tc::tmem_relinquish_pair();
        } else {
            tc::tmem_alloc(tmem_holder, TCOLS);
            tc::tmem_relinquish();
        }
    }
    tc::pdl_wait();   // no global memory access above
    tc::pdl_trigger();
    tc::tc_fence_before();
    __syncthreads();
    if constexpr (PAIR) tc::cluster_sync();   // both CTAs' barriers exist before either signals the other
    tc::tc_fence_after();
    const uint32_t tmem = *tmem_holder;

    // tile origins along the X extent (n = tap*Cp + ci) and the channel extent (co)
    const int mrow0 = blockIdx.x * C::BM, ncol0 = blockIdx.y * BN;
    const int bhalf = PAIR ? (int) prank * C::BNL : 0;   // this CTA's B columns within the tile
    const int x0 = XA ? mrow0 : ncol0 + bhalf;
    const int co0 = XA ? ncol0 + bhalf : mrow0;
    const int chunk0 = blockIdx.z * p.chunks_per_split;
    const int KT = min(p.chunks_per_split, p.nchunks - chunk0);   // chunks of this split
    const int NG = (KT + KB - 1) / KB;                              // pipeline stages they fill
    bool ok = true;
    // 32 accumulator columns of this warp's rows: the accumulator, plus the second issuer's (odd chunks)
    auto ld_acc = [&](int c0, uint32_t(&v)[32]) {
        tc::tmem_ld_32x32b_x32(tmem + ((uint32_t) (warp * 32) << 16) + (uint32_t) c0, v);
        tc::tmem_ld_wait();
        if constexpr (ISS2) {
            if (KT >= 2) {
                uint32_t u[32];
                tc::tmem_ld_32x32b_x32(tmem + ((uint32_t) (warp * 32) << 16) + (uint32_t) (BN + c0), u);
                tc::tmem_ld_wait();
#pragma unroll
                for (int i = 0; i < 32; i++) v[i] = __float_as_uint(__fadd_rn(__uint_as_float(v[i]), __uint_as_float(u[i])));
            }
        }
    };
    // fn(c0, v) for the 32-column blocks c0 = 0, 32, ... of this warp's accumulator rows, with the
    // next block's TMEM load in flight while fn runs (each use of v follows its wait)
    auto for_acc_blocks = [&](auto &&fn) {
        uint32_t va[32], ua[32], vb[32], ub[32];
        const uint32_t rowb = tmem + ((uint32_t) (warp * 32) << 16);
        auto issue = [&](int c0, uint32_t(&v)[32], uint32_t(&u)[32]) {
            tc::tmem_ld_32x32b_x32(rowb + (uint32_t) c0, v);
            if constexpr (ISS2) {
                if (KT >= 2) tc::tmem_ld_32x32b_x32(rowb + (uint32_t) (BN + c0), u);
            }
        };
        auto finish = [&](uint32_t(&v)[32], const uint32_t(&u)[32]) {
            if constexpr (ISS2) {
                if (KT >= 2) {
#pragma unroll
                    for (int i = 0; i < 32; i++) v[i] = __float_as_uint(__fadd_rn(__uint_as_float(v[i]), __uint_as_float(u[i])));
                }
            }
        };
        issue(0, va, ua);
        tc::tmem_ld_wait();
        finish(va, ua);
#pragma unroll 1
        for (int c0 = 0; c0 < BN; c0 += 64) {
            const bool has_b = c0 + 32 < BN, has_a = c0 + 64 < BN;
            if (has_b) issue(c0 + 32, vb, ub);
            fn(c0, va);
            if (!has_b) break;
            tc::tmem_ld_wait();
            finish(vb, ub);
            if (has_a) issue(c0 + 64, va, ua);
            fn(c0 + 32, vb);
            if (has_a) {
                tc::tmem_ld_wait();
                finish(va, ua);
            }
        }
    };
    // One cluster (2..8 splits) writing dW by TMA: the ranks exchange their partial tiles' 32 x 32
    // blocks through the workspace; each block's owner copies the ranks' copies into its idle ring
    // ([blocks per rank][ranks] 4 KB slots, then 8 KB of staging per epilogue warp) and adds them.
    constexpr int NBLK = 4 * (BN / 32);
    constexpr uint32_t RECV_MAX = (uint32_t) (NBLK + 7) * 4096u;
    constexpr bool PUSH_FITS = (size_t) STAGES * C::STAGE_BYTES >= (size_t) RECV_MAX + 4 * 8192;
    const bool push = !PAIR && PUSH_FITS && p.cluster && p.xchg;

    if (IM2C && warp < 4) {
        // one thread: im2col TMA for each 64-channel X atom (a fixed tap and channel chunk
        // for the CTA, 64 consecutive pixels per stage) and tiled TMA for dY
        if (threadIdx.x == 0) {
            int a_ci[C::X_ATOMS];
            uint16_t a_oy[C::X_ATOMS], a_ox[C::X_ATOMS];
#pragma unroll
            for (int a = 0; a < C::X_ATOMS; a++) {
                const int n = min(x0 + 64 * a, p.Nx - 64);  // atoms past Nx load a valid (unused) chunk
                uint32_t tap, ci;
                p.dcp.divmod(n, tap, ci);
                a_ci[a] = ci;
                a_oy[a] = (uint16_t) (((int) tap / p.kw) * p.vdil);
                a_ox[a] = (uint16_t) (((int) tap % p.kw) * p.hdil);
            }
            const uint32_t xoff = XA ? 0 : C::A_BYTES;
            const uint32_t dyoff = XA ? C::A_BYTES : 0;
            // pairs: every load of both CTAs completes on the even CTA's full barrier
            const uint32_t lead_full = PAIR ? tc::mapa_shared(tc::smem_u32(full), 0) : 0u;
            for (int g = 0; g < NG; g++) {
                const int s = g % STAGES;
                const uint32_t ph = (g / STAGES) & 1;
                if (g >= STAGES && !(ok = tc::mbar_wait(&empty[s], ph ^ 1, p.err, 11))) break;
                const int nch = min(KB, KT - g * KB);
                if (!PAIR || prank == 0)
                    tc::mbar_arrive_expect_tx(&full[s], (PAIR ? 2 : 1) * nch * (C::X_ATOMS * C::ATOM_BYTES + C::DY_BYTES));
                const uint32_t fb = lead_full + (uint32_t) s * 8u;
                for (int c = 0; c < nch; c++) {
                    const int pbase = (chunk0 + g * KB + c) * C::BK;
                    uint32_t q, ow, oh, b;
                    p.dwo.divmod(pbase, q, ow);
                    p.dho.divmod(q, b, oh);
                    const int h0 = (int) oh * p.vstr - p.vpad, w0 = (int) ow * p.hstr - p.hpad;
                    const uint32_t st0 = tc::smem_u32(base + s * C::STAGE_BYTES + c * C::CHUNK_BYTES);
#pragma unroll
                    for (int a = 0; a < C::X_ATOMS; a++) {
                        const uint32_t d = st0 + xoff + a * C::ATOM_BYTES;
                        if (PAIR) {
                            if (p.x2d)
                                tc::tma_load_2d_pair(d, &xmap, a_ci[a], pbase, fb);
                            else
                                tc::tma_load_im2col_4d_pair(d, &xmap, a_ci[a], w0, h0, (int) b, a_ox[a], a_oy[a], fb);
                        } else if (p.x2d) {   // one tap: the atom's channels are columns a_ci of the [P][Cp] matrix
                            tc::tma_load_2d(d, &xmap, a_ci[a], pbase, &full[s]);
                        } else {
                            tc::tma_load_im2col_4d(d, &xmap, a_ci[a], w0, h0, (int) b, a_ox[a], a_oy[a], &full[s]);
                        }
                    }
#pragma unroll
                    for (int a = 0; a < C::DY_ATOMS; a++) {
                        if (PAIR)
                            tc::tma_load_2d_pair(st0 + dyoff + a * C::ATOM_BYTES, &dymap, co0 + 64 * a, pbase, fb);
                        else
                            tc::tma_load_2d(st0 + dyoff + a * C::ATOM_BYTES, &dymap, co0 + 64 * a, pbase, &full[s]);
                    }
                }
            }
        }
        // epilogue below runs on all four warps
    } else if (warp < GW) {
        const int t = threadIdx.x;
        const int piece = t & 7;
        constexpr int RSTEP = 4 * GW;   // pixel rows r0 + RSTEP*i, i < 64 / RSTEP
        const int r0 = t >> 3;
        // per X atom: the tap and channel of this thread's 8-channel piece (fixed for the CTA)
        int a_ci[C::X_ATOMS], a_oy[C::X_ATOMS], a_ox[C::X_ATOMS];
        bool a_ok[C::X_ATOMS];
#pragma unroll
        for (int a = 0; a < C::X_ATOMS; a++) {
            const int n = x0 + 64 * a + 8 * piece;
            uint32_t tap, ci;
            p.dcp.divmod(n, tap, ci);
            a_ok[a] = n < p.Nx;
            const int kx = (int) tap / p.kw, ky = (int) tap % p.kw;
            a_ci[a] = ci;
            a_oy[a] = kx * p.vdil - p.vpad;
            a_ox[a] = ky * p.hdil - p.hpad;
        }
        const uint32_t xoff = XA ? 0 : C::A_BYTES;  // X tile inside the stage
        const uint32_t dyoff = XA ? C::A_BYTES : 0;
        for (int kt = 0; kt < KT; kt++) {
            const int s = kt % STAGES;
            const uint32_t ph = (kt / STAGES) & 1;
            if (kt >= STAGES) ok = tc::mbar_wait(&empty[s], ph ^ 1, p.err, 11);
            if (!ok) break;
            const int pbase = (chunk0 + kt) * C::BK;
            const uint32_t sX = tc::smem_u32(base + s * C::STAGE_BYTES + xoff);
#pragma unroll
            for (int i = 0; i < 64 / RSTEP; i++) {
                const int r = r0 + RSTEP * i;
                const int pix = pbase + r;
                int bb = -1, iy0 = 0, ix0 = 0;
                if (pix < p.P) {
                    uint32_t q, ow, oh, b;
                    p.dwo.divmod(pix, q, ow);
                    p.dho.divmod(q, b, oh);
                    bb = b;
                    iy0 = (int) oh * p.vstr;
                    ix0 = (int) ow * p.hstr;
                }
#pragma unroll
                for (int a = 0; a < C::X_ATOMS; a++) {
                    const int iy = iy0 + a_oy[a], ix = ix0 + a_ox[a];
                    const bool v = bb >= 0 && a_ok[a] && (unsigned) iy < (unsigned) p.H && (unsigned) ix < (unsigned) p.W;
                    const bf16 *src = v ? p.x + ((((size_t) bb * p.H + iy) * p.W + ix) * p.Cp + a_ci[a]) : p.x;
                    // L1-cached: a piece is re-read by the neighbouring taps and pixels
                    tc::cp_async_16_ca(sX + a * 8192 + r * 128 + ((piece ^ (r & 7)) << 4), src, v ? 16u : 0u);
                }
            }
            tc::cp_async_commit();
            if (t == 0) {
                tc::mbar_arrive_expect_tx(&full[s], C::DY_BYTES);
                const uint32_t sD = tc::smem_u32(base + s * C::STAGE_BYTES + dyoff);
#pragma unroll
                for (int a = 0; a < C::DY_ATOMS; a++) tc::tma_load_2d(sD + a * 8192, &dymap, co0 + 64 * a, pbase, &full[s]);
            }
            if (kt >= C::LAG) {
                tc::cp_async_wait<C::LAG>();
                tc::fence_proxy_async_smem();
                tc::mbar_arrive(&full[(kt - C::LAG) % STAGES]);
            }
        }
        tc::cp_async_wait<0>();
        tc::fence_proxy_async_smem();
        if (ok)
            for (int kt = (KT > C::LAG ? KT - C::LAG : 0); kt < KT; kt++) tc::mbar_arrive(&full[kt % STAGES]);
    }
    if (warp < 4) {
        // epilogue: FP32 partial tile -> workspace [split][Mext][Next]
        if (ok) ok = tc::mbar_wait(accum, 0, p.err, 13);
        ok = __all_sync(0xffffffffu, ok);   // tcgen05.ld below is warp-collective
        tc::tc_fence_after();
        const int m = mrow0 + warp * 32 + lane;
        const int Mext = XA ? p.Nx : p.kn, Next = XA ? p.kn : p.Nx;
        float *wrow = p.ws + ((size_t) blockIdx.z * Mext + m) * Next;
        if (push) {
            // the partial tile leaves TMEM after the cluster barrier below
        } else if (!PAIR && p.cluster) {
            // this split's partial tile into shared memory (the ring is idle now), rows padded by
            // 4 floats against bank conflicts; the cluster adds the splits below
            float *R = reinterpret_cast<float *>(base);
#pragma unroll 1
            for (int c0 = 0; c0 < BN; c0 += 32) {
                uint32_t v[32];
                if (ok && KT > 0) {   // a split past the last chunk (grouped clusters) adds zero
                    ld_acc(c0, v);
                } else {
#pragma unroll
                    for (int jj = 0; jj < 32; jj++) v[jj] = 0u;
                }
                float4 *dst = reinterpret_cast<float4 *>(R + (size_t) (warp * 32 + lane) * (BN + 4) + c0);
#pragma unroll
                for (int q = 0; q < 8; q++)
                    dst[q] = make_float4(__uint_as_float(v[4 * q]), __uint_as_float(v[4 * q + 1]),
                                         __uint_as_float(v[4 * q + 2]), __uint_as_float(v[4 * q + 3]));
            }
        } else if (ok && p.direct && p.dw_tma) {
            // single split: 32 x 32 blocks staged in the idle ring (two 4 KB buffers per warp) and
            // written by TMA, one store per block (a block lies in one tap: Cp % 32 == 0)
            const uint32_t stg = tc::smem_u32(base) + (uint32_t) warp * 8192u;
            for_acc_blocks([&](int c0, const uint32_t(&v)[32]) {
                const uint32_t buf = stg + (uint32_t) ((c0 >> 5) & 1) * 4096u;
                if (c0 >= 64) {   // the store issued from this buffer two blocks ago has read it
                    if (lane == 0) wg_bulk_wait_read<1>();
                    __syncwarp();
                }
                wg_stage_block<XA>(buf, lane, v);
                tc::fence_proxy_async_smem();
                __syncwarp();
                if (lane == 0) {
                    const int nf = XA ? mrow0 + warp * 32 : ncol0 + c0;   // first K index of the block
                    const int cf = XA ? ncol0 + c0 : mrow0 + warp * 32;   // first output channel
                    uint32_t tap = 0, ci = 0;
                    if (nf < p.Nx) p.dcp.divmod((uint32_t) nf, tap, ci);
                    if (nf < p.Nx && cf < p.kn && (int) ci < p.C)
                        wg_store_3d(&p.dwmap, buf, cf, (int) tap, (int) ci);   // rows ci >= C, co >= kn clipped
                    wg_bulk_commit();
                }
            });
            if (lane == 0) wg_bulk_wait_all();
            __syncwarp();
        } else if (ok && p.direct) {
            // single split: dW written in the reference layout (lanes hold consecutive rows)
            const int khw = p.kh * p.kw;
#pragma unroll 1
            for (int c0 = 0; c0 < BN; c0 += 32) {
                uint32_t v[32];
                ld_acc(c0, v);
                if (m >= Mext) continue;
#pragma unroll 4
                for (int jj = 0; jj < 32; jj++) {
                    const int col = ncol0 + c0 + jj;
                    if (col >= Next) break;
                    const int n = XA ? m : col, co = XA ? col : m;
                    uint32_t tap, ci;
                    p.dcp.divmod((uint32_t) n, tap, ci);
                    if ((int) ci >= p.C) continue;
                    const size_t o = p.layout == 0 ? ((size_t) ci * khw + tap) * p.kn + co
                                                   : ((size_t) co * p.C + ci) * khw + tap;
                    p.dw[o] = __uint_as_float(v[jj]);
                }
            }
        } else if (ok && p.ws_tma) {
            // partial tile -> workspace [split][Mext][Next]: 32 x 32 blocks staged (rows = this
            // warp's accumulator rows) and written by TMA, clipped at Mext and Next
            const uint32_t stg = tc::smem_u32(base) + (uint32_t) warp * 8192u;
            const int mb = mrow0 + warp * 32;
            for_acc_blocks([&](int c0, const uint32_t(&v)[32]) {
                const uint32_t buf = stg + (uint32_t) ((c0 >> 5) & 1) * 4096u;
                if (c0 >= 64) {
                    if (lane == 0) wg_bulk_wait_read<1>();
                    __syncwarp();
                }
                wg_stage_block<true>(buf, lane, v);
                tc::fence_proxy_async_smem();
                __syncwarp();
                if (lane == 0) {
                    if (mb < Mext && ncol0 + c0 < Next) wg_store_part(&p.wsmap, buf, ncol0 + c0, mb, (int) blockIdx.z);
                    wg_bulk_commit();
                }
            });
            if (lane == 0) wg_bulk_wait_all();
            __syncwarp();
        } else if (ok) {
#pragma unroll 1
            for (int c0 = 0; c0 < BN; c0 += 32) {
                uint32_t v[32];
                ld_acc(c0, v);
                const int nb = ncol0 + c0;
                if (m < Mext && nb < Next) {
                    if (nb + 32 <= Next && (Next & 3) == 0) {
                        float4 *dst = reinterpret_cast<float4 *>(wrow + nb);
#pragma unroll
                        for (int q = 0; q < 8; q++)
                            dst[q] = make_float4(__uint_as_float(v[4 * q]), __uint_as_float(v[4 * q + 1]),
                                                 __uint_as_float(v[4 * q + 2]), __uint_as_float(v[4 * q + 3]));
                    } else {
#pragma unroll
                        for (int jj = 0; jj < 32; jj++)
                            if (nb + jj < Next) wrow[nb + jj] = __uint_as_float(v[jj]);
                    }
                }
            }
        }
    } else if (warp == GW || (ISS2 && warp == GW + 1)) {
        if (lane == 0 && (!PAIR || prank == 0)) {
            constexpr uint32_t idesc = tc::idesc_bf16(PAIR ? 256 : 128, BN, 1, 1);
            const int j = warp - GW;   // issuer: chunk parity it takes (ISS2), accumulator
            const uint32_t dt = tmem + (uint32_t) (j * BN);
            for (int g = 0; g < NG; g++) {
                const int s = g % STAGES;
                const uint32_t ph = (g / STAGES) & 1;
                if (!tc::mbar_wait(&full[s], ph, p.err, 12)) {
                    ok = false;
                    break;
                }
                tc::tc_fence_after();
                const int nch = min(KB, KT - g * KB);
                // descriptors built once per stage; a 16-row K step (2048 bytes) adds 128 to the start field
                const uint64_t ad0 = tc::sw128_desc(tc::smem_u32(base + s * C::STAGE_BYTES), C::ATOM_BYTES, 1024);
#pragma unroll
                for (int c = 0; c < KB; c++) {
                    if (c >= nch) break;
                    if (ISS2 && c != j) continue;
                    const uint64_t ad = ad0 + ((c * C::CHUNK_BYTES) >> 4), bd = ad + (C::A_BYTES >> 4);
#pragma unroll
                    for (int k = 0; k < C::BK / 16; k++) {
                        if constexpr (PAIR)
                            tc::mma_f16_pair(dt, ad + 128 * k, bd + 128 * k, idesc, (g | c | k) != 0);
                        else
                            tc::mma_f16(dt, ad + 128 * k, bd + 128 * k, idesc, (g | (ISS2 ? 0 : c) | k) != 0);
                    }
                }
                if constexpr (PAIR)
                    tc::mma_commit_pair(&empty[s], (uint16_t) 3);   // both CTAs' stage s is free
                else
                    tc::mma_commit(&empty[s]);
            }
            if constexpr (PAIR)
                tc::mma_commit_pair(accum, (uint16_t) 3);
            else
                tc::mma_commit(accum);
        }
        __syncwarp();
    }

    if (push) {
        // partial tiles exchanged through L2: each rank writes its 32 x 32 blocks to the workspace
        // ([tile][rank][block][32 x 32], 16-byte chunks of row r at chunk q ^ (r & 7)) by bulk
        // copies, the cluster barrier publishes them, and each block's owner (rank b % nrank)
        // copies the ranks' copies of its blocks into its idle ring, adds them in rank order and
        // writes dW by TMA
        uint32_t rank, nrank;
        asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(rank));
        asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(nrank));
        const int tile = blockIdx.x + gridDim.x * blockIdx.y;
        float *gp = p.ws + (size_t) tile * nrank * NBLK * 1024;
        if (warp < 4) {
            // each block staged in shared memory (rows = this warp's accumulator rows) and written
            // as one 4 KB bulk copy
            const uint32_t stg = tc::smem_u32(base) + RECV_MAX + (uint32_t) warp * 8192u;
            auto send = [&](int c0, const uint32_t(&v)[32]) {
                const int cb = c0 >> 5;
                const uint32_t buf = stg + (uint32_t) (cb & 1) * 4096u;
                if (cb >= 2) {
                    if (lane == 0) wg_bulk_wait_read<1>();
                    __syncwarp();
                }
                wg_stage_block<true>(buf, lane, v);
                tc::fence_proxy_async_smem();
                __syncwarp();
                if (lane == 0) {
                    wg_bulk_store(gp + ((size_t) rank * NBLK + cb * 4 + warp) * 1024, buf, 4096u);
                    wg_bulk_commit();
                }
            };
            if (ok && KT > 0) {
                for_acc_blocks(send);
            } else {   // a timed-out split adds zero
                uint32_t z[32];
#pragma unroll
                for (int jj = 0; jj < 32; jj++) z[jj] = 0u;
#pragma unroll 1
                for (int c0 = 0; c0 < BN; c0 += 32) send(c0, z);
            }
            if (lane == 0) wg_bulk_wait_all();   // written before the barrier publishes them
            __syncwarp();
            asm volatile("fence.proxy.async;" ::: "memory");
        }
        asm volatile("barrier.cluster.arrive.release.aligned;\nbarrier.cluster.wait.acquire.aligned;" ::: "memory");
        if (warp < 4) {
            asm volatile("fence.proxy.async;" ::: "memory");
            const uint32_t Rloc = tc::smem_u32(base);
            const int per = (NBLK + (int) nrank - 1) / (int) nrank;   // blocks each rank owns (at most)
            int nb = 0;
            for (int j = warp; j < per; j += 4)
                if (j * (int) nrank + (int) rank < NBLK) nb++;
            if (lane == 0 && nb > 0) {
                tc::mbar_arrive_expect_tx(&xbar[warp], (uint32_t) (nb * (int) nrank) * 4096u);
                for (int j = warp; j < per; j += 4) {
                    const int b = j * (int) nrank + (int) rank;
                    if (b >= NBLK) break;
                    for (int z = 0; z < (int) nrank; z++)
                        wg_bulk_load(Rloc + (uint32_t) (j * (int) nrank + z) * 4096u, gp + ((size_t) z * NBLK + b) * 1024,
                                     4096u, &xbar[warp]);
                }
            }
            const bool okx = nb == 0 || tc::mbar_wait(&xbar[warp], 0, p.err, 14);
            const uint32_t stg = Rloc + RECV_MAX + (uint32_t) warp * 8192u;
            int i = 0;
#pragma unroll 1
            for (int j = warp; okx && j < per; j += 4, i++) {
                const int b = j * (int) nrank + (int) rank;
                if (b >= NBLK) break;
                const int rb = b & 3, cb = b >> 2;
                float a[32];
#pragma unroll
                for (int jj = 0; jj < 32; jj++) a[jj] = 0.0f;
#pragma unroll 1
                for (int z = 0; z < (int) nrank; z++) {
                    const uint32_t src = Rloc + (uint32_t) (j * (int) nrank + z) * 4096u + (uint32_t) lane * 128u;
#pragma unroll
                    for (int q = 0; q < 8; q++) {
                        float4 t;
                        asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];"
                                     : "=f"(t.x), "=f"(t.y), "=f"(t.z), "=f"(t.w)
                                     : "r"(src + ((q ^ (lane & 7)) << 4)));
                        a[4 * q] = __fadd_rn(a[4 * q], t.x);
                        a[4 * q + 1] = __fadd_rn(a[4 * q + 1], t.y);
                        a[4 * q + 2] = __fadd_rn(a[4 * q + 2], t.z);
                        a[4 * q + 3] = __fadd_rn(a[4 * q + 3], t.w);
                    }
                }
                uint32_t v[32];
#pragma unroll
                for (int jj = 0; jj < 32; jj++) v[jj] = __float_as_uint(a[jj]);
                const uint32_t buf = stg + (uint32_t) (i & 1) * 4096u;
                if (i >= 2) {
                    if (lane == 0) wg_bulk_wait_read<1>();
                    __syncwarp();
                }
                wg_stage_block<XA>(buf, lane, v);
                tc::fence_proxy_async_smem();
                __syncwarp();
                if (lane == 0) {
                    const int nf = XA ? mrow0 + rb * 32 : ncol0 + cb * 32;
                    const int cf = XA ? ncol0 + cb * 32 : mrow0 + rb * 32;
                    uint32_t tap = 0, ci = 0;
                    if (nf < p.Nx) p.dcp.divmod((uint32_t) nf, tap, ci);
                    if (nf < p.Nx && cf < p.kn && (int) ci < p.C) wg_store_3d(&p.dwmap, buf, cf, (int) tap, (int) ci);
                    wg_bulk_commit();
                }
            }
            if (lane == 0) wg_bulk_wait_all();
            __syncwarp();
        }
    } else if (!PAIR && p.cluster) {
        // dW = sum of the cluster's partial tiles in split (cluster rank) order; rank r adds rows
        // [r*rows, (r+1)*rows) across all ranks' shared memory and writes them.  With grouped
        // clusters (p.groups > 1) the slice goes to gws instead, and the last cluster of the
        // tile to arrive adds the groups' slices in group order and writes dW.
        asm volatile("barrier.cluster.arrive.release.aligned;\nbarrier.cluster.wait.acquire.aligned;" ::: "memory");
        if (warp < 4) {
            uint32_t rank, nrank;
            asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(rank));
            asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(nrank));
            const int rows = (128 + (int) nrank - 1) / (int) nrank, r0 = (int) rank * rows;
            const int nr = min(rows, 128 - r0);
            const int Mext = XA ? p.Nx : p.kn, Next = XA ? p.kn : p.Nx, khw = p.kh * p.kw;
            const uint32_t Rloc = tc::smem_u32(base);
            const int G = p.groups > 1 ? p.groups : 1;
            const int tile = blockIdx.x + gridDim.x * blockIdx.y;
            // this cluster's slice of the tile in gws: [tile][group][128][BN]
            float *gslice = G > 1 ? p.gws + ((size_t) (tile * G + (int) (blockIdx.z / nrank)) * 128) * BN : nullptr;
            // lanes along rows when rows are dW's contiguous index (co, NHWC layout), else along columns
            const bool row_fast = !XA && p.layout == 0;
            auto write_dw = [&](int row, int c4, const float (&a)[4]) {
                const int m = mrow0 + row;
                if (m >= Mext) return;
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const int col = ncol0 + 4 * c4 + q;
                    if (col >= Next) break;
                    const int n = XA ? m : col, co = XA ? col : m;
                    uint32_t tap, ci;
                    p.dcp.divmod((uint32_t) n, tap, ci);
                    if ((int) ci >= p.C) continue;
                    const size_t o = p.layout == 0 ? ((size_t) ci * khw + tap) * p.kn + co
                                                   : ((size_t) co * p.C + ci) * khw + tap;
                    p.dw[o] = a[q];
                }
            };
            for (int e = threadIdx.x; e < nr * (BN / 4); e += 128) {
                const int rr = row_fast ? e % nr : e / (BN / 4), c4 = row_fast ? e / nr : e % (BN / 4);
                const int row = r0 + rr;
                const uint32_t off = (uint32_t) ((row * (BN + 4) + 4 * c4) * 4);
                // every rank's four values in flight at once, then added in rank order
                float4 b[16];
#pragma unroll
                for (int z = 0; z < 16; z++) {
                    if (z < (int) nrank) {
                        uint32_t ra;
                        asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(ra) : "r"(Rloc + off), "r"(z));
                        asm volatile("ld.shared::cluster.v4.f32 {%0, %1, %2, %3}, [%4];"
                                     : "=f"(b[z].x), "=f"(b[z].y), "=f"(b[z].z), "=f"(b[z].w)
                                     : "r"(ra));
                    }
                }
                float a[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
                for (int z = 0; z < 16; z++) {
                    if (z < (int) nrank) {
                        a[0] = __fadd_rn(a[0], b[z].x);
                        a[1] = __fadd_rn(a[1], b[z].y);
                        a[2] = __fadd_rn(a[2], b[z].z);
                        a[3] = __fadd_rn(a[3], b[z].w);
                    }
                }
                if (G > 1)
                    __stcg(reinterpret_cast<float4 *>(gslice + (size_t) row * BN + 4 * c4), make_float4(a[0], a[1], a[2], a[3]));
                else
                    write_dw(row, c4, a);
            }
            if (G > 1) {
                // publish this slice, then count the tile's arrivals at this rank's slice
                __threadfence();
                asm volatile("bar.sync 1, 128;" ::: "memory");
                __shared__ int s_last;
                if (threadIdx.x == 0) {
                    unsigned *cnt = p.counters + (size_t) tile * nrank + rank;
                    const unsigned old = atomicAdd(cnt, 1u);
                    s_last = old == (unsigned) (G - 1);
                    if (s_last) atomicExch(cnt, 0u);   // every group has arrived: zero for the next call
                    __threadfence();
                }
                asm volatile("bar.sync 1, 128;" ::: "memory");
                if (s_last) {
                    for (int e = threadIdx.x; e < nr * (BN / 4); e += 128) {
                        const int rr = row_fast ? e % nr : e / (BN / 4), c4 = row_fast ? e / nr : e % (BN / 4);
                        const int row = r0 + rr;
                        const float *src = p.gws + ((size_t) tile * G * 128 + row) * BN + 4 * c4;
                        float a[4] = {0.f, 0.f, 0.f, 0.f};
                        for (int g0 = 0; g0 < G; g0 += 8) {
                            float4 v[8];
#pragma unroll
                            for (int j = 0; j < 8; j++)
                                if (g0 + j < G) v[j] = __ldcg(reinterpret_cast<const float4 *>(src + (size_t) (g0 + j) * 128 * BN));
#pragma unroll
                            for (int j = 0; j < 8; j++) {
                                if (g0 + j < G) {
                                    a[0] = __fadd_rn(a[0], v[j].x);
                                    a[1] = __fadd_rn(a[1], v[j].y);
                                    a[2] = __fadd_rn(a[2], v[j].z);
                                    a[3] = __fadd_rn(a[3], v[j].w);
                                }
                            }
                        }
                        write_dw(row, c4, a);
                    }
                }
            }
        }
        // no rank leaves while another still reads its shared memory
        asm volatile("barrier.cluster.arrive.release.aligned;\nbarrier.cluster.wait.acquire.aligned;" ::: "memory");
    }
    tc::tc_fence_before();
    __syncthreads();
    if constexpr (PAIR) tc::cluster_sync();   // the pair's TMEM is released together
    tc::tc_fence_after();
    if (warp == GW) {
        if constexpr (PAIR)
            tc::tmem_dealloc_pair(tmem, TCOLS);
        else
            tc::tmem_dealloc(tmem, TCOLS);
    }
}

// First pass of the reduction when there are many splits: group g sums the
// splits [g*per, min((g+1)*per, splits)) in split order into gs[g].  The
// grouping depends only on the split count, so results stay bit-reproducible.
__global__ void wgrad_group_sum_kernel(const float *__restrict__ ws, float *__restrict__ gs, int splits, int per,
                                       size_t plane) {
    tc::pdl_wait();
    tc::pdl_trigger();
    const size_t i = blockIdx.x * (size_t) blockDim.x + threadIdx.x;
    if (i >= plane) return;
    const int z0 = blockIdx.y * per, z1 = min(splits, z0 + per);
    float s = ws[(size_t) z0 * plane + i];
    int z = z0 + 1;
    for (; z + 8 <= z1; z += 8) {
        float v[8];
#pragma unroll
        for (int j = 0; j < 8; j++) v[j] = ws[(size_t) (z + j) * plane + i];
#pragma unroll
        for (int j = 0; j < 8; j++) s = __fadd_rn(s, v[j]);
    }
    for (; z < z1; z++) s = __fadd_rn(s, ws[(size_t) z * plane + i]);
    gs[(size_t) blockIdx.y * plane + i] = s;
}

// dW = sum over splits in increasing order, written in the requested layout:
//   layout 0 (NHWC API): [ci][kh][kw][co];  layout 1 (NCHW API): [co][ci][kh][kw].
// 32 x 32 tiles of (co, n = tap*Cp + ci): the split partials are read along their
// contiguous dimension, summed z = 0, 1, ... in order, and written through shared memory.
__global__ void wgrad_reduce_kernel(const float *__restrict__ ws, float *__restrict__ dw, int splits, int xa, int Nx,
                                    int kn, int C, int Cp, int khw, int layout) {
    tc::pdl_wait();
    tc::pdl_trigger();
    __shared__ float tile[32][33];
    const int co0 = blockIdx.x * 32, n0 = blockIdx.y * 32;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const size_t plane = (size_t) Nx * kn;
    for (int k = 0; k < 4; k++) {
        const int r = ty + 8 * k;
        int co, n;
        size_t off;
        if (xa) {  // partials [n][co]: read along co
            n = n0 + r;
            co = co0 + tx;
            off = (size_t) n * kn + co;
        } else {   // partials [co][n]: read along n
            co = co0 + r;
            n = n0 + tx;
            off = (size_t) co * Nx + n;
        }
        float s = 0.0f;
        if (co < kn && n < Nx) {
            // loads eight splits ahead, adds strictly in split order
            s = ws[off];
            int z = 1;
            for (; z + 8 <= splits; z += 8) {
                float v[8];
#pragma unroll
                for (int j = 0; j < 8; j++) v[j] = ws[(size_t) (z + j) * plane + off];
#pragma unroll
                for (int j = 0; j < 8; j++) s = __fadd_rn(s, v[j]);
            }
            for (; z < splits; z++) s = __fadd_rn(s, ws[(size_t) z * plane + off]);
        }
        if (xa) tile[tx][r] = s;   // tile[co][n]
        else tile[r][tx] = s;
    }
    __syncthreads();
    for (int k = 0; k < 4; k++) {
        const int r = ty + 8 * k;
        int co, n;
        if (layout == 0) {  // write along co
            co = co0 + tx;
            n = n0 + r;
        } else {            // write along n
            co = co0 + r;
            n = n0 + tx;
        }
        if (co >= kn || n >= Nx) continue;
        const int tap = n / Cp, ci = n - tap * Cp;
        if (ci >= C) continue;
        const size_t o = layout == 0 ? ((size_t) ci * khw + tap) * kn + co : ((size_t) co * C + ci) * khw + tap;
        dw[o] = layout == 0 ? tile[tx][r] : tile[r][tx];
    }
}

template <int BN, int STAGES, bool XA, bool IM2C, int KB = 1, bool ISS2 = false, int BKP = 64, bool PAIR = false>
cudaError_t launch_wg(const TcWgradParams &p, const CUtensorMap &map, const CUtensorMap &xmap, dim3 grid,
                      cudaStream_t st) {
    using C = WgCfg<BN, STAGES, XA, KB, BKP, PAIR>;
    auto kern = tc_wgrad_kernel<BN, STAGES, XA, IM2C, KB, ISS2, BKP, PAIR>;
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) C::SMEM);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    // Weight-gradient work runs beside the forward / input-gradient chain on a side
    // stream: launched without programmatic serialization, so that its grids do not
    // hold SMs early while the persistent chain kernels want them.
    constexpr int THREADS = WgWarps<IM2C, ISS2>::THREADS;
    if (!PAIR && !p.cluster) return cg_launch_ex(CG_PDL_OFF, kern, grid, dim3(THREADS), C::SMEM, st, p, map, xmap);
    // the splits of one tile as a cluster along z
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = dim3(THREADS);
    cfg.dynamicSmemBytes = C::SMEM;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = PAIR ? 2 : 1;   // pairs: adjacent M tiles (grid.x is even)
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = PAIR ? 1 : (p.groups > 1 ? p.csize : grid.z);
    cfg.attrs = at;
    cfg.numAttrs = 1;
    cg_note_launch();
    return cudaLaunchKernelEx(&cfg, kern, p, map, xmap);
}

// Whether `splits` CTAs of this configuration can be resident together as one cluster.
template <int BN, int STAGES, bool XA, bool IM2C, int KB = 1, bool ISS2 = false, int BKP = 64>
bool cluster_fits(int splits) {
    using C = WgCfg<BN, STAGES, XA, KB, BKP>;
    auto kern = tc_wgrad_kernel<BN, STAGES, XA, IM2C, KB, ISS2, BKP>;
    static int cached[9] = {-1, -1, -1, -1, -1, -1, -1, -1, -1};
    if (splits < 2 || splits > 8) return false;
    if (cached[splits] < 0) {
        if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) C::SMEM) != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(1, 1, splits);
        cfg.blockDim = dim3(WgWarps<IM2C, ISS2>::THREADS);
        cfg.dynamicSmemBytes = C::SMEM;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = 1;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = splits;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        int n = 0;
        if (cudaOccupancyMaxActiveClusters(&n, kern, &cfg) != cudaSuccess) {
            cudaGetLastError();
            n = 0;
        }
        cached[splits] = n;
    }
    return cached[splits] > 0;
}

// im2col path: two 64-pixel chunks per stage (64-wide tiles: 2 stages of 48 KB, two CTAs
// per SM; 128 / 256-wide: 3 x 64 KB / 2 x 96 KB); cp.async path: one chunk per stage.
template <bool IM2C>
cudaError_t launch_wg_any(const TcWgradParams &p, const CUtensorMap &dymap, const CUtensorMap &xmap, int bn, int xa,
                          dim3 grid, cudaStream_t st) {
    if constexpr (IM2C) {
        if (p.pair) {   // CTA pairs, 128-pixel chunks: 256 x 256 tiles, 3 stages of 64 KB per CTA; 256 x 128, 4 x 48 KB
            if ((bn != 128 && bn != 256) || (grid.x & 1)) return cudaErrorInvalidValue;
            if (bn == 128)
                return xa ? launch_wg<128, 4, true, IM2C, 1, false, 128, true>(p, dymap, xmap, grid, st)
                          : launch_wg<128, 4, false, IM2C, 1, false, 128, true>(p, dymap, xmap, grid, st);
            return xa ? launch_wg<256, 3, true, IM2C, 1, false, 128, true>(p, dymap, xmap, grid, st)
                      : launch_wg<256, 3, false, IM2C, 1, false, 128, true>(p, dymap, xmap, grid, st);
        }
        if (p.kb1) {   // one chunk per stage: 64-wide 4 stages of 24 KB, 128-wide 6 x 32 KB, 256-wide 4 x 48 KB
            if (xa) {
                switch (bn) {
                    case 64: return launch_wg<64, 4, true, IM2C, 1>(p, dymap, xmap, grid, st);
                    case 128: return launch_wg<128, 6, true, IM2C, 1>(p, dymap, xmap, grid, st);
                    case 256: return launch_wg<256, 4, true, IM2C, 1>(p, dymap, xmap, grid, st);
                    default: return cudaErrorInvalidValue;
                }
            }
            switch (bn) {
                case 64: return launch_wg<64, 4, false, IM2C, 1>(p, dymap, xmap, grid, st);
                case 128: return launch_wg<128, 6, false, IM2C, 1>(p, dymap, xmap, grid, st);
                case 256: return launch_wg<256, 4, false, IM2C, 1>(p, dymap, xmap, grid, st);
                default: return cudaErrorInvalidValue;
            }
        }
        if (p.wide) {   // 128-pixel chunks, one per stage (each TMA box twice the bytes)
            if (xa) {
                switch (bn) {
                    case 64: return launch_wg<64, 4, true, IM2C, 1, false, 128>(p, dymap, xmap, grid, st);
                    case 128: return launch_wg<128, 3, true, IM2C, 1, false, 128>(p, dymap, xmap, grid, st);
                    case 256: return launch_wg<256, 2, true, IM2C, 1, false, 128>(p, dymap, xmap, grid, st);
                    default: return cudaErrorInvalidValue;
                }
            }
            switch (bn) {
                case 64: return launch_wg<64, 4, false, IM2C, 1, false, 128>(p, dymap, xmap, grid, st);
                case 128: return launch_wg<128, 3, false, IM2C, 1, false, 128>(p, dymap, xmap, grid, st);
                case 256: return launch_wg<256, 2, false, IM2C, 1, false, 128>(p, dymap, xmap, grid, st);
                default: return cudaErrorInvalidValue;
            }
        }
        if (p.iss2) {   // two MMA issuers on the two-chunk stages
            if (xa) {
                switch (bn) {
                    case 64: return launch_wg<64, 2, true, IM2C, 2, true>(p, dymap, xmap, grid, st);
                    case 128: return launch_wg<128, 3, true, IM2C, 2, true>(p, dymap, xmap, grid, st);
                    case 256: return launch_wg<256, 2, true, IM2C, 2, true>(p, dymap, xmap, grid, st);
                    default: return cudaErrorInvalidValue;
                }
            }
            switch (bn) {
                case 64: return launch_wg<64, 2, false, IM2C, 2, true>(p, dymap, xmap, grid, st);
                case 128: return launch_wg<128, 3, false, IM2C, 2, true>(p, dymap, xmap, grid, st);
                case 256: return launch_wg<256, 2, false, IM2C, 2, true>(p, dymap, xmap, grid, st);
                default: return cudaErrorInvalidValue;
            }
        }
        if (xa) {
            switch (bn) {
                case 64: return launch_wg<64, 2, true, IM2C, 2>(p, dymap, xmap, grid, st);
                case 128: return launch_wg<128, 3, true, IM2C, 2>(p, dymap, xmap, grid, st);
                case 256: return launch_wg<256, 2, true, IM2C, 2>(p, dymap, xmap, grid, st);
                default: return cudaErrorInvalidValue;
            }
        }
        switch (bn) {
            case 64: return launch_wg<64, 2, false, IM2C, 2>(p, dymap, xmap, grid, st);
            case 128: return launch_wg<128, 3, false, IM2C, 2>(p, dymap, xmap, grid, st);
            case 256: return launch_wg<256, 2, false, IM2C, 2>(p, dymap, xmap, grid, st);
            default: return cudaErrorInvalidValue;
        }
    } else {
        if (xa) {
            switch (bn) {
                case 64: return launch_wg<64, 4, true, IM2C>(p, dymap, xmap, grid, st);
                case 128: return launch_wg<128, 3, true, IM2C>(p, dymap, xmap, grid, st);
                default: return cudaErrorInvalidValue;
            }
        }
        switch (bn) {
            case 64: return launch_wg<64, 4, false, IM2C>(p, dymap, xmap, grid, st);
            case 128: return launch_wg<128, 3, false, IM2C>(p, dymap, xmap, grid, st);
            case 256: return launch_wg<256, 4, false, IM2C>(p, dymap, xmap, grid, st);
            default: return cudaErrorInvalidValue;
        }
    }
}

}  // namespace

namespace {
// Tile counters of the grouped cluster reduction: zero at load, and every launch leaves the
// words it used at zero (the last cluster of each tile resets its counter).  Launches take
// consecutive ranges in turn, so that work queued on different streams uses different words.
constexpr int WG_COUNTERS = 1 << 16;
__device__ unsigned g_wgrad_counters[WG_COUNTERS];
std::mutex g_cnt_mu;
unsigned *g_cnt_base[64];
int g_cnt_next[64];
}  // namespace

unsigned *tc_wgrad_counters(int n) {
    int dev = 0;
    if (n <= 0 || n > WG_COUNTERS || cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
    std::lock_guard<std::mutex> lk(g_cnt_mu);
    if (!g_cnt_base[dev]) {
        void *a = nullptr;
        if (cudaGetSymbolAddress(&a, g_wgrad_counters) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        g_cnt_base[dev] = (unsigned *) a;
    }
    if (g_cnt_next[dev] + n > WG_COUNTERS) g_cnt_next[dev] = 0;
    unsigned *r = g_cnt_base[dev] + g_cnt_next[dev];
    g_cnt_next[dev] += (n + 31) / 32 * 32;
    return r;
}

bool tc_wgrad_cluster_ok(int bn, int xa, int im2col, int splits, int kb1, int iss2, int wide) {
    if (splits < 2 || splits > 8 || !cg_wgrad_cluster_enabled()) return false;
    if (im2col && wide) {
        if (xa) return bn == 64    ? cluster_fits<64, 4, true, true, 1, false, 128>(splits)
                       : bn == 128 ? cluster_fits<128, 3, true, true, 1, false, 128>(splits)
                                   : bn == 256 && cluster_fits<256, 2, true, true, 1, false, 128>(splits);
        return bn == 64    ? cluster_fits<64, 4, false, true, 1, false, 128>(splits)
               : bn == 128 ? cluster_fits<128, 3, false, true, 1, false, 128>(splits)
                           : bn == 256 && cluster_fits<256, 2, false, true, 1, false, 128>(splits);
    }
    if (im2col && iss2 && !kb1) {
        if (xa) return bn == 64    ? cluster_fits<64, 2, true, true, 2, true>(splits)
                       : bn == 128 ? cluster_fits<128, 3, true, true, 2, true>(splits)
                                   : bn == 256 && cluster_fits<256, 2, true, true, 2, true>(splits);
        return bn == 64    ? cluster_fits<64, 2, false, true, 2, true>(splits)
               : bn == 128 ? cluster_fits<128, 3, false, true, 2, true>(splits)
                           : bn == 256 && cluster_fits<256, 2, false, true, 2, true>(splits);
    }
    if (im2col && kb1) {
        if (xa) return bn == 64    ? cluster_fits<64, 4, true, true, 1>(splits)
                       : bn == 128 ? cluster_fits<128, 6, true, true, 1>(splits)
                                   : bn == 256 && cluster_fits<256, 4, true, true, 1>(splits);
        return bn == 64    ? cluster_fits<64, 4, false, true, 1>(splits)
               : bn == 128 ? cluster_fits<128, 6, false, true, 1>(splits)
                           : bn == 256 && cluster_fits<256, 4, false, true, 1>(splits);
    }
    if (im2col) {
        if (xa) return bn == 64    ? cluster_fits<64, 2, true, true, 2>(splits)
                       : bn == 128 ? cluster_fits<128, 3, true, true, 2>(splits)
                                   : bn == 256 && cluster_fits<256, 2, true, true, 2>(splits);
        return bn == 64    ? cluster_fits<64, 2, false, true, 2>(splits)
               : bn == 128 ? cluster_fits<128, 3, false, true, 2>(splits)
                           : bn == 256 && cluster_fits<256, 2, false, true, 2>(splits);
    }
    if (xa) return bn == 64 ? cluster_fits<64, 4, true, false>(splits) : bn == 128 && cluster_fits<128, 3, true, false>(splits);
    return bn == 64    ? cluster_fits<64, 4, false, false>(splits)
           : bn == 128 ? cluster_fits<128, 3, false, false>(splits)
                       : bn == 256 && cluster_fits<256, 4, false, false>(splits);
}

int tc_wgrad_stages(int bn, int im2col, int kb1, int wide, int pair) {
    if (im2col && pair) return bn == 128 ? 4 : 3;
    if (im2col && wide) return bn == 64 ? 4 : (bn == 128 ? 3 : 2);
    if (im2col) return kb1 ? (bn == 128 ? 6 : 4) : (bn == 128 ? 3 : 2);
    return bn == 128 ? 3 : 4;
}

cudaError_t tc_wgrad_launch(const TcWgradParams &p, const CUtensorMap &dymap, const CUtensorMap &xmap, int bn, int xa,
                            int mtiles, int ntiles, int splits, cudaStream_t st) {
    dim3 grid(mtiles, ntiles, splits);
    return p.im2col ? launch_wg_any<true>(p, dymap, xmap, bn, xa, grid, st)
                    : launch_wg_any<false>(p, dymap, xmap, bn, xa, grid, st);
}

int tc_wgrad_groups(int splits) {
    if (splits <= 16) return 0;
    int g = splits / 8;   // about eight splits per group
    if (g > 32) g = 32;
    const int per = (splits + g - 1) / g;
    return (splits + per - 1) / per;   // every group non-empty
}

cudaError_t tc_wgrad_reduce(float *ws, float *dw, int splits, int xa, int Nx, int kn, int C, int Cp, int kh, int kw,
                            int layout, cudaStream_t st) {
    const size_t plane = (size_t) Nx * kn;
    const int groups = tc_wgrad_groups(splits);
    const float *src = ws;
    int n = splits;
    if (groups) {
        float *gs = ws + (size_t) splits * plane;
        const int per = (splits + groups - 1) / groups;
        dim3 g1((unsigned) ((plane + 255) / 256), groups);
        if (cudaError_t e = cg_launch_ex(CG_PDL_OFF, wgrad_group_sum_kernel, g1, dim3(256), 0, st, (const float *) ws, gs, splits,
                                         per, plane))
            return e;
        src = gs;
        n = groups;
    }
    dim3 grid((kn + 31) / 32, (Nx + 31) / 32), block(32, 8);
    return cg_launch_ex(CG_PDL_OFF, wgrad_reduce_kernel, grid, block, 0, st, src, dw, n, xa, Nx, kn, C, Cp, kh * kw, layout);
}

// ------------------------------------------------------------ bias gradient
// db[co] = sum over the P pixels of dY[p][co] (dY BF16 [P][ld]), FP32, in a fixed
// order: pass 1 sums `rows` consecutive pixels per (group, 64-channel chunk) with
// four interleaved row streams combined in order; pass 2 adds the groups in order.
namespace {

__global__ void __launch_bounds__(256) bias_grad_pass1(const __nv_bfloat16 *__restrict__ dy, int P, int kn, int ld,
                                                       int rows, float *__restrict__ part) {
    __shared__ float acc[4][64];
    const int ch = blockIdx.x * 64 + (threadIdx.x & 63), r0 = threadIdx.x >> 6;
    const int p0 = blockIdx.y * rows, p1 = min(P, p0 + rows);
    float sacc = 0.0f;
    if (ch < kn)
        for (int p = p0 + r0; p < p1; p += 4) sacc = __fadd_rn(sacc, __bfloat162float(dy[(size_t) p * ld + ch]));
    acc[r0][threadIdx.x & 63] = sacc;
    __syncthreads();
    if (r0 == 0 && ch < kn)
        part[(size_t) blockIdx.y * kn + ch] =
            __fadd_rn(__fadd_rn(__fadd_rn(acc[0][threadIdx.x], acc[1][threadIdx.x]), acc[2][threadIdx.x]),
                      acc[3][threadIdx.x]);
}

__global__ void bias_grad_pass2(const float *__restrict__ part, int groups, int kn, float *__restrict__ db) {
    const int ch = blockIdx.x * blockDim.x + threadIdx.x;
    if (ch >= kn) return;
    float sacc = 0.0f;
    for (int g = 0; g < groups; g++) sacc = __fadd_rn(sacc, part[(size_t) g * kn + ch]);
    db[ch] = sacc;
}

}  // namespace

int tc_bias_grad_groups(long long P) {
    long long g = (P + 1023) / 1024;   // about 1024 pixels per group
    return (int) (g > 256 ? 256 : (g < 1 ? 1 : g));
}

cudaError_t tc_bias_grad(const void *dy, long long P, int kn, int ld, float *db, float *part, cudaStream_t st) {
    const int groups = tc_bias_grad_groups(P);
    const int rows = (int) ((P + groups - 1) / groups);
    dim3 g1((kn + 63) / 64, groups);
    bias_grad_pass1<<<g1, 256, 0, st>>>((const __nv_bfloat16 *) dy, (int) P, kn, ld, rows, part); cg_note_launch();
    bias_grad_pass2<<<(kn + 127) / 128, 128, 0, st>>>(part, groups, kn, db); cg_note_launch();
    return cudaGetLastError();
}

