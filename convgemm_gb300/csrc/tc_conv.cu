// BF16 tensor-core implicit-GEMM convolution (sm_103a, tcgen05 + TMEM + TMA).
//
// One kernel serves the forward pass (sconvGemmNHWC 'N', src/convGemm.c:65-70)
// and the input gradient (sconvGemmNHWC_back, src/convGemm.c:82-97), which it
// computes in gather form: every input-gradient pixel collects the taps that
// reach it, so there is no col2im/row2im scatter (src/im2row_nhwc.c:231-267)
// and no atomics.  A stride > 1 input gradient is split into stride-phase
// classes (pixels with the same (ih + pad) mod stride see the same taps), each
// a dense implicit GEMM of its own; their tiles share one launch.
//
// GEMM view of one class: D[m, n] = sum_k A[m, k] * B[n, k]
//   m = output pixel of the class (128 per tile),
//   n = output channel (BN per tile, in TMEM columns),
//   k = tap * Cin + ci over the class's taps (64 per pipeline stage).
// A comes straight from the NHWC activation into the 128-byte-swizzled K-major
// layout the tensor core reads: by im2col-mode TMA (128 pixels x 64 channels of
// one tap per load, out-of-range taps zero-filled) when the channels come in
// blocks of 64, else by 16-byte cp.async gathers, zero-filled for padding — no
// im2row buffer exists anywhere.  B is the packed weight matrix [Cout][K]
// loaded by TMA.  The FP32 accumulator lives in TMEM.
//
// The kernel is persistent: each CTA walks tiles blockIdx.x, +gridDim.x, ...
// with two TMEM accumulators, so the epilogue of one tile runs while the MMAs
// of the next accumulate.  Warp roles (288 threads):
//   warps 0-3  load A (one thread issuing the im2col TMA, or all four warps
//              gathering), thread 0 also issues the B TMA; stage ring of STAGES;
//   warps 4-7  epilogue: TMEM -> registers (tcgen05.ld), scale/shift/ReLU,
//              BF16, then either a 128-byte-swizzled shared-memory tile and a
//              TMA store (pixels contiguous in the output), or direct stores
//              (the strided pixels of an input-gradient class);
//   warp 8     allocates TMEM; one lane issues tcgen05.mma and the commits.
#include <cuda_bf16.h>

#include "cg_common.cuh"
#include "tc_conv.h"
#include "tc_epi.cuh"
#include "tc_ptx.cuh"

namespace {

using bf16 = __nv_bfloat16;

// Operand forms of the kernel.
constexpr int MODE_BF16 = 0;  // BF16 x BF16, kind::f16
constexpr int MODE_FP8 = 1;   // E4M3 x E4M3, kind::f8f6f4 (64-byte K rows, 64-byte swizzle)
constexpr int MODE_X3 = 2;    // 3xBF16: hi*hi + hi*lo + lo*hi into one accumulator, FP32 output
constexpr int MODE_FP8W = 3;  // E4M3 with 128-channel K blocks: 128-byte K rows, 128-byte swizzle

// KB 64-deep K blocks per pipeline stage: one full barrier and one MMA commit
// cover KB blocks (a barrier round trip costs ~400 cycles, a 128 x 64 x 64 block
// of BF16 MMAs ~150).
// MT 128-row M tiles share every weight tile: each K block loads MT activation
// tiles and one weight tile and issues MT MMAs into MT accumulators, which cuts
// the shared-memory bytes per FLOP (the operand delivery from L2 bounds the kernel).
// EW epilogue warps: 4 (one per TMEM lane quarter), or 8 (two per quarter, taking
// alternate 64-column chunks) for short-K tiles, whose time goes to the epilogue's
// latency chain (TMEM load, scale/shift, convert, staging) rather than the MMAs.
template <int BN, int STAGES, int KB = 1, int MODE = MODE_BF16, int MT = 1, int EW = 4>
struct TcCfg {
    static constexpr int BM = 128, BK = MODE == MODE_FP8W ? 128 : 64;   // K elements per block
    static constexpr int ROWB = MODE == MODE_FP8 ? 64 : 128;  // bytes of one K row of a block
    static constexpr int NOPS = MODE == MODE_X3 ? 2 : 1;      // hi / lo copies of each operand
    static constexpr uint32_t A_TILE = BM * ROWB;
    static constexpr uint32_t B_TILE = BN * ROWB;
    static constexpr uint32_t A_BLOCK = NOPS * A_TILE;
    static constexpr uint32_t B_BLOCK = NOPS * B_TILE;
    static constexpr uint32_t A_BYTES = KB * MT * A_BLOCK;
    static constexpr uint32_t B_BYTES = KB * B_BLOCK;
    static constexpr uint32_t STAGE_BYTES = A_BYTES + B_BYTES;
    static constexpr uint32_t SBO = 8 * ROWB;                  // 8-row swizzle atom
    static constexpr uint32_t LAYOUT = ROWB == 128 ? 2 : 4;    // SWIZZLE_128B / SWIZZLE_64B
    static constexpr bool OUTF32 = MODE == MODE_X3;
    static constexpr int CW = OUTF32 ? 32 : 64;                // output columns per 128-byte staging row
    static constexpr uint32_t EPI_BYTES = EW * 32 * 128;       // one 32-row x 128-byte chunk per epilogue warp
    // cp.async groups in flight per producer thread; the other STAGES - LAG slots let the
    // MMA run ahead of the arrivals (LAG = STAGES - 1 would lock the two in step)
    static constexpr int LAG = STAGES / 2;
    // shared tables: tap offsets, the class table, scale/shift (whole vectors up to 1024 channels)
    static constexpr size_t TAB_BYTES = TC_MAXCLS * TC_MAXTAPS * 4 + TC_MAXCLS * 128 + 2 * 1024 * 4;
    // output staging buffers: two when they fit beside the stage ring, else one
    static constexpr int EPI_BUFS =
        (1024 + (size_t) STAGES * STAGE_BYTES + 2 * EPI_BYTES + 256 + TAB_BYTES <= 232448) ? 2 : 1;
    static constexpr size_t SMEM = 1024 + (size_t) STAGES * STAGE_BYTES + EPI_BUFS * EPI_BYTES + 256 + TAB_BYTES;
    static_assert(SMEM <= 232448, "shared memory above the 227 KB per-block limit");
    static_assert(EW == 4 || EW == 8, "four or eight epilogue warps");
    // warps: 0 producer (0-3 on the cp.async path), 4..4+EW-1 epilogue, the MMA issuer in
    // warp 8 (EW = 4) or in the otherwise idle warp 1 (EW = 8)
    static constexpr int THREADS = EW == 8 ? 384 : 288;
    static constexpr int MMA_WARP = EW == 8 ? 1 : 8;
    static constexpr int ISS2_WARP = EW == 8 ? 2 : 1;   // the second MMA issuer (an otherwise idle warp)
    static constexpr int NCH = BN / CW;   // output chunks of one accumulator
    // TMEM: MT accumulators of BN columns, double-buffered when 512 columns allow (four buffers
    // for tiles of <= 128 columns)
    static constexpr int ACC_BUFS = BN * MT <= 128 ? 4 : (2 * BN * MT <= 512 ? 2 : 1);
    static constexpr uint32_t TMEM_COLS = ACC_BUFS * BN * MT;
};

__device__ __forceinline__ uint64_t op_desc(uint32_t saddr, uint32_t sbo, uint32_t layout) {
    uint64_t d = tc::sw128_desc(saddr, 16, sbo);
    d &= ~((uint64_t) 7 << 61);
    return d | ((uint64_t) layout << 61);
}

__device__ __forceinline__ uint32_t pack_bf16x2(float a, float b) {
    __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<uint32_t *>(&v);
}

template <int N>
__device__ __forceinline__ void epi_bar() { asm volatile("bar.sync 1, %0;" ::"n"(N) : "memory"); }

__device__ __forceinline__ void tma_store_2d(const CUtensorMap *map, uint32_t src, int x, int y) {
    asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%2, %3}], [%1];" ::"l"((uint64_t) map),
                 "r"(src), "r"(x), "r"(y)
                 : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void bulk_wait_read() {
    asm volatile("cp.async.bulk.wait_group.read %0;" ::"n"(N) : "memory");
}
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

struct Tile {
    int cls, m0, n0;
};

// The scalars of a class, copied to shared memory at kernel start (reading the
// kernel parameters with a runtime class index would cost generic-memory loads
// on every tile).
struct ClsS {
    int Hg, Wg, oy0, ox0, osy, osx, isy, isx, iby, ibx, ntaps, kbeg, ktiles, tile0, lo_y, lo_x, mint_y, mint_x, gbase;
    FastDiv dwg, dhg;
};
static_assert(sizeof(ClsS) <= 128, "class table entry");

__device__ __forceinline__ Tile decode_tile(const ClsS *cls, int ncls, int ntiles, int bn, int t, int mt = 1) {
    int c = 0;
    while (c + 1 < ncls && t >= cls[c + 1].tile0) c++;
    const int local = t - cls[c].tile0;
    Tile tl;
    tl.cls = c;
    tl.m0 = (local / ntiles) * 128 * mt;
    tl.n0 = (local % ntiles) * bn;
    return tl;
}

template <int BN, int STAGES, int KB, bool IM2C, int MODE, int MT, int EW, bool STATS>
__global__ void __launch_bounds__(EW == 8 ? 384 : 288, 1)
    tc_conv_kernel(const __grid_constant__ TcConvParams p, const __grid_constant__ CUtensorMap wmap,
                   const __grid_constant__ CUtensorMap omap, const __grid_constant__ TcMaps amaps) {
    using C = TcCfg<BN, STAGES, KB, MODE, MT, EW>;
    static_assert(EW == 4 || (IM2C && MT * C::NCH >= 2), "eight epilogue warps: im2col path, two chunks or more");
    // Two MMA-issuing threads on the BF16 im2col path: one per M tile (MT = 2), or one per N half
    // (MT = 1, BN >= 128).  One thread's instruction stream issues N <= 128 MMAs more slowly than the
    // tensor core runs them; both wait for the same stage and commit to it.
    constexpr bool SPLIT = IM2C && MODE == MODE_BF16 && (MT == 2 || BN >= 128);
    static_assert(IM2C || (KB == 1 && MODE == MODE_BF16), "the cp.async gather fills one BF16 K block per stage");
    static_assert(MT == 1 || (IM2C && MODE == MODE_BF16), "two M tiles per weight tile: BF16 im2col path only");
    extern __shared__ uint8_t smem_raw[];
    uint8_t *base = (uint8_t *) (((uintptr_t) smem_raw + 1023) & ~(uintptr_t) 1023);
    uint8_t *epi_smem = base + STAGES * C::STAGE_BYTES;
    uint64_t *full = (uint64_t *) (epi_smem + C::EPI_BUFS * C::EPI_BYTES);
    uint64_t *empty = full + STAGES;
    uint64_t *acc_full = empty + STAGES;
    uint64_t *acc_empty = acc_full + 4;
    uint32_t *tmem_holder = (uint32_t *) (acc_empty + 4);
    // per-class tap offsets (packed y:16 | x:16) and the tile's epilogue scale/shift, in shared
    // memory: indexing the kernel parameters with runtime values would go through slow generic loads
    int32_t *tap_tab = (int32_t *) (epi_smem + C::EPI_BUFS * C::EPI_BYTES + 256);
    ClsS *cls_tab = (ClsS *) (tap_tab + TC_MAXCLS * TC_MAXTAPS);
    float *sc_tab = (float *) (cls_tab + TC_MAXCLS);   // [1024]: all channels, or the tile's BN
    float *sh_tab = sc_tab + 1024;
    const bool sc_all = p.Cout <= 1024;              // whole scale/shift vectors fit

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; s++) {
            // im2col: the one expect_tx arrival; gather: 128 producer threads + the expect_tx
            tc::mbar_init(&full[s], IM2C ? 1 : 128 + 1);
            tc::mbar_init(&empty[s], SPLIT ? 2 : 1);
        }
        for (int b = 0; b < C::ACC_BUFS; b++) {
            tc::mbar_init(&acc_full[b], SPLIT ? 2 : 1);
            tc::mbar_init(&acc_empty[b], 32 * EW);
        }
        tc::fence_mbar_init();
        tc::prefetch_tmap(&wmap);
        if (p.epi_tma) tc::prefetch_tmap(&omap);
        if (IM2C)
            for (int c = 0; c < p.ncls; c++) {
                tc::prefetch_tmap(&amaps.a[c]);
                if (MODE == MODE_X3) tc::prefetch_tmap(&amaps.alo[c]);
            }
        if (MODE == MODE_X3) tc::prefetch_tmap(&amaps.wlo);
    }
    for (int i = threadIdx.x; i < p.ncls * TC_MAXTAPS; i += blockDim.x) {
        const int c = i / TC_MAXTAPS, t = i % TC_MAXTAPS;
        tap_tab[i] = ((int32_t) p.cls[c].toy[t] << 16) | ((int32_t) p.cls[c].tox[t] & 0xFFFF);
    }
    if (threadIdx.x < (unsigned) p.ncls) {
        const TcClass &c = p.cls[threadIdx.x];
        ClsS &d = cls_tab[threadIdx.x];
        d.Hg = c.Hg; d.Wg = c.Wg; d.oy0 = c.oy0; d.ox0 = c.ox0; d.osy = c.osy; d.osx = c.osx;
        d.isy = c.isy; d.isx = c.isx; d.iby = c.iby; d.ibx = c.ibx; d.ntaps = c.ntaps; d.kbeg = c.kbeg;
        d.ktiles = c.ktiles; d.tile0 = c.tile0; d.lo_y = c.lo_y; d.lo_x = c.lo_x; d.mint_y = c.mint_y;
        d.mint_x = c.mint_x; d.gbase = c.gbase; d.dwg = c.dwg; d.dhg = c.dhg;
    }
    // everything above touched only shared memory and kernel parameters; the next kernel may
    // launch once every CTA has started its last tile (pdl_trigger in the producer loop), so
    // its waiting CTAs do not hold SMs that work on other streams could use
    tc::pdl_wait();
    if (sc_all)
        for (int n = threadIdx.x; n < p.Cout; n += blockDim.x) {
            sc_tab[n] = p.scale ? __ldg(p.scale + n) : 1.0f;
            sh_tab[n] = p.shift ? __ldg(p.shift + n) : 0.0f;
        }
    if (warp == C::MMA_WARP) {
        tc::tmem_alloc(tmem_holder, C::TMEM_COLS);
        tc::tmem_relinquish();
    }
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tmem = *tmem_holder;
    bool ok = true;

    if (IM2C && warp < 4 && warp != C::MMA_WARP && !(SPLIT && warp == C::ISS2_WARP)) {
        // ------------------------------------------------ producer: one thread, im2col TMA for A, TMA for B
        if (threadIdx.x == 0) {
            uint32_t it = 0;
            for (int tile = blockIdx.x; tile < p.ntiles_total && ok; tile += gridDim.x) {
                if (tile + (int) gridDim.x >= p.ntiles_total) tc::pdl_trigger();   // this CTA's last tile
                const Tile tl = decode_tile(cls_tab, p.ncls, p.ntiles, BN, tile, MT);
                const ClsS &cl = cls_tab[tl.cls];
                const int32_t *taps = tap_tab + tl.cls * TC_MAXTAPS;
                const int ktiles = cl.ktiles, kbeg = cl.kbeg, mint_y = cl.mint_y, mint_x = cl.mint_x;
                int h0[MT], w0[MT], bb0[MT];   // im2col start of each M tile (beyond the class: zero-filled)
#pragma unroll
                for (int mt = 0; mt < MT; mt++) {
                    uint32_t q, jw, j, b;
                    cl.dwg.divmod(tl.m0 + mt * 128, q, jw);
                    cl.dhg.divmod(q, b, j);
                    h0[mt] = (int) j * cl.isy + cl.lo_y;
                    w0[mt] = (int) jw * cl.isx + cl.lo_x;
                    bb0[mt] = (int) b;
                }
                const CUtensorMap *am = &amaps.a[tl.cls];
                int tap = 0, ci0 = 0;   // k = tap*Cin + ci0, walked incrementally
                for (int kt = 0; kt < ktiles; kt += KB, it++) {
                    const int s = it % STAGES;
                    const uint32_t ph = (it / STAGES) & 1;
                    if (it >= (uint32_t) STAGES && !(ok = tc::mbar_wait(&empty[s], ph ^ 1, p.err, 1))) break;
                    const int nkb = min(KB, ktiles - kt);
                    const uint32_t sa = tc::smem_u32(base + s * C::STAGE_BYTES);
                    tc::mbar_arrive_expect_tx(&full[s], nkb * (MT * C::A_BLOCK + C::B_BLOCK));
                    for (int kb = 0; kb < nkb; kb++) {
                        const int32_t to = taps[tap];
                        const uint16_t offy = (uint16_t) ((to >> 16) - mint_y);
                        const uint16_t offx = (uint16_t) ((int32_t) (int16_t) (to & 0xFFFF) - mint_x);
                        const uint32_t ab = sa + kb * MT * C::A_BLOCK, bb = sa + C::A_BYTES + kb * C::B_BLOCK;
                        const int kcol = kbeg + (kt + kb) * C::BK;
#pragma unroll
                        for (int mt = 0; mt < MT; mt++)
                            tc::tma_load_im2col_4d(ab + mt * C::A_BLOCK, am, ci0, w0[mt], h0[mt], bb0[mt], offx, offy,
                                                   &full[s]);
                        tc::tma_load_2d(bb, &wmap, kcol, tl.n0, &full[s]);
                        if (MODE == MODE_X3) {
                            tc::tma_load_im2col_4d(ab + C::A_TILE, &amaps.alo[tl.cls], ci0, w0[0], h0[0], bb0[0], offx,
                                                   offy, &full[s]);
                            tc::tma_load_2d(bb + C::B_TILE, &amaps.wlo, kcol, tl.n0, &full[s]);
                        }
                        ci0 += C::BK;
                        if (ci0 == p.Cin) {
                            ci0 = 0;
                            tap++;
                        }
                    }
                }
            }
        }
    } else if (!IM2C && warp < 4) {
        // ------------------------------------------------ producers: gather A, TMA B
        const int t = threadIdx.x;
        const int piece = t & 7;   // 16-byte piece of the 128-byte K row
        const int r0 = t >> 3;     // rows r0 + 16*i
        uint32_t it = 0;
        for (int tile = blockIdx.x; tile < p.ntiles_total && ok; tile += gridDim.x) {
            if (t == 0 && tile + (int) gridDim.x >= p.ntiles_total) tc::pdl_trigger();   // this CTA's last tile
            const Tile tl = decode_tile(cls_tab, p.ncls, p.ntiles, BN, tile);
            const ClsS &cl = cls_tab[tl.cls];
            const int32_t *taps = tap_tab + tl.cls * TC_MAXTAPS;
            const int M = p.B * cl.Hg * cl.Wg;
            int rb[8], ry[8], rx[8];
#pragma unroll
            for (int i = 0; i < 8; i++) {
                const int m = tl.m0 + r0 + 16 * i;
                if (m < M) {
                    uint32_t q, jw, j, b;
                    cl.dwg.divmod(m, q, jw);
                    cl.dhg.divmod(q, b, j);
                    rb[i] = b;
                    ry[i] = (int) j * cl.isy + cl.iby;
                    rx[i] = (int) jw * cl.isx + cl.ibx;
                } else {
                    rb[i] = -1;
                    ry[i] = rx[i] = 0;
                }
            }
            for (int kt = 0; kt < cl.ktiles; kt++, it++) {
                const int s = it % STAGES;
                const uint32_t ph = (it / STAGES) & 1;
                if (it >= (uint32_t) STAGES) ok = tc::mbar_wait(&empty[s], ph ^ 1, p.err, 1);
                if (!ok) break;
                const int k = kt * C::BK + piece * 8;
                uint32_t tap, ci;
                p.dcin.divmod(k, tap, ci);
                const bool kval = (int) tap < cl.ntaps;
                const int32_t to = kval ? taps[tap] : 0;
                const int oy = to >> 16, ox = (int32_t) (int16_t) (to & 0xFFFF);
                const uint32_t sA = tc::smem_u32(base + s * C::STAGE_BYTES);
#pragma unroll
                for (int i = 0; i < 8; i++) {
                    const int r = r0 + 16 * i;
                    const int iy = ry[i] + oy, ix = rx[i] + ox;
                    const bool v =
                        kval && rb[i] >= 0 && (unsigned) iy < (unsigned) p.Hin && (unsigned) ix < (unsigned) p.Win;
                    const bf16 *src = v ? p.in + ((((size_t) rb[i] * p.Hin + iy) * p.Win + ix) * p.Cin + ci) : p.in;
                    tc::cp_async_16(sA + r * 128 + ((piece ^ (r & 7)) << 4), src, v ? 16u : 0u);
                }
                tc::cp_async_commit();
                if (t == 0) {
                    tc::mbar_arrive_expect_tx(&full[s], C::B_BYTES);
                    tc::tma_load_2d(tc::smem_u32(base + s * C::STAGE_BYTES + C::A_BYTES), &wmap,
                                    cl.kbeg + kt * C::BK, tl.n0, &full[s]);
                }
                if (it >= (uint32_t) C::LAG) {
                    tc::cp_async_wait<C::LAG>();
                    tc::fence_proxy_async_smem();
                    tc::mbar_arrive(&full[(it - C::LAG) % STAGES]);
                }
            }
        }
        tc::cp_async_wait<0>();
        tc::fence_proxy_async_smem();
        if (ok)
            for (uint32_t j = (it > (uint32_t) C::LAG ? it - C::LAG : 0); j < it; j++) tc::mbar_arrive(&full[j % STAGES]);
    } else if (warp >= 4 && warp < 4 + EW) {
        // ------------------------------------------------ epilogue
        const int ew = (warp - 4) & 3;    // TMEM lane quarter (a warp reads lanes 32 * (warp % 4) ..)
        const int half = (warp - 4) >> 2; // EW = 8: which alternate chunks this warp takes
        const int row = ew * 32 + lane;   // tile row = TMEM lane
        const int et = threadIdx.x - 128; // 0 .. 32 * EW - 1
        uint8_t *const stg_warp = epi_smem + (warp - 4) * 4096;   // this warp's 32 x 128-byte staging
        uint32_t lt = 0;                  // local tile count
        int ebuf = 0;                     // staging buffer toggle
        for (int tile = blockIdx.x; tile < p.ntiles_total && ok; tile += gridDim.x, lt++) {
            const Tile tl = decode_tile(cls_tab, p.ncls, p.ntiles, BN, tile, MT);
            const ClsS &cl = cls_tab[tl.cls];
            const int M = p.B * cl.Hg * cl.Wg;
            const int buf = lt % C::ACC_BUFS;
            const float *scp = sc_tab, *shp = sh_tab;
            if (sc_all) {
                scp += tl.n0;
                shp += tl.n0;
            } else {
                // this tile's scale/shift (the previous tile's readers passed the barrier below)
                epi_bar<32 * EW>();
                for (int j = et; j < BN; j += 32 * EW) {
                    const int n = min(tl.n0 + j, p.Cout - 1);
                    sc_tab[j] = p.scale ? __ldg(p.scale + n) : 1.0f;
                    sh_tab[j] = p.shift ? __ldg(p.shift + n) : 0.0f;
                }
                epi_bar<32 * EW>();
            }
            ok = tc::mbar_wait(&acc_full[buf], (lt / C::ACC_BUFS) & 1, p.err, 3);
            if (!ok) break;
            tc::tc_fence_after();
            // items: (accumulator mt, chunk c0) in order; with eight warps the two warps of a
            // lane quarter take alternate items
            constexpr int NIT = MT * C::NCH, STEP = EW / 4;
#pragma unroll 1
            for (int item = half; item < NIT; item += STEP) {
                const int mt = item / C::NCH, c0 = (item % C::NCH) * C::CW;
                const int m0 = tl.m0 + mt * 128;   // this accumulator's first output row
                const int m = m0 + row;
                uint8_t *orow = nullptr;   // this row of the output (BF16, or FP32 for MODE_X3)
                if (!p.epi_tma && m < M) {
                    uint32_t q, jw, j, b;
                    cl.dwg.divmod(m, q, jw);
                    cl.dhg.divmod(q, b, j);
                    const int oy = cl.oy0 + cl.osy * (int) j, ox = cl.ox0 + cl.osx * (int) jw;
                    orow = (uint8_t *) p.out +
                           ((((size_t) b * p.Hout + oy) * p.Wout + ox) * p.Cout) * (C::OUTF32 ? 4 : 2);
                }
                uint32_t v0[32], v1[32];
                const uint32_t ta = tmem + ((uint32_t) (ew * 32) << 16) + (uint32_t) ((buf * MT + mt) * BN + c0);
                tc::tmem_ld_32x32b_x32(ta, v0);
                if (C::CW == 64) tc::tmem_ld_32x32b_x32(ta + 32, v1);
                tc::tmem_ld_wait();
                if (item + STEP >= NIT) {
                    // this warp's last read of the accumulator: its share of the TMEM buffer
                    // goes back to the MMA warp
                    tc::tc_fence_before();
                    tc::mbar_arrive(&acc_empty[buf]);
                }
                const int nb = tl.n0 + c0;
                if constexpr (STATS) if (m0 + ew * 32 < M) {
                    // column statistics of this chunk's 64 columns over the warp's 32 rows (group
                    // gbase + (m0 + 32 ew) / 32 of the class; the classes' groups are concatenated):
                    // the forward's batch-norm sums, or, for the masked input gradient, the sums of
                    // the masked output (the bias gradient of the layer that produced the mask)
                    if (p.mask && m < M && nb < p.Cout) {
                        size_t pix = (size_t) m;
                        if (!p.epi_tma) {
                            uint32_t q, jw, j, b;
                            cl.dwg.divmod(m, q, jw);
                            cl.dhg.divmod(q, b, j);
                            pix = ((size_t) b * p.Hout + cl.oy0 + cl.osy * (int) j) * p.Wout + cl.ox0 + cl.osx * (int) jw;
                        }
                        const __nv_bfloat16 *mrow = p.mask + pix * p.Cout + nb;
#pragma unroll
                        for (int q = 0; q < 8; q++) {
                            uint4 mv = make_uint4(0, 0, 0, 0);
                            if (nb + 8 * q + 8 <= p.Cout) mv = __ldg(reinterpret_cast<const uint4 *>(mrow) + q);
                            const uint32_t mw[4] = {mv.x, mv.y, mv.z, mv.w};
#pragma unroll
                            for (int e = 0; e < 4; e++) {
                                const int jj = 8 * q + 2 * e;
                                uint32_t &lo = jj < 32 ? v0[jj] : v1[jj - 32];
                                uint32_t &hi = jj + 1 < 32 ? v0[jj + 1] : v1[jj - 31];
                                if ((mw[e] & 0xFFFFu) - 1u >= 0x7F80u) lo = 0u;   // mask <= 0 (or NaN)
                                if ((mw[e] >> 16) - 1u >= 0x7F80u) hi = 0u;
                            }
                        }
                    }
                    float *part = p.stats + (size_t) (cl.gbase + (m0 >> 5) + ew) * 2 * p.Cout;
#pragma unroll
                    for (int h = 0; h < 2; h++) {
                        float sum, sq;
                        tc::stats_cols32(h ? v1 : v0, scp + c0 + 32 * h, shp + c0 + 32 * h, m < M, sum, sq);
                        const int col = nb + 32 * h + lane;
                        if (col < p.Cout) {
                            part[col] = sum;
                            part[p.Cout + col] = sq;
                        }
                    }
                }
                if (!C::OUTF32 && p.accum && m < M && nb < p.Cout) {
                    // accumulate (the reference's dx += ...): add the output's current 64 values in FP32
                    size_t pix = (size_t) m;
                    if (!p.epi_tma) {
                        uint32_t q, jw, j, b;
                        cl.dwg.divmod(m, q, jw);
                        cl.dhg.divmod(q, b, j);
                        pix = ((size_t) b * p.Hout + cl.oy0 + cl.osy * (int) j) * p.Wout + cl.ox0 + cl.osx * (int) jw;
                    }
                    const uint4 *orow4 = reinterpret_cast<const uint4 *>(p.out + pix * p.Cout + nb);
#pragma unroll
                    for (int q = 0; q < 8; q++) {
                        uint4 ov = make_uint4(0, 0, 0, 0);
                        if (nb + 8 * q + 8 <= p.Cout) ov = orow4[q];
                        const uint32_t ow[4] = {ov.x, ov.y, ov.z, ov.w};
#pragma unroll
                        for (int e = 0; e < 4; e++) {
                            const int jj = 8 * q + 2 * e;   // column of the low half
                            uint32_t &lo = jj < 32 ? v0[jj] : v1[jj - 32];
                            uint32_t &hi = jj + 1 < 32 ? v0[jj + 1] : v1[jj - 31];
                            lo = __float_as_uint(__uint_as_float(lo) + __uint_as_float(ow[e] << 16));
                            hi = __float_as_uint(__uint_as_float(hi) + __uint_as_float(ow[e] & 0xFFFF0000u));
                        }
                    }
                }
                uint32_t pk[32];   // one 128-byte output row chunk
                if (C::OUTF32) {
#pragma unroll
                    for (int jj = 0; jj < 32; jj++) {
                        float a = fmaf(__uint_as_float(v0[jj]), scp[c0 + jj], shp[c0 + jj]);
                        if (p.relu) a = fmaxf(a, 0.0f);
                        pk[jj] = __float_as_uint(a);
                    }
                } else if (p.relu) {
                    tc::epi_bf16_64<true>(v0, v1, scp + c0, shp + c0, pk);
                } else {
                    tc::epi_bf16_64<false>(v0, v1, scp + c0, shp + c0, pk);
                }
                if (!C::OUTF32 && p.mask && m < M && nb < p.Cout) {
                    // ReLU backward: keep the outputs where the mask (the activation the ReLU
                    // produced, laid out like the output) is positive
                    size_t pix = (size_t) m;
                    if (!p.epi_tma) {
                        uint32_t q, jw, j, b;
                        cl.dwg.divmod(m, q, jw);
                        cl.dhg.divmod(q, b, j);
                        pix = ((size_t) b * p.Hout + cl.oy0 + cl.osy * (int) j) * p.Wout + cl.ox0 + cl.osx * (int) jw;
                    }
                    const __nv_bfloat16 *mrow = p.mask + pix * p.Cout + nb;
#pragma unroll
                    for (int q = 0; q < 8; q++) {
                        uint4 mv = make_uint4(0, 0, 0, 0);
                        if (nb + 8 * q + 8 <= p.Cout) mv = __ldg(reinterpret_cast<const uint4 *>(mrow) + q);
                        const uint32_t mw[4] = {mv.x, mv.y, mv.z, mv.w};
#pragma unroll
                        for (int e = 0; e < 4; e++) {
                            const uint32_t lo = mw[e] & 0xFFFFu, hi = mw[e] >> 16;
                            // positive: sign clear, not zero, not NaN
                            const uint32_t klo = (lo - 1u) < 0x7F80u ? 0x0000FFFFu : 0u;
                            const uint32_t khi = (hi - 1u) < 0x7F80u ? 0xFFFF0000u : 0u;
                            pk[4 * q + e] &= klo | khi;
                        }
                    }
                }
                if (p.epi_tma) {
                    // each warp stages its 32 rows (4 KB) and stores them with its own TMA
                    // store: no barrier across the epilogue warps (out-of-range rows/columns
                    // are clipped by the store)
                    if (lane == 0) {
                        if (C::EPI_BUFS == 2) bulk_wait_read<1>();
                        else bulk_wait_read<0>();
                    }
                    __syncwarp();
                    uint8_t *stg = stg_warp + ebuf * C::EPI_BYTES;
#pragma unroll
                    for (int q = 0; q < 8; q++) {
                        uint4 u = make_uint4(pk[4 * q], pk[4 * q + 1], pk[4 * q + 2], pk[4 * q + 3]);
                        *reinterpret_cast<uint4 *>(stg + lane * 128 + ((q ^ (lane & 7)) << 4)) = u;
                    }
                    tc::fence_proxy_async_smem();
                    __syncwarp();
                    if (lane == 0 && nb < p.Cout && m0 + ew * 32 < M) {
                        tma_store_2d(&omap, tc::smem_u32(stg), nb, m0 + ew * 32);
                        bulk_commit();
                    }
                    if (C::EPI_BUFS == 2) ebuf ^= 1;
                } else if (!C::OUTF32 && nb + C::CW <= p.Cout && __any_sync(0xFFFFFFFFu, orow != nullptr)) {
                    // rows scattered over the output (stride-phase classes): staged through this warp's
                    // buffer, then each store instruction writes four whole 128-byte rows (eight lanes
                    // per row) instead of 16 bytes of 32 rows
                    uint8_t *stg = stg_warp + ebuf * C::EPI_BYTES;
                    if (lane == 0 && C::EPI_BUFS == 2) bulk_wait_read<1>();
                    else if (lane == 0) bulk_wait_read<0>();
                    __syncwarp();
#pragma unroll
                    for (int q = 0; q < 8; q++)
                        *reinterpret_cast<uint4 *>(stg + lane * 128 + ((q ^ (lane & 7)) << 4)) =
                            make_uint4(pk[4 * q], pk[4 * q + 1], pk[4 * q + 2], pk[4 * q + 3]);
                    __syncwarp();
                    const unsigned long long my = (unsigned long long) (orow ? orow + (size_t) nb * 2 : nullptr);
#pragma unroll
                    for (int q = 0; q < 8; q++) {
                        const int r = q * 4 + (lane >> 3), ch = lane & 7;
                        const unsigned long long dst = __shfl_sync(0xFFFFFFFFu, my, r);
                        const uint4 u = *reinterpret_cast<const uint4 *>(stg + r * 128 + ((ch ^ (r & 7)) << 4));
                        if (dst) *reinterpret_cast<uint4 *>((uint8_t *) dst + ch * 16) = u;
                    }
                    __syncwarp();
                    if (C::EPI_BUFS == 2) ebuf ^= 1;
                } else if (orow && nb < p.Cout) {
                    if (nb + C::CW <= p.Cout) {
                        uint4 *dst = reinterpret_cast<uint4 *>(orow + (size_t) nb * (C::OUTF32 ? 4 : 2));
#pragma unroll
                        for (int q = 0; q < 8; q++) dst[q] = make_uint4(pk[4 * q], pk[4 * q + 1], pk[4 * q + 2], pk[4 * q + 3]);
                    } else if (C::OUTF32) {
                        float *o = reinterpret_cast<float *>(orow);
#pragma unroll
                        for (int jj = 0; jj < 32; jj++)
                            if (nb + jj < p.Cout) o[nb + jj] = __uint_as_float(pk[jj]);
                    } else {
                        bf16 *o = reinterpret_cast<bf16 *>(orow);
#pragma unroll
                        for (int jj = 0; jj < 32; jj++) {
                            __nv_bfloat162 h = *reinterpret_cast<const __nv_bfloat162 *>(&pk[jj]);
                            if (nb + 2 * jj < p.Cout) o[nb + 2 * jj] = h.x;
                            if (nb + 2 * jj + 1 < p.Cout) o[nb + 2 * jj + 1] = h.y;
                        }
                    }
                }
            }
        }
        if (lane == 0) bulk_wait_all();
    } else {
        // ------------------------------------------------ MMA issuer
        if (lane == 0) {
            // issuer `me`: its M tile (MT = 2) or N half (MT = 1) when SPLIT, else everything
            const int me = (SPLIT && warp == C::ISS2_WARP) ? 1 : 0;
            constexpr int NI = (SPLIT && MT == 1) ? BN / 2 : BN;   // N of one MMA instruction
            constexpr bool F8 = MODE == MODE_FP8 || MODE == MODE_FP8W;
            constexpr uint32_t idesc = F8 ? tc::idesc_e4m3(128, BN) : tc::idesc_bf16(128, NI, 0, 0);
            const uint32_t n_off = (SPLIT && MT == 1) ? (uint32_t) (me * NI) : 0u;   // accumulator column
            const uint64_t b_off = (SPLIT && MT == 1) ? (uint64_t) (me * NI * C::ROWB) >> 4 : 0u;   // B rows
            uint32_t it = 0, lt = 0;
            for (int tile = blockIdx.x; tile < p.ntiles_total && ok; tile += gridDim.x, lt++) {
                const Tile tl = decode_tile(cls_tab, p.ncls, p.ntiles, BN, tile, MT);
                const int KT = cls_tab[tl.cls].ktiles;
                const int buf = lt % C::ACC_BUFS;
                if (lt >= (uint32_t) C::ACC_BUFS) {
                    ok = tc::mbar_wait(&acc_empty[buf], ((lt / C::ACC_BUFS) - 1) & 1, p.err, 4);
                    if (!ok) break;
                    tc::tc_fence_after();
                }
                const uint32_t dt = tmem + (uint32_t) (buf * MT * BN);
                for (int kt = 0; kt < KT; kt += KB, it++) {
                    const int s = it % STAGES;
                    const uint32_t ph = (it / STAGES) & 1;
                    if (!tc::mbar_wait(&full[s], ph, p.err, 2)) {
                        ok = false;
                        break;
                    }
                    tc::tc_fence_after();
                    const int nkb = min(KB, KT - kt);
                    const uint32_t a0 = tc::smem_u32(base + s * C::STAGE_BYTES);
                    // descriptors built once per stage; an offset of d bytes adds d / 16 to the
                    // start field (the stage stays below 256 KB, so the field never carries)
                    const uint64_t ad0 = op_desc(a0, C::SBO, C::LAYOUT);
                    const uint64_t bd0 = ad0 + (C::A_BYTES >> 4);
#pragma unroll
                    for (int kb = 0; kb < KB; kb++) {
                        if (kb >= nkb) break;
                        // each MMA consumes 32 bytes of every K row: 16 BF16 or 32 E4M3 elements
#pragma unroll
                        for (int k = 0; k < C::ROWB / 32; k++) {
                            const uint32_t acc = (kt | kb | k) != 0;
                            const uint64_t bd = bd0 + ((kb * C::B_BLOCK + k * 32) >> 4) + b_off;
#pragma unroll
                          for (int mt = 0; mt < MT; mt++) {
                            if (SPLIT && MT == 2 && mt != me) continue;
                            const uint64_t ad = ad0 + (((kb * MT + mt) * C::A_BLOCK + k * 32) >> 4);
                            const uint32_t dtm = dt + (uint32_t) (mt * BN) + n_off;
                            if (F8) {
                                tc::mma_f8(dtm, ad, bd, idesc, acc);
                            } else {
                                tc::mma_f16(dtm, ad, bd, idesc, acc);
                                if (MODE == MODE_X3) {
                                    const uint64_t adl = ad + (C::A_TILE >> 4);
                                    const uint64_t bdl = bd + (C::B_TILE >> 4);
                                    tc::mma_f16(dtm, ad, bdl, idesc, 1);   // hi * lo
                                    tc::mma_f16(dtm, adl, bd, idesc, 1);   // lo * hi
                                }
                            }
                          }
                        }
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
    if (warp == C::MMA_WARP) tc::tmem_dealloc(tmem, C::TMEM_COLS);
}

template <int BN, int STAGES, int KB, bool IM2C, int MODE, int MT = 1, int EW = 4, bool STATS = false>
cudaError_t launch_bn(const TcConvParams &p, const CUtensorMap &wmap, const CUtensorMap &omap, const TcMaps &amaps,
                      int grid, cudaStream_t st) {
    static_assert(!STATS || (MODE == MODE_BF16 && MT == 1 && EW == 4), "statistics: BF16, one M tile, four warps");
    using C = TcCfg<BN, STAGES, KB, MODE, MT, EW>;
    auto kern = tc_conv_kernel<BN, STAGES, KB, IM2C, MODE, MT, EW, STATS>;
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) C::SMEM);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    return cg_launch_pdl(kern, dim3(grid), dim3(C::THREADS), C::SMEM, st, p, wmap, omap, amaps);
}

}  // namespace

// Stage shapes (~192 KB of ring each).  BF16 im2col: BN=64 4 stages of 2 K blocks,
// BN=128 3 x 2, BN=256 3 x 1 with two output staging buffers (its tiles are often
// single-block 1x1 layers bound by the output stores).  FP8 blocks are half the bytes,
// 3xBF16 blocks twice.
int tc_conv_stages(int bn, int im2col, int mt, int ew, int kb1) {
    if (!im2col) return bn == 64 ? 8 : (bn == 128 ? 6 : 4);
    if (ew == 8) return mt == 2 ? 3 : (bn == 128 ? 4 : 3);
    if (mt == 2) return bn == 256 ? 3 : 4;
    if (kb1 && bn != 256) return bn == 64 ? 8 : 6;
    return bn == 64 ? 4 : 3;
}

cudaError_t tc_conv_launch(const TcConvParams &p, const CUtensorMap &wmap, const CUtensorMap &omap,
                           const TcMaps &amaps, int grid, cudaStream_t st) {
    if (p.mode == MODE_FP8) {
        switch (p.bn) {
            case 64: return launch_bn<64, 4, 4, true, MODE_FP8>(p, wmap, omap, amaps, grid, st);
            case 128: return launch_bn<128, 3, 4, true, MODE_FP8>(p, wmap, omap, amaps, grid, st);
            case 256: return launch_bn<256, 3, 2, true, MODE_FP8>(p, wmap, omap, amaps, grid, st);
            default: return cudaErrorInvalidValue;
        }
    }
    if (p.mode == MODE_FP8W) {   // 128-channel blocks: 16 KB per 128-row block, as BF16
        switch (p.bn) {
            case 64: return launch_bn<64, 4, 2, true, MODE_FP8W>(p, wmap, omap, amaps, grid, st);
            case 128: return launch_bn<128, 3, 2, true, MODE_FP8W>(p, wmap, omap, amaps, grid, st);
            case 256: return launch_bn<256, 3, 1, true, MODE_FP8W>(p, wmap, omap, amaps, grid, st);
            default: return cudaErrorInvalidValue;
        }
    }
    if (p.mode == MODE_X3) {
        switch (p.bn) {
            case 64: return launch_bn<64, 4, 1, true, MODE_X3>(p, wmap, omap, amaps, grid, st);
            case 128: return launch_bn<128, 3, 1, true, MODE_X3>(p, wmap, omap, amaps, grid, st);
            case 256: return launch_bn<256, 2, 1, true, MODE_X3>(p, wmap, omap, amaps, grid, st);
            default: return cudaErrorInvalidValue;
        }
    }
    if (p.stats) {
        // forward with batch statistics (tc_conv_kernel's STATS form): one M tile, four epilogue warps
        if (p.mode != MODE_BF16 || p.mt != 1 || p.ew != 4) return cudaErrorInvalidValue;
        if (p.im2col) {
            switch (p.bn) {
                case 64: return launch_bn<64, 4, 2, true, MODE_BF16, 1, 4, true>(p, wmap, omap, amaps, grid, st);
                case 128: return launch_bn<128, 3, 2, true, MODE_BF16, 1, 4, true>(p, wmap, omap, amaps, grid, st);
                case 256: return launch_bn<256, 3, 1, true, MODE_BF16, 1, 4, true>(p, wmap, omap, amaps, grid, st);
                default: return cudaErrorInvalidValue;
            }
        }
        switch (p.bn) {
            case 64: return launch_bn<64, 8, 1, false, MODE_BF16, 1, 4, true>(p, wmap, omap, amaps, grid, st);
            case 128: return launch_bn<128, 6, 1, false, MODE_BF16, 1, 4, true>(p, wmap, omap, amaps, grid, st);
            case 256: return launch_bn<256, 4, 1, false, MODE_BF16, 1, 4, true>(p, wmap, omap, amaps, grid, st);
            default: return cudaErrorInvalidValue;
        }
    }
    if (p.im2col && p.ew == 8) {
        // eight epilogue warps (short-K tiles): one K block per stage, two staging buffers
        if (p.mt == 2) {
            switch (p.bn) {
                case 64: return launch_bn<64, 3, 1, true, MODE_BF16, 2, 8>(p, wmap, omap, amaps, grid, st);
                case 128: return launch_bn<128, 3, 1, true, MODE_BF16, 2, 8>(p, wmap, omap, amaps, grid, st);
                default: return cudaErrorInvalidValue;
            }
        }
        switch (p.bn) {
            case 128: return launch_bn<128, 4, 1, true, MODE_BF16, 1, 8>(p, wmap, omap, amaps, grid, st);
            case 256: return launch_bn<256, 3, 1, true, MODE_BF16, 1, 8>(p, wmap, omap, amaps, grid, st);
            default: return cudaErrorInvalidValue;
        }
    }
    if (p.im2col && p.mt == 2) {
        // two M tiles per weight tile: 40 / 48 / 64 KB per K block
        switch (p.bn) {
            case 64: return launch_bn<64, 4, 1, true, MODE_BF16, 2>(p, wmap, omap, amaps, grid, st);
            case 128: return launch_bn<128, 4, 1, true, MODE_BF16, 2>(p, wmap, omap, amaps, grid, st);
            case 256: return launch_bn<256, 3, 1, true, MODE_BF16, 2>(p, wmap, omap, amaps, grid, st);
            default: return cudaErrorInvalidValue;
        }
    }
    if (p.mt != 1) return cudaErrorInvalidValue;
    if (p.im2col && p.kb1) {
        switch (p.bn) {
            case 64: return launch_bn<64, 8, 1, true, MODE_BF16>(p, wmap, omap, amaps, grid, st);
            case 128: return launch_bn<128, 6, 1, true, MODE_BF16>(p, wmap, omap, amaps, grid, st);
            default: break;   // 256-wide tiles keep their three one-block stages
        }
    }
    if (p.im2col) {
        switch (p.bn) {
            case 64: return launch_bn<64, 4, 2, true, MODE_BF16>(p, wmap, omap, amaps, grid, st);
            case 128: return launch_bn<128, 3, 2, true, MODE_BF16>(p, wmap, omap, amaps, grid, st);
            case 256: return launch_bn<256, 3, 1, true, MODE_BF16>(p, wmap, omap, amaps, grid, st);
            default: return cudaErrorInvalidValue;
        }
    }
    switch (p.bn) {
        case 64: return launch_bn<64, 8, 1, false, MODE_BF16>(p, wmap, omap, amaps, grid, st);
        case 128: return launch_bn<128, 6, 1, false, MODE_BF16>(p, wmap, omap, amaps, grid, st);
        case 256: return launch_bn<256, 4, 1, false, MODE_BF16>(p, wmap, omap, amaps, grid, st);
        default: return cudaErrorInvalidValue;
    }
}
