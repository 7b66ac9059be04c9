// BF16 forward / input gradient of stride-1 convolutions with 64-channel input blocks and
// several taps (the 3x3 layers with 64 input channels: ResNet-50 stage 1, VGG's first
// blocks): sconvGemmNHWC('N') (src/convGemm.c:65-70) and sconvGemmNHWC_back
// (src/convGemm.c:82-97) for those shapes.
//
// The general kernel loads one im2col TMA tile per tap, so each input pixel crosses L2 ->
// shared memory kh*kw times, which bounds these N = 64 layers.  Here a tile is R output rows
// x Wc output columns of one image, laid out as tile rows r = i * Wp + j (Wp = Wc + the
// horizontal tap span; rows with j >= Wc are computed and dropped), and
//   * one TMA load per 64-channel block brings the input slab of the tile -- (R + vertical
//     tap span) rows x Wp columns x 64 channels, zero outside the image -- into shared memory
//     with the 128-byte swizzle: one 128-byte row per pixel;
//   * tap t, whose input pixel sits (dy_t, dx_t) from the tile's first, is then the
//     128 consecutive slab rows starting at dy_t * Wp + dx_t: a K-major SW128 operand at a
//     start that is a whole number of 128-byte rows (the swizzle is address-based, so the
//     descriptor's matrix base offset stays 0);
//   * the packed weights of the CTA's N tile (all taps x channel blocks, SW128) are
//     resident;
//   * the MMAs run in the general kernel's K order (tap-major, 16 K per MMA), so results
//     are bit-identical to it;
//   * the epilogue applies scale / shift / ReLU and stores each valid row directly.
// Each input pixel crosses L2 -> shared memory about (R + span) / R times instead of kh*kw.
#include <algorithm>
#include <cstring>

#include <cuda_bf16.h>

#include "cg_common.cuh"
#include "tc_epi.cuh"
#include "tc_host.h"
#include "tc_ptx.cuh"

namespace {

constexpr int SLAB_BN = 64;                       // output channels per tile (one 64-column chunk)
constexpr int SLAB_MAXTAPS = 16;
constexpr int SLAB_MAXBUF = 4;
constexpr int SLAB_ACC = 4;                       // accumulator buffers (one per MMA issuer at most)
constexpr uint32_t SLAB_W_MAX = 96 * 1024;        // resident weights
constexpr size_t SLAB_SMEM = 232448;              // the per-block opt-in maximum
constexpr uint32_t SLAB_STAGE = 128 * 128;        // one output staging buffer: a tile's valid rows x 128 B

struct SlabParams {
    __nv_bfloat16 *out;          // NHWC [B][Hout][Wout][Cout]
    const float *scale, *shift;
    int relu, B, Hout, Wout, Cout, cblocks, ntaps, ntn;
    int R, Wc, Wp, Hs;           // tile rows / columns, slab width / height
    int nrg, nwc, mtiles;        // row groups per image, column chunks per row group, M tiles
    int ty0, tx0;                // input offset of slab row 0 / column 0 from the tile's first output pixel
    int kbeg;                    // first K column of the class in the packed weights
    int nbuf;                    // slab buffers
    int nstage;                  // output staging buffers (1 or 2)
    int niss;                    // MMA-issuing threads (2..4): issuer k takes the CTA's tiles k, k + niss, ...
    uint32_t buf_bytes;          // one slab buffer (1024-aligned)
    uint32_t slab_tx;            // bytes one slab load delivers
    uint32_t w_bytes;            // resident weights of one N tile
    int *err;
    uint32_t aoff[SLAB_MAXTAPS];  // byte offset of tap t's first row in a slab buffer
};

__device__ __forceinline__ void tma_store_4d(const CUtensorMap *map, uint32_t src, int c0, int c1, int c2, int c3) {
    asm volatile("cp.async.bulk.tensor.4d.global.shared::cta.bulk_group [%0, {%2, %3, %4, %5}], [%1];" ::"l"(
                     (uint64_t) map),
                 "r"(src), "r"(c0), "r"(c1), "r"(c2), "r"(c3)
                 : "memory");
    asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}

__global__ void __launch_bounds__(288, 1)
    tc_slab_kernel(const __grid_constant__ SlabParams p, const __grid_constant__ CUtensorMap xmap,
                   const __grid_constant__ CUtensorMap wmap, const __grid_constant__ CUtensorMap omap) {
    tc::pdl_wait();   // pdl_trigger: the producer's last tile
    extern __shared__ uint8_t smem_raw[];
    uint8_t *base = (uint8_t *) (((uintptr_t) smem_raw + 1023) & ~(uintptr_t) 1023);
    uint8_t *wres = base;                                   // tap t, block cb at (t * cblocks + cb) * 8 KB
    uint8_t *slab = base + p.w_bytes;                       // p.nbuf buffers of p.buf_bytes
    uint8_t *stage = slab + (size_t) p.nbuf * p.buf_bytes; // p.nstage output staging buffers
    uint64_t *bars = (uint64_t *) (stage + (size_t) p.nstage * SLAB_STAGE);
    uint64_t *slab_full = bars, *slab_free = bars + SLAB_MAXBUF;
    uint64_t *acc_full = bars + 2 * SLAB_MAXBUF, *acc_empty = acc_full + SLAB_ACC, *wfull = acc_empty + SLAB_ACC;
    uint32_t *tmem_holder = (uint32_t *) (wfull + 1);
    float *sc_tab = (float *) (bars + 32);                  // 256 bytes of barriers above
    float *sh_tab = sc_tab + SLAB_BN;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int n0 = (blockIdx.x % p.ntn) * SLAB_BN;          // this CTA's N tile
    const int m_first = blockIdx.x / p.ntn, m_step = gridDim.x / p.ntn;
    if (threadIdx.x == 0) {
        for (int s = 0; s < p.nbuf; s++) {
            tc::mbar_init(&slab_full[s], 1);
            tc::mbar_init(&slab_free[s], 1);   // the MMA commit of the tile that read the buffer
        }
        for (int b = 0; b < SLAB_ACC; b++) {
            tc::mbar_init(&acc_full[b], 1);
            tc::mbar_init(&acc_empty[b], 128);
        }
        tc::mbar_init(wfull, 1);
        tc::fence_mbar_init();
        tc::prefetch_tmap(&xmap);
        tc::prefetch_tmap(&wmap);
        tc::prefetch_tmap(&omap);
        // the N tile's packed weights, every tap and channel block: K column kbeg + (t*cblocks + cb) * 64
        tc::mbar_arrive_expect_tx(wfull, p.w_bytes);
        for (int j = 0; j < p.ntaps * p.cblocks; j++)
            tc::tma_load_2d(tc::smem_u32(wres + (size_t) j * 8192), &wmap, p.kbeg + j * 64, n0, wfull);
    } else if (warp >= 4 && warp < 8) {
        for (int n = threadIdx.x - 128; n < SLAB_BN; n += 128) {
            const int nn = min(n0 + n, p.Cout - 1);
            sc_tab[n] = p.scale ? __ldg(p.scale + nn) : 1.0f;
            sh_tab[n] = p.shift ? __ldg(p.shift + nn) : 0.0f;
        }
    } else if (warp == 8) {
        tc::tmem_alloc(tmem_holder, SLAB_ACC * SLAB_BN);
        tc::tmem_relinquish();
    }
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tmem = *tmem_holder;
    bool ok = true;

    if (warp == 0) {
        // ------------------------------------------------ producer: one slab load per (tile, channel block)
        if (lane == 0) {
            uint32_t it = 0;
            for (int m = m_first; m < p.mtiles && ok; m += m_step) {
                if (m + m_step >= p.mtiles) tc::pdl_trigger();   // this CTA's last tile
                const int wc = m % p.nwc, q = m / p.nwc, rg = q % p.nrg, b = q / p.nrg;
                const int oy0 = rg * p.R, ox0 = wc * p.Wc;
                for (int cb = 0; cb < p.cblocks; cb++, it++) {
                    const int s = it % p.nbuf;
                    const uint32_t ph = (it / p.nbuf) & 1;
                    if (it >= (uint32_t) p.nbuf && !(ok = tc::mbar_wait(&slab_free[s], ph ^ 1, p.err, 51))) break;
                    tc::mbar_arrive_expect_tx(&slab_full[s], p.slab_tx);
                    tc::tma_load_4d(tc::smem_u32(slab + (size_t) s * p.buf_bytes), &xmap, cb * 64, ox0 + p.tx0,
                                   oy0 + p.ty0, b, &slab_full[s]);
                }
            }
        }
        __syncwarp();
    } else if (warp >= 4 && warp < 8) {
        // ------------------------------------------------ epilogue: this thread's tile row, compacted
        // into the staging box [R][Wc][64 channels] (128-byte swizzle) of one TMA store per tile
        const int ew = warp - 4, r = ew * 32 + lane, et = threadIdx.x - 128;
        const int i = r / p.Wp, jj = r % p.Wp;
        const bool inbox = i < p.R && jj < p.Wc;
        const int drow = i * p.Wc + jj;
        uint32_t lt = 0;
        for (int m = m_first; m < p.mtiles && ok; m += m_step, lt++) {
            const int wc = m % p.nwc, q = m / p.nwc, rg = q % p.nrg, b = q / p.nrg;
            const int buf = lt % SLAB_ACC;
            if (!(ok = tc::mbar_wait(&acc_full[buf], (lt / SLAB_ACC) & 1, p.err, 53))) break;
            tc::tc_fence_after();
            uint32_t v0[32], v1[32];
            const uint32_t ta = tmem + ((uint32_t) (ew * 32) << 16) + (uint32_t) (buf * SLAB_BN);
            tc::tmem_ld_32x32b_x32(ta, v0);
            tc::tmem_ld_32x32b_x32(ta + 32, v1);
            tc::tmem_ld_wait();
            tc::tc_fence_before();
            tc::mbar_arrive(&acc_empty[buf]);
            uint32_t pk[32];
            if (p.relu)
                tc::epi_bf16_64<true>(v0, v1, sc_tab, sh_tab, pk);
            else
                tc::epi_bf16_64<false>(v0, v1, sc_tab, sh_tab, pk);
            uint8_t *stg = stage + (size_t) (p.nstage == 2 ? (lt & 1) : 0) * SLAB_STAGE;
            // the store that last read this staging buffer is done reading it
            if (et == 0) {
                if (p.nstage == 2)
                    asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory");
                else
                    asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
            }
            asm volatile("bar.sync 1, 128;" ::: "memory");
            if (inbox) {
#pragma unroll
                for (int c = 0; c < 8; c++)
                    *reinterpret_cast<uint4 *>(stg + drow * 128 + ((c ^ (drow & 7)) << 4)) =
                        make_uint4(pk[4 * c], pk[4 * c + 1], pk[4 * c + 2], pk[4 * c + 3]);
            }
            tc::fence_proxy_async_smem();
            asm volatile("bar.sync 1, 128;" ::: "memory");
            // rows and columns past the output (partial row groups, column chunks, N tiles) are clipped
            if (et == 0) tma_store_4d(&omap, tc::smem_u32(stg), n0, wc * p.Wc, rg * p.R, b);
        }
        if (et == 0) asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
    } else if (warp == 8 || (warp >= 1 && warp < p.niss)) {
        // ------------------------------------------------ MMA issuers: lane 0 of warp 8 (issuer 0) and
        // of warps 1 .. niss-1; issuer k takes this CTA's tiles k, k + niss, ..., each into its own
        // accumulator buffer (one thread's instruction stream cannot issue N = 64 MMAs as fast as
        // the tensor core runs them)
        if (lane == 0) {
            const uint32_t me = warp == 8 ? 0u : (uint32_t) warp;
            constexpr uint32_t idesc = tc::idesc_bf16(128, SLAB_BN, 0, 0);
            const uint32_t wbase = tc::smem_u32(wres);
            uint32_t ao[SLAB_MAXTAPS];   // tap row offsets in registers (no table loads between the MMAs)
#pragma unroll
            for (int t = 0; t < SLAB_MAXTAPS; t++) ao[t] = p.aoff[t];
            if (!(ok = tc::mbar_wait(wfull, 0, p.err, 50))) ok = false;
            tc::tc_fence_after();
            for (uint32_t lt = me, m = m_first + me * m_step; (int) m < p.mtiles && ok;
                 lt += p.niss, m += p.niss * m_step) {
                const uint32_t it = lt * p.cblocks;   // the producer's slab index of this tile's first block
                const int buf = lt % SLAB_ACC;
                if (lt >= (uint32_t) SLAB_ACC) {
                    if (!(ok = tc::mbar_wait(&acc_empty[buf], ((lt / SLAB_ACC) + 1) & 1, p.err, 54))) break;
                    tc::tc_fence_after();
                }
                const uint32_t dt = tmem + (uint32_t) (buf * SLAB_BN);
                // every channel block's slab of the tile, then the MMAs in the general kernel's K
                // order (tap-major, then channel block), so that the sums round identically
                int sbuf[SLAB_MAXBUF];
                for (int cb = 0; cb < p.cblocks && ok; cb++) {
                    sbuf[cb] = (it + cb) % p.nbuf;
                    ok = tc::mbar_wait(&slab_full[sbuf[cb]], ((it + cb) / p.nbuf) & 1, p.err, 52);
                }
                if (!ok) break;
                tc::tc_fence_after();
                // descriptors built once per (tap, block); a 32-byte K step adds 2 to the start field
                if (p.cblocks == 1) {
                    const uint64_t a0 = tc::sw128_desc(tc::smem_u32(slab + (size_t) sbuf[0] * p.buf_bytes), 16, 1024);
                    const uint64_t b0 = tc::sw128_desc(wbase, 16, 1024);
#pragma unroll
                    for (int t = 0; t < SLAB_MAXTAPS; t++) {
                        if (t >= p.ntaps) break;
                        const uint64_t ad = a0 + (ao[t] >> 4), bd = b0 + (uint64_t) t * (8192 >> 4);
#pragma unroll
                        for (int k = 0; k < 4; k++) tc::mma_f16(dt, ad + 2 * k, bd + 2 * k, idesc, (t | k) != 0);
                    }
                } else {
                    uint64_t ab[SLAB_MAXBUF];
                    for (int cb = 0; cb < p.cblocks; cb++)
                        ab[cb] = tc::sw128_desc(tc::smem_u32(slab + (size_t) sbuf[cb] * p.buf_bytes), 16, 1024);
                    const uint64_t b0 = tc::sw128_desc(wbase, 16, 1024);
#pragma unroll
                    for (int t = 0; t < SLAB_MAXTAPS; t++) {
                        if (t >= p.ntaps) break;
                        for (int cb = 0; cb < p.cblocks; cb++) {
                            const uint64_t ad = ab[cb] + (ao[t] >> 4);
                            const uint64_t bd = b0 + (uint64_t) (t * p.cblocks + cb) * (8192 >> 4);
#pragma unroll
                            for (int k = 0; k < 4; k++)
                                tc::mma_f16(dt, ad + 2 * k, bd + 2 * k, idesc, (cb | t | k) != 0);
                        }
                    }
                }
                for (int cb = 0; cb < p.cblocks; cb++) tc::mma_commit(&slab_free[sbuf[cb]]);
                tc::mma_commit(&acc_full[buf]);
            }
        }
        __syncwarp();
    }
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    if (warp == 8) tc::tmem_dealloc(tmem, SLAB_ACC * SLAB_BN);
}

}  // namespace

namespace {

// Tile and slab geometry of a plan; false when the slab kernel does not apply.
bool slab_geom(const TcPlan &pl, SlabParams &p) {
    if (pl.ncls != 1 || pl.Cin % 64 || pl.Cout % 8) return false;
    const TcClass &c = pl.cls[0];
    if (c.osy != 1 || c.osx != 1 || c.oy0 || c.ox0 || c.isy != 1 || c.isx != 1 || c.Hg != pl.Hout || c.Wg != pl.Wout)
        return false;
    if (c.ntaps < 2 || c.ntaps > SLAB_MAXTAPS) return false;
    memset(&p, 0, sizeof(p));
    p.cblocks = pl.Cin / 64;
    p.ntaps = c.ntaps;
    p.w_bytes = (uint32_t) p.ntaps * p.cblocks * 8192;
    if (p.w_bytes > SLAB_W_MAX) return false;
    int dymin = 1 << 20, dymax = -(1 << 20), dxmin = 1 << 20, dxmax = -(1 << 20);
    for (int t = 0; t < c.ntaps; t++) {
        const int dy = c.iby + c.toy[t], dx = c.ibx + c.tox[t];
        dymin = std::min(dymin, dy);
        dymax = std::max(dymax, dy);
        dxmin = std::min(dxmin, dx);
        dxmax = std::max(dxmax, dx);
    }
    const int sy = dymax - dymin, sx = dxmax - dxmin;
    // tile shape: R output rows x Wc columns with R*Wc + (R-1)*sx <= 128 tile rows, at least 3/4 of
    // them valid; the fewest tiles per image (the MMAs of a tile cost the same however many of its
    // rows are valid), then the fewest slab rows loaded per tile
    long long best_tiles = 1LL << 62, best_rows = 1LL << 62;
    p.R = 0;
    for (int R = 1; R <= 16 && R <= pl.Hout; R++) {
        const int Wc = std::min(pl.Wout, (128 - (R - 1) * sx) / R);
        if (Wc < 1 || R * Wc < 96 || Wc + sx > 256 || R + sy > 256) continue;
        const long long tiles = (long long) ((pl.Hout + R - 1) / R) * ((pl.Wout + Wc - 1) / Wc);
        const long long rows = (long long) (R + sy) * (Wc + sx);
        if (tiles < best_tiles || (tiles == best_tiles && rows < best_rows)) {
            best_tiles = tiles;
            best_rows = rows;
            p.R = R;
            p.Wc = Wc;
        }
    }
    if (p.R == 0) return false;
    p.Wp = p.Wc + sx;
    p.Hs = p.R + sy;
    p.ty0 = dymin;
    p.tx0 = dxmin;
    uint32_t rows = (uint32_t) p.Hs * p.Wp;
    for (int t = 0; t < c.ntaps; t++) {
        const uint32_t r0 = (uint32_t) ((c.iby + c.toy[t] - dymin) * p.Wp + (c.ibx + c.tox[t] - dxmin));
        p.aoff[t] = r0 * 128;
        rows = std::max(rows, r0 + 128);   // the operand reads 128 rows (the rows past the tile's are dropped)
    }
    p.buf_bytes = (rows * 128 + 1023) / 1024 * 1024;
    // output staging: two 16 KB buffers when they fit beside three slab buffers, else one
    const size_t fixed = 1024 + p.w_bytes + 256 + 2 * SLAB_BN * 4;
    p.nstage = fixed + 3 * (size_t) p.buf_bytes + 2 * SLAB_STAGE <= SLAB_SMEM ? 2 : 1;
    const size_t avail = SLAB_SMEM - fixed - (size_t) p.nstage * SLAB_STAGE;
    p.nbuf = (int) std::min<size_t>(SLAB_MAXBUF, avail / p.buf_bytes);
    // all channel blocks of a tile are resident together (the MMAs run tap-major), for the tiles
    // the MMA issuers work on at the same time
    p.niss = std::min(SLAB_ACC, p.nbuf / p.cblocks);
    if (p.niss < 2) return false;
    p.slab_tx = (uint32_t) p.Hs * p.Wp * 128;
    p.kbeg = c.kbeg;
    return true;
}

}  // namespace

bool tc_slab_applicable(const TcPlan &pl) {
    SlabParams p;
    return slab_geom(pl, p);
}

convgemm_status_t tc_slab_run(const TcPlan &pl, const cg_shape &s, const void *in, const void *wpacked, void *out,
                              const float *scale, const float *shift, int relu, cudaStream_t st) {
    SlabParams p;
    if (!slab_geom(pl, p)) return cg_set_error(CONVGEMM_ERROR_NOT_SUPPORTED, "slab convolution: shape");
    if (((uintptr_t) out & 15) || ((uintptr_t) in & 15) || ((uintptr_t) wpacked & 15))
        return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "slab convolution: tensors must be 16-byte aligned");
    p.out = (__nv_bfloat16 *) out;
    p.scale = scale;
    p.shift = shift;
    p.relu = relu;
    p.B = s.b;
    p.Hout = pl.Hout;
    p.Wout = pl.Wout;
    p.Cout = pl.Cout;
    p.ntn = (pl.Cout + SLAB_BN - 1) / SLAB_BN;
    p.nrg = (pl.Hout + p.R - 1) / p.R;
    p.nwc = (pl.Wout + p.Wc - 1) / p.Wc;
    const long long mt = (long long) s.b * p.nrg * p.nwc;
    if (mt >= (1LL << 31)) return cg_set_error(CONVGEMM_ERROR_NOT_SUPPORTED, "slab convolution: too many tiles");
    p.mtiles = (int) mt;
    p.err = cg_device_error_word();
    if (!p.err) return cg_set_error(CONVGEMM_ERROR_CUDA, "device error word unavailable");
    // gathered tensor [B][Hin][Win][Cin]: box {64 channels, Wp, Hs, 1}, 128-byte swizzle
    CUtensorMap xmap, wmap;
    {
        const unsigned long long dims[4] = {(unsigned long long) pl.Cin, (unsigned long long) pl.Win,
                                            (unsigned long long) pl.Hin, (unsigned long long) s.b};
        const unsigned long long str[3] = {2ull * pl.Cin, 2ull * pl.Cin * pl.Win, 2ull * pl.Cin * pl.Win * pl.Hin};
        const unsigned box[4] = {64, (unsigned) p.Wp, (unsigned) p.Hs, 1};
        const unsigned estr[4] = {1, 1, 1, 1};
        if (convgemm_status_t e = tc_make_map_nd(&xmap, 4, in, dims, str, box, estr, 1)) return e;
    }
    if (convgemm_status_t e = tc_make_map_2d_sw(&wmap, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, wpacked, pl.Cout, pl.Ktot,
                                                64, SLAB_BN, CU_TENSOR_MAP_SWIZZLE_128B))
        return e;
    // output [B][Hout][Wout][Cout]: box {64 channels, Wc, R, 1}, 128-byte swizzle
    CUtensorMap omap;
    {
        const unsigned long long dims[4] = {(unsigned long long) pl.Cout, (unsigned long long) pl.Wout,
                                            (unsigned long long) pl.Hout, (unsigned long long) s.b};
        const unsigned long long str[3] = {2ull * pl.Cout, 2ull * pl.Cout * pl.Wout,
                                           2ull * pl.Cout * pl.Wout * pl.Hout};
        const unsigned box[4] = {64, (unsigned) p.Wc, (unsigned) p.R, 1};
        const unsigned estr[4] = {1, 1, 1, 1};
        if (convgemm_status_t e = tc_make_map_nd(&omap, 4, out, dims, str, box, estr, 1)) return e;
    }
    const int sms = tc_num_sms();
    const long long want = (long long) p.mtiles * p.ntn;
    int grid = (int) std::min<long long>(want, sms);
    grid = std::max(1, grid / p.ntn) * p.ntn;   // a whole number of CTAs per N tile
    const size_t smem = 1024 + p.w_bytes + (size_t) p.nbuf * p.buf_bytes + (size_t) p.nstage * SLAB_STAGE + 256 +
                        2 * SLAB_BN * 4;
    static bool attr = false;
    if (!attr) {
        if (cudaError_t e = cudaFuncSetAttribute(tc_slab_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 (int) SLAB_SMEM))
            return cg_cuda_check(e, "slab convolution attribute");
        attr = true;
    }
    return cg_cuda_check(cg_launch_pdl(tc_slab_kernel, dim3(grid), dim3(288), smem, st, p, xmap, wmap, omap),
                         "slab convolution launch");
}
