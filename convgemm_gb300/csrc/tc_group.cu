// Persistent grouped BF16 forward convolution: many convolutions of uneven
// shapes (each an sconvGemmNHWC('N'), src/convGemm.c:65-70) in ONE launch.
//
// A device-resident problem table holds, for every convolution, its im2col
// tensor map (activations), weight and output tensor maps, geometry, tile
// width and epilogue.  The tiles of all problems are numbered consecutively
// (problem-major; inside a problem, pixel tiles x channel tiles with the
// channel tile fastest); persistent CTAs walk them blockIdx.x, +gridDim.x, ...
// The tile width (64/128/256 output channels) is a per-problem runtime value:
// shared memory and TMEM are sized for 256 and the MMA instruction descriptor
// carries N, so one launch mixes tile shapes chosen per shape by the autotuner.
//
// Warp roles as in tc_conv.cu: warp 0 lane 0 issues the im2col TMA for the
// activations and the tiled TMA for the weights; warps 4-7 drain TMEM through
// the fused scale/shift/ReLU epilogue and TMA-store BF16; warp 8 owns TMEM and
// issues tcgen05.mma.  Channels that are not a multiple of 64 are read as
// 64-channel boxes whose tail TMA zero-fills; the packed weights carry zeros there.
#include <algorithm>
#include <cstring>
#include <vector>
#include <cuda_bf16.h>

#include "../../include/convgemm_gpu.h"
#include "cg_common.cuh"
#include "prep.h"
#include "tc_host.h"
#include "tc_epi.cuh"
#include "tc_ptx.cuh"

namespace {

using bf16 = __nv_bfloat16;

struct alignas(64) GroupProblem {
    CUtensorMap amap;   // im2col map of x: 128 pixels x 64 channels per load
    CUtensorMap wmap;   // packed weights [kn][taps * c64]: box 64 x bn
    CUtensorMap omap;   // y as [pixels][kn]: box 64 x 32 (one epilogue warp's rows)
    int tile0, tile_end, count, ntiles_n, bn, M;   // count: convolutions in the table
    int ktiles, cpb, isy, isx, lo_y, lo_x, Cout, relu;
    uint32_t idesc;
    FastDiv dwg, dhg;
    const float *scale, *shift;
    int32_t taps[TC_MAXTAPS];   // (offy << 16) | offx of each tap
};

constexpr int GBN = 256;
constexpr int GSTAGES = 4;
constexpr uint32_t A_BYTES = 128 * 128;
constexpr uint32_t B_MAX = GBN * 128;
constexpr uint32_t STAGE_BYTES = A_BYTES + B_MAX;
constexpr uint32_t EPI_BYTES = 128 * 128;   // one 64-column chunk of a tile (4 KB per epilogue warp)
constexpr size_t GSMEM = 1024 + GSTAGES * STAGE_BYTES + EPI_BYTES + 256 + 2 * GBN * 4;
static_assert(GSMEM <= 232448, "shared memory above the 227 KB per-block limit");

__device__ __forceinline__ void epi_bar() { asm volatile("bar.sync 1, 128;" ::: "memory"); }

__device__ __forceinline__ int advance(const GroupProblem *probs, int nprob, int pi, int tile) {
    while (pi + 1 < nprob && tile >= __ldg(&probs[pi + 1].tile0)) pi++;
    return pi;
}

__global__ void __launch_bounds__(288, 1)
    tc_group_kernel(const GroupProblem *__restrict__ probs, int nprob, int total, int *err) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t *base = (uint8_t *) (((uintptr_t) smem_raw + 1023) & ~(uintptr_t) 1023);
    uint8_t *epi = base + GSTAGES * STAGE_BYTES;
    uint64_t *full = (uint64_t *) (epi + EPI_BYTES);
    uint64_t *empty = full + GSTAGES;
    uint64_t *acc_full = empty + GSTAGES;
    uint64_t *acc_empty = acc_full + 2;
    uint32_t *tmem_holder = (uint32_t *) (acc_empty + 2);
    float *sc_tab = (float *) (epi + EPI_BYTES + 256);
    float *sh_tab = sc_tab + GBN;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    tc::pdl_wait();   // pdl_trigger: when the producer starts this CTA's last tile
    // a table prepared for another count, or a tile count beyond the table: run nothing
    if (__ldg(&probs[0].count) != nprob) {
        if (threadIdx.x == 0) atomicCAS(err, 0, 25);
        return;
    }
    total = min(total, __ldg(&probs[nprob - 1].tile_end));
    if (threadIdx.x == 0) {
        for (int s = 0; s < GSTAGES; s++) {
            tc::mbar_init(&full[s], 1);
            tc::mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; b++) {
            tc::mbar_init(&acc_full[b], 1);
            tc::mbar_init(&acc_empty[b], 128);
        }
        tc::fence_mbar_init();
    }
    if (warp == 8) {
        tc::tmem_alloc(tmem_holder, 2 * GBN);
        tc::tmem_relinquish();
    }
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tmem = *tmem_holder;
    bool ok = true;

    if (warp < 4) {
        if (threadIdx.x == 0) {
            // ---------------------------------------------- producer
            uint32_t it = 0;
            int pi = 0;
            for (int tile = blockIdx.x; tile < total && ok; tile += gridDim.x) {
                if (tile + (int) gridDim.x >= total) tc::pdl_trigger();   // this CTA's last tile
                pi = advance(probs, nprob, pi, tile);
                const GroupProblem *P = probs + pi;
                const int local = tile - __ldg(&P->tile0), ntn = __ldg(&P->ntiles_n), bn = __ldg(&P->bn);
                const int m0 = (local / ntn) * 128, n0 = (local % ntn) * bn;
                const int ktiles = __ldg(&P->ktiles), cpb = __ldg(&P->cpb);
                const FastDiv dwg = P->dwg, dhg = P->dhg;
                uint32_t q, jw, j, b;
                dwg.divmod(m0, q, jw);
                dhg.divmod(q, b, j);
                const int h0 = (int) j * __ldg(&P->isy) + __ldg(&P->lo_y);
                const int w0 = (int) jw * __ldg(&P->isx) + __ldg(&P->lo_x);
                const uint32_t tx_bytes = A_BYTES + (uint32_t) bn * 128;
                int tap = 0, cc = 0;
                for (int kt = 0; kt < ktiles; kt++, it++) {
                    const int s = it % GSTAGES;
                    const uint32_t ph = (it / GSTAGES) & 1;
                    if (it >= (uint32_t) GSTAGES && !(ok = tc::mbar_wait(&empty[s], ph ^ 1, err, 21))) break;
                    const int32_t to = __ldg(&P->taps[tap]);
                    const uint32_t sa = tc::smem_u32(base + s * STAGE_BYTES);
                    tc::mbar_arrive_expect_tx(&full[s], tx_bytes);
                    tc::tma_load_im2col_4d(sa, &P->amap, cc * 64, w0, h0, (int) b, (uint16_t) (to & 0xFFFF),
                                           (uint16_t) (to >> 16), &full[s]);
                    tc::tma_load_2d(sa + A_BYTES, &P->wmap, kt * 64, n0, &full[s]);
                    if (++cc == cpb) {
                        cc = 0;
                        tap++;
                    }
                }
            }
        }
    } else if (warp < 8) {
        // -------------------------------------------------- epilogue
        const int ew = warp - 4, row = ew * 32 + lane, et = threadIdx.x - 128;
        uint32_t lt = 0;
        int pi = 0;
        for (int tile = blockIdx.x; tile < total && ok; tile += gridDim.x, lt++) {
            pi = advance(probs, nprob, pi, tile);
            const GroupProblem *P = probs + pi;
            const int local = tile - __ldg(&P->tile0), ntn = __ldg(&P->ntiles_n), bn = __ldg(&P->bn);
            const int m0 = (local / ntn) * 128, n0 = (local % ntn) * bn;
            const int Cout = __ldg(&P->Cout), relu = __ldg(&P->relu), M = __ldg(&P->M);
            const float *scale = P->scale, *shift = P->shift;
            epi_bar();   // the previous tile's readers of the tables are done
            for (int jj = et; jj < bn; jj += 128) {
                const int n = min(n0 + jj, Cout - 1);
                sc_tab[jj] = scale ? __ldg(scale + n) : 1.0f;
                sh_tab[jj] = shift ? __ldg(shift + n) : 0.0f;
            }
            epi_bar();
            const int buf = lt & 1;
            ok = tc::mbar_wait(&acc_full[buf], (lt >> 1) & 1, err, 23);
            if (!ok) break;
            tc::tc_fence_after();
            for (int c0 = 0; c0 < bn; c0 += 64) {
                uint32_t v0[32], v1[32];
                const uint32_t ta = tmem + ((uint32_t) (ew * 32) << 16) + (uint32_t) (buf * GBN + c0);
                tc::tmem_ld_32x32b_x32(ta, v0);
                tc::tmem_ld_32x32b_x32(ta + 32, v1);
                tc::tmem_ld_wait();
                if (c0 + 64 >= bn) {
                    tc::tc_fence_before();
                    tc::mbar_arrive(&acc_empty[buf]);
                }
                uint32_t pk[32];
                if (relu)
                    tc::epi_bf16_64<true>(v0, v1, sc_tab + c0, sh_tab + c0, pk);
                else
                    tc::epi_bf16_64<false>(v0, v1, sc_tab + c0, sh_tab + c0, pk);
                // each warp stages its 32 rows and stores them itself: no barrier across warps
                if (lane == 0) asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
                __syncwarp();
                uint8_t *stg = epi + ew * (EPI_BYTES / 4);
#pragma unroll
                for (int qq = 0; qq < 8; qq++)
                    *reinterpret_cast<uint4 *>(stg + lane * 128 + ((qq ^ (lane & 7)) << 4)) =
                        make_uint4(pk[4 * qq], pk[4 * qq + 1], pk[4 * qq + 2], pk[4 * qq + 3]);
                tc::fence_proxy_async_smem();
                __syncwarp();
                if (lane == 0 && n0 + c0 < Cout && m0 + ew * 32 < M) {
                    asm volatile(
                        "cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%2, %3}], [%1];" ::"l"(
                            (uint64_t) &P->omap),
                        "r"(tc::smem_u32(stg)), "r"(n0 + c0), "r"(m0 + ew * 32)
                        : "memory");
                    asm volatile("cp.async.bulk.commit_group;" ::: "memory");
                }
            }
        }
        if (lane == 0) asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
    } else {
        // -------------------------------------------------- MMA issuer
        if (lane == 0) {
            uint32_t it = 0, lt = 0;
            int pi = 0;
            for (int tile = blockIdx.x; tile < total && ok; tile += gridDim.x, lt++) {
                pi = advance(probs, nprob, pi, tile);
                const GroupProblem *P = probs + pi;
                const int ktiles = __ldg(&P->ktiles);
                const uint32_t idesc = __ldg(&P->idesc);
                const int buf = lt & 1;
                if (lt >= 2) {
                    ok = tc::mbar_wait(&acc_empty[buf], ((lt >> 1) - 1) & 1, err, 24);
                    if (!ok) break;
                    tc::tc_fence_after();
                }
                const uint32_t dt = tmem + (uint32_t) (buf * GBN);
                for (int kt = 0; kt < ktiles; kt++, it++) {
                    const int s = it % GSTAGES;
                    const uint32_t ph = (it / GSTAGES) & 1;
                    if (!tc::mbar_wait(&full[s], ph, err, 22)) {
                        ok = false;
                        break;
                    }
                    tc::tc_fence_after();
                    // descriptors built once per stage; a 32-byte K step adds 2 to the start field
                    const uint64_t ad = tc::sw128_desc(tc::smem_u32(base + s * STAGE_BYTES), 16, 1024);
                    const uint64_t bd = ad + (A_BYTES >> 4);
#pragma unroll
                    for (int k = 0; k < 4; k++) tc::mma_f16(dt, ad + 2 * k, bd + 2 * k, idesc, (kt | k) != 0);
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
    if (warp == 8) tc::tmem_dealloc(tmem, 2 * GBN);
}

inline int rup(int v, int m) { return (v + m - 1) / m * m; }

convgemm_status_t check_group_shape(const convgemm_shape_t &s, const char *fn) {
    if (s.b < 1 || s.h < 1 || s.w < 1 || s.c < 1 || s.kn < 1 || s.kh < 1 || s.kw < 1 || s.vstride < 1 ||
        s.hstride < 1 || s.vdil < 1 || s.hdil < 1 || s.vpad < 0 || s.hpad < 0 ||
        s.h + 2LL * s.vpad - (long long) s.vdil * (s.kh - 1) < 1 ||
        s.w + 2LL * s.hpad - (long long) s.hdil * (s.kw - 1) < 1)
        return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "%s: invalid geometry", fn);
    if (s.c % 8 || s.kn % 8 || s.kh * s.kw > TC_MAXTAPS || s.vstride > 8 || s.hstride > 8)
        return cg_set_error(CONVGEMM_ERROR_NOT_SUPPORTED, "%s: needs c %% 8 == 0, kn %% 8 == 0, <= 49 taps, strides <= 8",
                            fn);
    return CONVGEMM_SUCCESS;
}

}  // namespace

extern "C" size_t convgemm_group_weights_size(const convgemm_shape_t *shape) {
    if (!shape || check_group_shape(*shape, "convgemm_group_weights_size")) return 0;
    return (size_t) shape->kn * (size_t) (shape->kh * shape->kw * rup(shape->c, 64)) * 2;
}

extern "C" convgemm_status_t convgemm_group_pack_weights(convgemm_layout_t layout, const convgemm_shape_t *shape,
                                                         const float *weights, void *packed, void *stream) {
    if (!shape || !weights || !packed)
        return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "convgemm_group_pack_weights: NULL");
    if (convgemm_status_t e = check_group_shape(*shape, "convgemm_group_pack_weights")) return e;
    const convgemm_shape_t &s = *shape;
    const int c64 = rup(s.c, 64);
    return cg_cuda_check(prep_pack_fwd(weights, layout == CONVGEMM_NCHW, s.c, s.kh, s.kw, s.kn, c64, s.kh * s.kw * c64,
                                       packed, (cudaStream_t) stream),
                         "pack grouped weights");
}

extern "C" size_t convgemm_group_table_size(int n) { return n > 0 ? (size_t) n * sizeof(GroupProblem) : 0; }

extern "C" convgemm_status_t convgemm_group_prepare(int n, const convgemm_group_conv_t *convs, void *table,
                                                    size_t table_bytes, int *total_tiles) {
    const char *fn = "convgemm_group_prepare";
    if (n < 1 || !convs || !table || !total_tiles)
        return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "%s: bad arguments", fn);
    if (table_bytes < convgemm_group_table_size(n) || ((uintptr_t) table & 63))
        return cg_set_error(CONVGEMM_ERROR_WORKSPACE, "%s: table needs %zu bytes, 64-byte aligned", fn,
                            convgemm_group_table_size(n));
    // Tiles go to the persistent CTAs round-robin, so the table lists the
    // convolutions by decreasing K length (the cost of one of their tiles):
    // every CTA then gets a similar mix of long and short tiles.
    std::vector<int> order(n);
    for (int i = 0; i < n; i++) order[i] = i;
    auto klen = [&](int i) {
        const convgemm_shape_t &s = convs[i].shape;
        return (long long) s.kh * s.kw * rup(s.c > 0 ? s.c : 1, 64);
    };
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return klen(a) > klen(b); });
    std::vector<GroupProblem> host(n);
    int t0 = 0;
    for (int oi = 0; oi < n; oi++) {
        const int i = order[oi];
        const convgemm_group_conv_t &cv = convs[i];
        if (convgemm_status_t e = check_group_shape(cv.shape, fn)) return e;
        if (!cv.x || !cv.w || !cv.y) return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "%s: conv %d has a NULL tensor", fn, i);
        const cg_shape s = cg_from_public(cv.shape);
        const ConvGeom g = make_geom(s);
        const int bn = cv.bn == 64 || cv.bn == 128 || cv.bn == 256 ? cv.bn : (s.kn >= 256 ? 256 : (s.kn > 64 ? 128 : 64));
        const int c64 = rup(s.c, 64);
        GroupProblem &P = host[oi];
        memset(&P, 0, sizeof(P));
        const int lo_y = -s.vpad, lo_x = -s.hpad;
        const int up_y = lo_y + (g.ho - 1) * s.vstride - (s.h - 1), up_x = lo_x + (g.wo - 1) * s.hstride - (s.w - 1);
        if (lo_y < -128 || lo_x < -128 || up_y < -128 || up_y > 127 || up_x < -128 || up_x > 127)
            return cg_set_error(CONVGEMM_ERROR_NOT_SUPPORTED, "%s: conv %d: padding outside the im2col box range", fn, i);
        if (convgemm_status_t e = tc_make_im2col_map(&P.amap, cv.x, s.b, s.h, s.w, s.c, lo_y, lo_x, up_y, up_x,
                                                     s.vstride, s.hstride, 128, 2))
            return e;
        if (convgemm_status_t e = tc_make_map_2d(&P.wmap, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, cv.w, s.kn,
                                                 s.kh * s.kw * c64, 64, bn))
            return e;
        if (convgemm_status_t e = tc_make_map_2d(&P.omap, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, cv.y, g.P, s.kn, 64, 32))
            return e;
        if (g.P > (1LL << 31) - 256 || (long long) s.b * s.h * s.w * c64 > (1LL << 31) - 1)
            return cg_set_error(CONVGEMM_ERROR_NOT_SUPPORTED, "%s: conv %d has more than 2^31 elements", fn, i);
        P.tile0 = t0;
        P.count = n;
        P.ntiles_n = (s.kn + bn - 1) / bn;
        P.bn = bn;
        P.M = (int) g.P;
        P.cpb = c64 / 64;
        P.ktiles = s.kh * s.kw * P.cpb;
        P.isy = s.vstride;
        P.isx = s.hstride;
        P.lo_y = lo_y;
        P.lo_x = lo_x;
        P.Cout = s.kn;
        P.relu = cv.relu;
        P.idesc = tc::idesc_bf16(128, bn, 0, 0);
        P.dwg = FastDiv(g.wo);
        P.dhg = FastDiv(g.ho);
        P.scale = cv.scale;
        P.shift = cv.shift;
        for (int kx = 0; kx < s.kh; kx++)
            for (int ky = 0; ky < s.kw; ky++)
                P.taps[kx * s.kw + ky] = ((kx * s.vdil) << 16) | (ky * s.hdil);
        const long long end = t0 + (long long) ((g.P + 127) / 128) * P.ntiles_n;
        if (end > (1LL << 31) - 1) return cg_set_error(CONVGEMM_ERROR_NOT_SUPPORTED, "%s: more than 2^31 tiles", fn);
        t0 = (int) end;
        P.tile_end = t0;
    }
    *total_tiles = t0;
    return cg_cuda_check(cudaMemcpy(table, host.data(), sizeof(GroupProblem) * n, cudaMemcpyHostToDevice),
                         "copy group table");
}

extern "C" convgemm_status_t convgemm_group_launch(const void *table, int n, int total_tiles, void *stream) {
    if (!table || n < 1 || total_tiles < 1 || ((uintptr_t) table & 63))
        return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "convgemm_group_launch: bad arguments");
    int *err = cg_device_error_word();
    if (!err) return cg_set_error(CONVGEMM_ERROR_CUDA, "device error word unavailable");
    static bool attr = false;
    if (!attr) {
        if (convgemm_status_t e = cg_cuda_check(
                cudaFuncSetAttribute(tc_group_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) GSMEM),
                "grouped kernel attributes"))
            return e;
        attr = true;
    }
    const int sms = tc_num_sms();
    const int grid = total_tiles < sms ? total_tiles : sms;
    return cg_cuda_check(cg_launch_pdl(tc_group_kernel, dim3(grid), dim3(288), GSMEM, (cudaStream_t) stream,
                                       (const GroupProblem *) table, n, total_tiles, err),
                         "grouped kernel launch");
}
