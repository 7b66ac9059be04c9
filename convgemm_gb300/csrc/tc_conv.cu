// BF16 tensor-core implicit-GEMM convolution (sm_103a, tcgen05 + TMEM + TMA).
//
// One kernel serves the forward pass (sconvGemmNHWC 'N', src/convGemm.c:65-70)
// and the input gradient (sconvGemmNHWC_back, src/convGemm.c:82-97), which it
// computes in gather form: every input-gradient pixel collects the taps that
// reach it, so there is no col2im/row2im scatter (src/im2row_nhwc.c:231-267)
// and no atomics.  A stride > 1 input gradient is split into stride-phase
// classes (pixels with the same (ih + pad) mod stride see the same taps), one
// per blockIdx.z, each a dense implicit GEMM of its own.
//
// GEMM view of one class: D[m, n] = sum_k A[m, k] * B[n, k]
//   m = output pixel of the class (128 per CTA),
//   n = output channel (BN per CTA, in TMEM columns),
//   k = tap * Cin + ci over the class's taps (64 per pipeline stage).
// A is gathered from the NHWC activation with 16-byte cp.async (zero-filled
// for padding) straight into the 128-byte-swizzled K-major layout the tensor
// core reads — no im2row buffer exists anywhere.  B is the packed weight
// matrix [Cout][K] loaded by TMA.  The FP32 accumulator lives in TMEM and the
// epilogue (per-channel scale/shift = folded bias + batch-norm, ReLU, BF16
// cast) runs TMEM -> registers -> global.
//
// Warp roles (160 threads): warps 0-3 gather A (thread 0 also issues the B
// TMA) and afterwards drain TMEM (warp w owns TMEM lanes 32w..32w+31); warp 4
// allocates TMEM and one lane issues the MMAs.
#include <cuda_bf16.h>

#include "cg_common.cuh"
#include "tc_conv.h"
#include "tc_ptx.cuh"

namespace {

using bf16 = __nv_bfloat16;

template <int BN, int STAGES>
struct TcCfg {
    static constexpr int BM = 128, BK = 64;
    static constexpr uint32_t A_BYTES = BM * BK * 2;
    static constexpr uint32_t B_BYTES = BN * BK * 2;
    static constexpr uint32_t STAGE_BYTES = A_BYTES + B_BYTES;
    static constexpr int LAG = STAGES - 1;  // cp.async groups kept in flight per producer thread
    static constexpr size_t SMEM = 1024 + (size_t) STAGES * STAGE_BYTES + 256;
};

__device__ __forceinline__ uint32_t pack_bf16x2(float a, float b) {
    __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<uint32_t *>(&v);
}

template <int BN, int STAGES>
__global__ void __launch_bounds__(160, 1)
    tc_conv_kernel(const __grid_constant__ TcConvParams p, const __grid_constant__ CUtensorMap wmap) {
    using C = TcCfg<BN, STAGES>;
    const TcClass &cl = p.cls[blockIdx.z];
    if ((int) blockIdx.x >= cl.mtiles) return;

    extern __shared__ uint8_t smem_raw[];
    uint8_t *base = (uint8_t *) (((uintptr_t) smem_raw + 1023) & ~(uintptr_t) 1023);
    uint64_t *full = (uint64_t *) (base + STAGES * C::STAGE_BYTES);
    uint64_t *empty = full + STAGES;
    uint64_t *accum = empty + STAGES;
    uint32_t *tmem_holder = (uint32_t *) (accum + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; s++) {
            tc::mbar_init(&full[s], 128 + 1);
            tc::mbar_init(&empty[s], 1);
        }
        tc::mbar_init(accum, 1);
        tc::fence_mbar_init();
        tc::prefetch_tmap(&wmap);
    }
    if (warp == 4) {
        tc::tmem_alloc(tmem_holder, BN);
        tc::tmem_relinquish();
    }
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tmem = *tmem_holder;

    const int m0 = blockIdx.x * C::BM, n0 = blockIdx.y * BN;
    const int M = p.B * cl.Hg * cl.Wg;
    const int KT = cl.ktiles;
    bool ok = true;

    if (warp < 4) {
        // ------------------------------------------------ producer: gather A
        const int t = threadIdx.x;
        const int piece = t & 7;   // 16-byte piece of the 128-byte K row
        const int r0 = t >> 3;     // rows r0 + 16*i
        int rb[8], ry[8], rx[8];
#pragma unroll
        for (int i = 0; i < 8; i++) {
            const int m = m0 + r0 + 16 * i;
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
        for (int kt = 0; kt < KT; kt++) {
            const int s = kt % STAGES;
            const uint32_t ph = (kt / STAGES) & 1;
            if (kt >= STAGES) ok = tc::mbar_wait(&empty[s], ph ^ 1, p.err, 1);
            if (!ok) break;
            const int k = kt * C::BK + piece * 8;
            uint32_t tap, ci;
            p.dcin.divmod(k, tap, ci);
            const bool kval = (int) tap < cl.ntaps;
            const int oy = kval ? cl.toy[tap] : 0, ox = kval ? cl.tox[tap] : 0;
            const uint32_t sA = tc::smem_u32(base + s * C::STAGE_BYTES);
#pragma unroll
            for (int i = 0; i < 8; i++) {
                const int r = r0 + 16 * i;
                const int iy = ry[i] + oy, ix = rx[i] + ox;
                const bool v = kval && rb[i] >= 0 && (unsigned) iy < (unsigned) p.Hin && (unsigned) ix < (unsigned) p.Win;
                const bf16 *src = v ? p.in + ((((size_t) rb[i] * p.Hin + iy) * p.Win + ix) * p.Cin + ci) : p.in;
                tc::cp_async_16(sA + r * 128 + ((piece ^ (r & 7)) << 4), src, v ? 16u : 0u);
            }
            tc::cp_async_commit();
            if (t == 0) {
                tc::mbar_arrive_expect_tx(&full[s], C::B_BYTES);
                tc::tma_load_2d(tc::smem_u32(base + s * C::STAGE_BYTES + C::A_BYTES), &wmap, cl.kbeg + kt * C::BK,
                                n0, &full[s]);
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

        // ------------------------------------------------ epilogue
        if (ok) ok = tc::mbar_wait(accum, 0, p.err, 3);
        tc::tc_fence_after();
        const int row = warp * 32 + lane;
        const int m = m0 + row;
        bf16 *orow = nullptr;
        if (m < M) {
            uint32_t q, jw, j, b;
            cl.dwg.divmod(m, q, jw);
            cl.dhg.divmod(q, b, j);
            const int oy = cl.oy0 + cl.osy * (int) j, ox = cl.ox0 + cl.osx * (int) jw;
            orow = p.out + (((size_t) b * p.Hout + oy) * p.Wout + ox) * p.Cout;
        }
        if (ok) {
#pragma unroll 1
            for (int c0 = 0; c0 < BN; c0 += 32) {
                uint32_t v[32];
                tc::tmem_ld_32x32b_x32(tmem + ((uint32_t) (warp * 32) << 16) + (uint32_t) c0, v);
                tc::tmem_ld_wait();
                const int nb = n0 + c0;
                if (orow && nb < p.Cout) {
                    float f[32];
#pragma unroll
                    for (int jj = 0; jj < 32; jj++) {
                        const int n = min(nb + jj, p.Cout - 1);
                        float a = __uint_as_float(v[jj]);
                        if (p.scale) a = a * __ldg(p.scale + n);
                        if (p.shift) a = a + __ldg(p.shift + n);
                        if (p.relu) a = fmaxf(a, 0.0f);
                        f[jj] = a;
                    }
                    if (nb + 32 <= p.Cout) {
                        uint4 *dst = reinterpret_cast<uint4 *>(orow + nb);
#pragma unroll
                        for (int q4 = 0; q4 < 4; q4++) {
                            uint4 u;
                            u.x = pack_bf16x2(f[q4 * 8 + 0], f[q4 * 8 + 1]);
                            u.y = pack_bf16x2(f[q4 * 8 + 2], f[q4 * 8 + 3]);
                            u.z = pack_bf16x2(f[q4 * 8 + 4], f[q4 * 8 + 5]);
                            u.w = pack_bf16x2(f[q4 * 8 + 6], f[q4 * 8 + 7]);
                            dst[q4] = u;
                        }
                    } else {
                        for (int jj = 0; jj < 32 && nb + jj < p.Cout; jj++) orow[nb + jj] = __float2bfloat16_rn(f[jj]);
                    }
                }
            }
        }
    } else {
        // ------------------------------------------------ MMA issuer
        if (lane == 0) {
            constexpr uint32_t idesc = tc::idesc_bf16(128, BN, 0, 0);
            for (int kt = 0; kt < KT; kt++) {
                const int s = kt % STAGES;
                const uint32_t ph = (kt / STAGES) & 1;
                if (!tc::mbar_wait(&full[s], ph, p.err, 2)) {
                    ok = false;
                    break;
                }
                tc::tc_fence_after();
                const uint32_t a0 = tc::smem_u32(base + s * C::STAGE_BYTES);
                const uint32_t b0 = a0 + C::A_BYTES;
#pragma unroll
                for (int k = 0; k < C::BK / 16; k++) {
                    const uint64_t ad = tc::sw128_desc(a0 + k * 32, 16, 1024);
                    const uint64_t bd = tc::sw128_desc(b0 + k * 32, 16, 1024);
                    tc::mma_f16(tmem, ad, bd, idesc, (kt | k) != 0);
                }
                tc::mma_commit(&empty[s]);
            }
            tc::mma_commit(accum);
        }
        __syncwarp();
    }

    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    if (warp == 4) tc::tmem_dealloc(tmem, BN);
}

template <int BN, int STAGES>
cudaError_t launch_bn(const TcConvParams &p, const CUtensorMap &map, dim3 grid, cudaStream_t st) {
    using C = TcCfg<BN, STAGES>;
    auto kern = tc_conv_kernel<BN, STAGES>;
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) C::SMEM);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    kern<<<grid, 160, C::SMEM, st>>>(p, map);
    return cudaGetLastError();
}

}  // namespace

cudaError_t tc_conv_launch(const TcConvParams &p, const CUtensorMap &map, int bn, int mtiles_max, int ntiles,
                           cudaStream_t st) {
    dim3 grid(mtiles_max, ntiles, p.ncls);
    switch (bn) {
        case 64: return launch_bn<64, 4>(p, map, grid, st);    // 97 KB: two CTAs per SM
        case 128: return launch_bn<128, 3>(p, map, grid, st);  // 97 KB: two CTAs per SM
        case 256: return launch_bn<256, 4>(p, map, grid, st);
        default: return cudaErrorInvalidValue;
    }
}
