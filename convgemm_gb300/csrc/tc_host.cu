// Host side of the BF16 tensor-core forms: problem planning (tap tables,
// stride-phase classes of the input gradient), packed-weight layouts, TMA
// tensor maps, and the public convgemm_*_bf16 entry points.
#include <cstring>
#include <mutex>
#include <vector>

#include "../../include/convgemm_gpu.h"
#include "cg_common.cuh"
#include "prep.h"
#include "tc_conv.h"
#include "tc_host.h"

namespace {

inline int round_up(int v, int m) { return (v + m - 1) / m * m; }

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
    static EncodeTiledFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (EncodeTiledFn) p;
    });
    return fn;
}

int pick_bn(int cout) { return cout >= 256 ? 256 : (cout > 64 ? 128 : 64); }

typedef CUresult (*EncodeIm2colFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                   const cuuint64_t *, const int *, const int *, cuuint32_t, cuuint32_t,
                                   const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                   CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeIm2colFn encode_im2col_fn() {
    static EncodeIm2colFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeIm2col", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (EncodeIm2colFn) p;
    });
    return fn;
}

}  // namespace

// im2col-mode map of a BF16 NHWC tensor [B][H][W][C]: `pixels` pixels x 64 channels per load,
// bounding box [lo, dim-1+up] per spatial dimension, traversal strides (sh, sw), 128-byte swizzle.
convgemm_status_t tc_make_map_nd(CUtensorMap *map, int rank, const void *ptr, const unsigned long long *dims,
                                  const unsigned long long *strides_bytes, const unsigned *box, const unsigned *estr,
                                  int swizzle128) {
    return tc_make_map_nd_dt(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, rank, ptr, dims, strides_bytes, box, estr, swizzle128);
}

convgemm_status_t tc_make_map_nd_dt(CUtensorMap *map, CUtensorMapDataType dt, int rank, const void *ptr,
                                     const unsigned long long *dims, const unsigned long long *strides_bytes,
                                     const unsigned *box, const unsigned *estr, int swizzle128) {
    EncodeTiledFn fn = encode_fn();
    if (!fn) return cg_set_error(CONVGEMM_ERROR_CUDA, "cuTensorMapEncodeTiled is unavailable");
    if ((uintptr_t) ptr & 15) return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "TMA operand not 16-byte aligned");
    cuuint64_t d[5], st[4];
    cuuint32_t b[5], e[5];
    for (int i = 0; i < rank; i++) {
        d[i] = dims[i];
        b[i] = box[i];
        e[i] = estr[i];
        if (i < rank - 1) {
            st[i] = strides_bytes[i];
            if (st[i] % 16) return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "TMA stride not a multiple of 16 bytes");
        }
    }
    CUresult r = fn(map, dt, (cuuint32_t) rank, const_cast<void *>(ptr), d, st, b, e,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, swizzle128 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_NONE,
                    CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return cg_set_error(CONVGEMM_ERROR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int) r);
    return CONVGEMM_SUCCESS;
}

convgemm_status_t tc_make_im2col_map(CUtensorMap *map, const void *ptr, int B, int H, int W, int C, int lo_h,
                                     int lo_w, int up_h, int up_w, int sh, int sw, int pixels, int elem_bytes,
                                     int chans) {
    EncodeIm2colFn fn = encode_im2col_fn();
    if (!fn) return cg_set_error(CONVGEMM_ERROR_CUDA, "cuTensorMapEncodeIm2col is unavailable");
    if (((uintptr_t) ptr & 15) || (C * elem_bytes) % 16)
        return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "im2col operand not 16-byte aligned");
    const cuuint64_t eb = (cuuint64_t) elem_bytes;
    cuuint64_t dims[4] = {(cuuint64_t) C, (cuuint64_t) W, (cuuint64_t) H, (cuuint64_t) B};
    cuuint64_t strides[3] = {(cuuint64_t) C * eb, (cuuint64_t) W * C * eb, (cuuint64_t) H * W * C * eb};
    int lower[2] = {lo_w, lo_h};
    int upper[2] = {up_w, up_h};
    cuuint32_t estr[4] = {1, (cuuint32_t) sw, (cuuint32_t) sh, 1};
    // `chans` channels per pixel: 128 B rows (64 BF16 or 128 E4M3, 128-byte swizzle) or 64 B rows
    // (64 E4M3, 64-byte swizzle)
    CUresult r = fn(map, elem_bytes == 1 ? CU_TENSOR_MAP_DATA_TYPE_UINT8 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4,
                    const_cast<void *>(ptr), dims, strides, lower, upper, (cuuint32_t) chans, (cuuint32_t) pixels, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE,
                    chans * elem_bytes == 64 ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_128B,
                    CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return cg_set_error(CONVGEMM_ERROR_CUDA, "cuTensorMapEncodeIm2col failed (%d)", (int) r);
    return CONVGEMM_SUCCESS;
}

// Fills the im2col fields of the plan's classes; false when some class cannot use
// im2col-mode TMA (channels not a multiple of 64, too many classes, corners beyond +-128).
bool tc_plan_im2col(TcPlan &pl) {
    if (pl.Cin % 64 || pl.ncls > TC_MAXIM2COL || pl.ncls < 1) return false;
    for (int c = 0; c < pl.ncls; c++) {
        TcClass &cl = pl.cls[c];
        int my = 1 << 30, mx = 1 << 30, Xy = -(1 << 30), Xx = -(1 << 30);
        for (int t = 0; t < cl.ntaps; t++) {
            my = cl.toy[t] < my ? cl.toy[t] : my;
            mx = cl.tox[t] < mx ? cl.tox[t] : mx;
            Xy = cl.toy[t] > Xy ? cl.toy[t] : Xy;
            Xx = cl.tox[t] > Xx ? cl.tox[t] : Xx;
        }
        cl.mint_y = my;
        cl.mint_x = mx;
        cl.lo_y = cl.iby + my;
        cl.lo_x = cl.ibx + mx;
        const int up_y = cl.lo_y + (cl.Hg - 1) * cl.isy - (pl.Hin - 1);
        const int up_x = cl.lo_x + (cl.Wg - 1) * cl.isx - (pl.Win - 1);
        if (cl.lo_y < -128 || cl.lo_y > 127 || cl.lo_x < -128 || cl.lo_x > 127 || up_y < -128 || up_y > 127 ||
            up_x < -128 || up_x > 127 || Xy - my > 65535 || Xx - mx > 65535 || cl.isy > 8 || cl.isx > 8)
            return false;
    }
    return true;
}

// 2-D row-major [rows][cols] tensor, box {64 (cols), box_rows}, 128-byte swizzle.
convgemm_status_t tc_make_map_2d(CUtensorMap *map, CUtensorMapDataType dt, int elem_bytes, const void *ptr,
                                 long long rows, long long cols, int box_cols, int box_rows) {
    return tc_make_map_2d_sw(map, dt, elem_bytes, ptr, rows, cols, box_cols, box_rows, CU_TENSOR_MAP_SWIZZLE_128B);
}

convgemm_status_t tc_make_map_2d_sw(CUtensorMap *map, CUtensorMapDataType dt, int elem_bytes, const void *ptr,
                                    long long rows, long long cols, int box_cols, int box_rows, CUtensorMapSwizzle sw) {
    EncodeTiledFn fn = encode_fn();
    if (!fn) return cg_set_error(CONVGEMM_ERROR_CUDA, "cuTensorMapEncodeTiled is unavailable");
    if (((uintptr_t) ptr & 15) || ((cols * elem_bytes) & 15))
        return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "TMA operand not 16-byte aligned");
    cuuint64_t dims[2] = {(cuuint64_t) cols, (cuuint64_t) rows};
    cuuint64_t strides[1] = {(cuuint64_t) cols * elem_bytes};
    cuuint32_t box[2] = {(cuuint32_t) box_cols, (cuuint32_t) box_rows};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = fn(map, dt, 2, const_cast<void *>(ptr), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, sw,
                    CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return cg_set_error(CONVGEMM_ERROR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int) r);
    return CONVGEMM_SUCCESS;
}

// ------------------------------------------------------------ planning
bool tc_plan_fwd(const cg_shape &s, TcPlan &pl) {
    const ConvGeom g = make_geom(s);
    if (s.kh * s.kw > TC_MAXTAPS) return false;
    pl.Cin = round_up(s.c, 8);
    pl.Cout = s.kn;
    pl.Hin = s.h;
    pl.Win = s.w;
    pl.Hout = g.ho;
    pl.Wout = g.wo;
    pl.ncls = 1;
    TcClass &c = pl.cls[0];
    memset(&c, 0, sizeof(c));
    c.Hg = g.ho;
    c.Wg = g.wo;
    c.oy0 = c.ox0 = 0;
    c.osy = c.osx = 1;
    c.isy = s.vstride;
    c.isx = s.hstride;
    c.iby = -s.vpad;
    c.ibx = -s.hpad;
    c.ntaps = s.kh * s.kw;
    for (int kx = 0; kx < s.kh; kx++)
        for (int ky = 0; ky < s.kw; ky++) {
            c.toy[kx * s.kw + ky] = (int16_t) (kx * s.vdil);
            c.tox[kx * s.kw + ky] = (int16_t) (ky * s.hdil);
            pl.kx[0][kx * s.kw + ky] = (int8_t) kx;
            pl.ky[0][kx * s.kw + ky] = (int8_t) ky;
        }
    c.kbeg = 0;
    c.ktiles = (c.ntaps * pl.Cin + 63) / 64;
    c.mtiles = (int) ((g.P + 127) / 128);
    c.dwg = FastDiv(c.Wg);
    c.dhg = FastDiv(c.Hg);
    pl.Ktot = c.ktiles * 64;
    pl.mtiles_max = c.mtiles;
    pl.has_empty_class = false;
    pl.bn = pick_bn(pl.Cout);
    return true;
}

bool tc_plan_dgrad(const cg_shape &s, TcPlan &pl) {
    const ConvGeom g = make_geom(s);
    const int sy = s.vstride, sx = s.hstride;
    if (sy * sx > TC_MAXCLS || s.kh * s.kw > TC_MAXTAPS) return false;
    pl.Cin = round_up(s.kn, 8);   // the gathered tensor is dY
    pl.Cout = s.c;
    pl.Hin = g.ho;
    pl.Win = g.wo;
    pl.Hout = s.h;
    pl.Wout = s.w;
    pl.ncls = 0;
    pl.has_empty_class = false;
    pl.mtiles_max = 0;
    int kb = 0;
    for (int cy = 0; cy < sy; cy++)
        for (int cx = 0; cx < sx; cx++) {
            const int Hg = s.h > cy ? (s.h - cy + sy - 1) / sy : 0;
            const int Wg = s.w > cx ? (s.w - cx + sx - 1) / sx : 0;
            if (Hg == 0 || Wg == 0) continue;
            TcClass &c = pl.cls[pl.ncls];
            memset(&c, 0, sizeof(c));
            int nt = 0;
            for (int kx = 0; kx < s.kh; kx++) {
                const int ty = cy + s.vpad - kx * s.vdil;
                if (((ty % sy) + sy) % sy) continue;
                for (int ky = 0; ky < s.kw; ky++) {
                    const int tx = cx + s.hpad - ky * s.hdil;
                    if (((tx % sx) + sx) % sx) continue;
                    c.toy[nt] = (int16_t) (ty / sy);
                    c.tox[nt] = (int16_t) (tx / sx);
                    pl.kx[pl.ncls][nt] = (int8_t) kx;
                    pl.ky[pl.ncls][nt] = (int8_t) ky;
                    nt++;
                }
            }
            if (nt == 0) {
                pl.has_empty_class = true;
                continue;
            }
            c.Hg = Hg;
            c.Wg = Wg;
            c.oy0 = cy;
            c.ox0 = cx;
            c.osy = sy;
            c.osx = sx;
            c.isy = c.isx = 1;
            c.iby = c.ibx = 0;
            c.ntaps = nt;
            c.kbeg = kb;
            c.ktiles = (nt * pl.Cin + 63) / 64;
            kb += c.ktiles * 64;
            c.mtiles = (int) (((long long) s.b * Hg * Wg + 127) / 128);
            c.dwg = FastDiv(Wg);
            c.dhg = FastDiv(Hg);
            if (c.mtiles > pl.mtiles_max) pl.mtiles_max = c.mtiles;
            pl.ncls++;
        }
    pl.Ktot = kb;
    pl.bn = pick_bn(pl.Cout);
    return true;
}

PackDgradInfo tc_pack_info(const TcPlan &pl) {
    PackDgradInfo info;
    memset(&info, 0, sizeof(info));
    info.ncls = pl.ncls;
    info.Ktot = pl.Ktot;
    for (int c = 0; c < pl.ncls; c++) {
        info.kbeg[c] = pl.cls[c].kbeg;
        info.ntaps[c] = pl.cls[c].ntaps;
        memcpy(info.kx[c], pl.kx[c], TC_MAXTAPS);
        memcpy(info.ky[c], pl.ky[c], TC_MAXTAPS);
    }
    return info;
}

int tc_num_sms() {
    static int n = 0;
    if (n == 0) {
        int dev = 0, v = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0) v = 148;
        n = v;
    }
    return n;
}

// Output channels per tile: fewest waves of tiles times the per-stage cost of a
// tile (the 16 KB A gather bounds a stage at ~128 cycles; the MMA takes 2*BN).
int tc_pick_bn(const TcPlan &pl, int sms) {
    int best = 64;
    long long best_cost = -1;
    for (int bn : {256, 128, 64}) {
        if (bn > 64 && bn / 2 >= pl.Cout) continue;
        long long tiles = 0;
        for (int c = 0; c < pl.ncls; c++) tiles += (long long) pl.cls[c].mtiles * ((pl.Cout + bn - 1) / bn);
        const long long waves = (tiles + sms - 1) / sms;
        const long long cost = waves * (bn * 2 > 128 ? bn * 2 : 128);
        if (best_cost < 0 || cost < best_cost) {
            best_cost = cost;
            best = bn;
        }
    }
    return best;
}

convgemm_status_t tc_run(const TcPlan &pl, const cg_shape &s, const void *in, const void *wpacked, void *out,
                         const float *scale, const float *shift, int relu, cudaStream_t st, int mode,
                         const void *in_lo, const void *w_lo, int bn_override, int aux_override,
                         const void *mask, float *stats, int accum) {
    if (pl.ncls == 0) return CONVGEMM_SUCCESS;
    // stride-1 layers with 64-channel blocks and several taps: operands from input slabs, unless the
    // tuning entry asks for the general kernel (aux bit 8)
    if (mode == 0 && !mask && !stats && !accum && !(aux_override & 8) && tc_slab_applicable(pl) && !((uintptr_t) out & 15) &&
        !((uintptr_t) in & 15) && !((uintptr_t) wpacked & 15))
        return tc_slab_run(pl, s, in, wpacked, out, scale, shift, relu, st);
    const int sms = tc_num_sms();
    TcConvParams p;
    memset(&p, 0, sizeof(p));
    p.mode = mode;
    p.bn = bn_override ? bn_override : tc_pick_bn(pl, sms);
    const int eb = mode == 1 ? 1 : 2;   // operand element bytes
    CUtensorMap wmap, omap;
    if (convgemm_status_t e = tc_make_map_2d_sw(&wmap, eb == 1 ? CU_TENSOR_MAP_DATA_TYPE_UINT8 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16,
                                                eb, wpacked, pl.Cout, pl.Ktot, 64, p.bn,
                                                eb == 1 ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_128B))
        return e;
    const TcClass &c0 = pl.cls[0];
    p.epi_tma = pl.ncls == 1 && c0.osy == 1 && c0.osx == 1 && c0.oy0 == 0 && c0.ox0 == 0 && c0.Hg == pl.Hout &&
                c0.Wg == pl.Wout && (pl.Cout % 8) == 0 && ((uintptr_t) out & 15) == 0;
    memset(&omap, 0, sizeof(omap));
    if (p.epi_tma) {
        // 128-byte rows of output: 64 BF16 or 32 FP32 (3xBF16) channels
        const bool f32 = mode == 2;
        if (convgemm_status_t e = tc_make_map_2d(&omap, f32 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16,
                                                 f32 ? 4 : 2, out, (long long) s.b * pl.Hout * pl.Wout, pl.Cout,
                                                 f32 ? 32 : 64, 32))
            return e;
    }
    p.in = (const __nv_bfloat16 *) in;
    p.out = (__nv_bfloat16 *) out;
    p.scale = scale;
    p.shift = shift;
    p.relu = relu;
    p.mask = (const __nv_bfloat16 *) mask;
    p.accum = accum;
    p.stats = stats;
    p.B = s.b;
    p.Hin = pl.Hin;
    p.Win = pl.Win;
    p.Cin = pl.Cin;
    p.Hout = pl.Hout;
    p.Wout = pl.Wout;
    p.Cout = pl.Cout;
    p.dcin = FastDiv(pl.Cin);
    p.err = cg_device_error_word();
    if (!p.err) return cg_set_error(CONVGEMM_ERROR_CUDA, "device error word unavailable");
    p.ntiles = (pl.Cout + p.bn - 1) / p.bn;
    p.ncls = pl.ncls;
    TcPlan pi = pl;
    TcMaps amaps;
    memset(&amaps, 0, sizeof(amaps));
    p.im2col = tc_plan_im2col(pi);
    if (mode != 0 && !p.im2col)
        return cg_set_error(CONVGEMM_ERROR_NOT_SUPPORTED,
                            "FP8 / 3xBF16 forms need channels a multiple of 64 (im2col-mode TMA)");
    // E4M3 with channels a multiple of 128: 128-channel K blocks (128-byte rows and swizzle, one
    // 16 KB box per 128-row block and four 32-deep MMAs per block, as BF16) instead of 64-byte rows
    bool f8w = mode == 1 && p.im2col && pl.Cin % 128 == 0 && pl.Ktot % 128 == 0;
    for (int c = 0; f8w && c < pi.ncls; c++)
        if (pi.cls[c].kbeg % 128 || pi.cls[c].ktiles % 2) f8w = false;
    if (f8w) {
        if (convgemm_status_t e = tc_make_map_2d_sw(&wmap, CU_TENSOR_MAP_DATA_TYPE_UINT8, 1, wpacked, pl.Cout, pl.Ktot,
                                                    128, p.bn, CU_TENSOR_MAP_SWIZZLE_128B))
            return e;
    }
    if (p.im2col) {
        p.cpb = pl.Cin / 64;
        for (int c = 0; c < pi.ncls; c++) {
            const TcClass &cl = pi.cls[c];
            const int up_y = cl.lo_y + (cl.Hg - 1) * cl.isy - (pl.Hin - 1);
            const int up_x = cl.lo_x + (cl.Wg - 1) * cl.isx - (pl.Win - 1);
            if (convgemm_status_t e = tc_make_im2col_map(&amaps.a[c], in, s.b, pl.Hin, pl.Win, pl.Cin, cl.lo_y,
                                                         cl.lo_x, up_y, up_x, cl.isy, cl.isx, 128, eb, f8w ? 128 : 64))
                return e;
            if (mode == 2)
                if (convgemm_status_t e = tc_make_im2col_map(&amaps.alo[c], in_lo, s.b, pl.Hin, pl.Win, pl.Cin,
                                                             cl.lo_y, cl.lo_x, up_y, up_x, cl.isy, cl.isx, 128, 2, 64))
                    return e;
        }
        if (mode == 2)
            if (convgemm_status_t e =
                    tc_make_map_2d(&amaps.wlo, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, w_lo, pl.Cout, pl.Ktot, 64, p.bn))
                return e;
    }
    // aux (tuning): bits 0-1 the M tiles per weight tile (1 / 2: BF16 im2col path only), bit 2
    // eight epilogue warps, bit 3 (above) the general kernel instead of the slab kernel; bits 0-2
    // zero = heuristic: one M tile, eight epilogue warps when every class
    // has at most 8 K blocks per tile (the epilogue, not the MMA, bounds such tiles)
    p.mt = ((aux_override & 3) == 2 && mode == 0 && p.im2col) ? 2 : 1;
    bool ew8 = (aux_override & 4) != 0;
    if ((aux_override & 7) == 0) {
        int kmax = 0;
        for (int c = 0; c < pl.ncls; c++) kmax = pl.cls[c].ktiles > kmax ? pl.cls[c].ktiles : kmax;
        ew8 = kmax <= 8;
    }
    p.ew = (ew8 && mode == 0 && p.im2col && (p.bn >= 128 || p.mt == 2) && !(p.bn == 256 && p.mt == 2)) ? 8 : 4;
    if (stats) {   // the statistics form: one M tile, four epilogue warps
        p.mt = 1;
        p.ew = 4;
    }
    // aux bit 4 (tuning): one K block per ring stage, twice the stages (BF16 im2col, one M tile,
    // four epilogue warps, 64 / 128-wide tiles)
    p.kb1 = (aux_override & 16) && mode == 0 && p.im2col && p.mt == 1 && p.ew == 4 && !stats && p.bn != 256;
    int t0 = 0, g0 = 0;
    if (f8w) p.mode = 3;   // MODE_FP8W: the classes count 128-channel K blocks
    for (int c = 0; c < pl.ncls; c++) {
        p.cls[c] = pi.cls[c];
        if (f8w) p.cls[c].ktiles /= 2;
        p.cls[c].tile0 = t0;
        p.cls[c].gbase = g0;   // statistics groups of 32 rows, classes concatenated
        t0 += (pl.cls[c].mtiles + p.mt - 1) / p.mt * p.ntiles;
        g0 += (int) (((long long) s.b * pl.cls[c].Hg * pl.cls[c].Wg + 31) / 32);
    }
    p.ntiles_total = t0;
    const int grid = t0 < sms ? t0 : sms;
    return cg_cuda_check(tc_conv_launch(p, wmap, omap, amaps, grid, st), "tensor-core conv launch");
}

// ------------------------------------------------------------ public API
convgemm_status_t tc_check_shape(const convgemm_shape_t *shape, const char *fn) {
    if (!shape) return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "%s: shape is NULL", fn);
    const convgemm_shape_t &s = *shape;
    if (s.b < 1 || s.h < 1 || s.w < 1 || s.c < 1 || s.kn < 1 || s.kh < 1 || s.kw < 1 || s.vstride < 1 ||
        s.hstride < 1 || s.vdil < 1 || s.hdil < 1 || s.vpad < 0 || s.hpad < 0)
        return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "%s: invalid geometry", fn);
    const long long ho = (s.h + 2LL * s.vpad - (long long) s.vdil * (s.kh - 1) - 1) / s.vstride + 1;
    const long long wo = (s.w + 2LL * s.hpad - (long long) s.hdil * (s.kw - 1) - 1) / s.hstride + 1;
    if (s.h + 2LL * s.vpad - (long long) s.vdil * (s.kh - 1) < 1 || s.w + 2LL * s.hpad - (long long) s.hdil * (s.kw - 1) < 1)
        return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "%s: the filter does not fit the padded input", fn);
    const long long lim = (1LL << 31) - 1;
    if ((long long) s.b * s.h * s.w * round_up(s.c, 8) > lim || (long long) s.b * ho * wo * round_up(s.kn, 8) > lim)
        return cg_set_error(CONVGEMM_ERROR_NOT_SUPPORTED, "%s: a tensor has more than 2^31-1 elements", fn);
    if (s.kh * s.kw > TC_MAXTAPS)
        return cg_set_error(CONVGEMM_ERROR_NOT_SUPPORTED, "%s: filters above 49 taps have no tensor-core kernel", fn);
    return CONVGEMM_SUCCESS;
}

extern "C" size_t convgemm_bf16_weights_size(const convgemm_shape_t *shape, int kind) {
    if (tc_check_shape(shape, "convgemm_bf16_weights_size")) return 0;
    const cg_shape s = cg_from_public(*shape);
    TcPlan pl;
    if (kind == CONVGEMM_OPERAND_FWD) {
        if (!tc_plan_fwd(s, pl)) return 0;
    } else if (kind == CONVGEMM_OPERAND_DGRAD) {
        if (!tc_plan_dgrad(s, pl)) return 0;
    } else {
        return 0;
    }
    return (size_t) pl.Cout * (size_t) (pl.Ktot > 0 ? pl.Ktot : 64) * 2;
}

extern "C" convgemm_status_t convgemm_bf16_pack_weights(convgemm_layout_t layout, const convgemm_shape_t *shape,
                                                        int kind, const float *weights, void *packed, void *stream) {
    if (convgemm_status_t e = tc_check_shape(shape, "convgemm_bf16_pack_weights")) return e;
    if (!weights || !packed) return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "convgemm_bf16_pack_weights: NULL");
    const cg_shape s = cg_from_public(*shape);
    const int nchw = layout == CONVGEMM_NCHW;
    TcPlan pl;
    cudaStream_t st = (cudaStream_t) stream;
    if (kind == CONVGEMM_OPERAND_FWD) {
        tc_plan_fwd(s, pl);
        return cg_cuda_check(prep_pack_fwd(weights, nchw, s.c, s.kh, s.kw, s.kn, pl.Cin, pl.Ktot, packed, st),
                             "pack weights");
    }
    if (kind == CONVGEMM_OPERAND_DGRAD) {
        if (!tc_plan_dgrad(s, pl))
            return cg_set_error(CONVGEMM_ERROR_NOT_SUPPORTED, "input gradient: more than 16 stride-phase classes");
        if (pl.Ktot == 0) return CONVGEMM_SUCCESS;
        return cg_cuda_check(prep_pack_dgrad(weights, nchw, s.c, s.kh, s.kw, s.kn, pl.Cin, tc_pack_info(pl), packed, st),
                             "pack weights");
    }
    return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "convgemm_bf16_pack_weights: bad kind %d", kind);
}

extern "C" convgemm_status_t convgemm_fold_epilogue(int kn, const convgemm_epilogue_t *epi, float *scale,
                                                    float *shift, void *stream) {
    if (kn < 1 || !scale || !shift) return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "convgemm_fold_epilogue: bad args");
    convgemm_epilogue_t e = {};
    if (epi) e = *epi;
    if (e.mean && !(e.inv_std && e.gamma && e.beta))
        return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "convgemm_fold_epilogue: batch-norm needs all parameters");
    return cg_cuda_check(prep_fold(kn, e.bias, e.mean, e.inv_std, e.gamma, e.beta, scale, shift, (cudaStream_t) stream),
                         "fold epilogue");
}

extern "C" convgemm_status_t convgemm_to_bf16_nhwc(convgemm_layout_t layout, int b, int c, int h, int w,
                                                   const float *in, void *out, void *stream) {
    if (b < 1 || c < 1 || h < 1 || w < 1 || !in || !out)
        return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "convgemm_to_bf16_nhwc: bad args");
    return cg_cuda_check(prep_to_bf16_nhwc(in, layout == CONVGEMM_NCHW, b, c, h, w, round_up(c, 8), out,
                                           (cudaStream_t) stream),
                         "cast to bf16");
}

extern "C" convgemm_status_t convgemm_fwd_bf16(const convgemm_shape_t *shape, const void *x, const void *wpacked,
                                               void *y, const float *scale, const float *shift, int relu,
                                               void *stream) {
    if (convgemm_status_t e = tc_check_shape(shape, "convgemm_fwd_bf16")) return e;
    if (!x || !wpacked || !y) return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "convgemm_fwd_bf16: NULL tensor");
    if (shape->kn % 8) return cg_set_error(CONVGEMM_ERROR_NOT_SUPPORTED, "convgemm_fwd_bf16: kn must be a multiple of 8");
    const cg_shape s = cg_from_public(*shape);
    TcPlan pl;
    tc_plan_fwd(s, pl);
    // c <= 8: MMA operands read straight from input slabs in shared memory
    if (tc_stem_applicable(s) && !((uintptr_t) y & 15) && !((uintptr_t) wpacked & 15) && !((uintptr_t) x & 15))
        return tc_stem_run(s, x, wpacked, pl.Ktot, y, scale, shift, relu, (cudaStream_t) stream);
    TcTune t{0, 0};
    tc_tune_get(CONVGEMM_TUNE_FWD, *shape, &t);
    return tc_run(pl, s, x, wpacked, y, scale, shift, relu, (cudaStream_t) stream, 0, nullptr, nullptr, t.bn,
                  t.splits);
}

namespace {

// dx = 0 where x <= 0, 8 BF16 values per thread (n8 groups of 8): applied before an accumulating,
// masked input gradient whose stride-phase classes do not reach every pixel, so that the pixels
// no tap reaches (which the kernel leaves alone) carry the mask too.
__global__ void relu_mask_bf16_kernel(uint4 *__restrict__ dx, const uint4 *__restrict__ x, size_t n8) {
    for (size_t i = blockIdx.x * (size_t) blockDim.x + threadIdx.x; i < n8; i += (size_t) gridDim.x * blockDim.x) {
        uint4 d = dx[i];
        const uint4 v = x[i];
        uint32_t *dw = &d.x;
        const uint32_t *xw = &v.x;
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const __nv_bfloat162 xv = *reinterpret_cast<const __nv_bfloat162 *>(&xw[j]);
            uint32_t keep = 0;
            if (__bfloat162float(xv.x) > 0.0f) keep |= 0x0000ffffu;
            if (__bfloat162float(xv.y) > 0.0f) keep |= 0xffff0000u;
            dw[j] &= keep;
        }
        dx[i] = d;
    }
}

convgemm_status_t dgrad_bf16(const convgemm_shape_t *shape, const void *dy, const void *wpacked, void *dx,
                             const void *mask, int accumulate, void *stream) {
    if (convgemm_status_t e = tc_check_shape(shape, "convgemm_dgrad_bf16")) return e;
    if (!dy || !wpacked || !dx) return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "convgemm_dgrad_bf16: NULL tensor");
    if (shape->c % 8) return cg_set_error(CONVGEMM_ERROR_NOT_SUPPORTED, "convgemm_dgrad_bf16: c must be a multiple of 8");
    const cg_shape s = cg_from_public(*shape);
    TcPlan pl;
    if (!tc_plan_dgrad(s, pl))
        return cg_set_error(CONVGEMM_ERROR_NOT_SUPPORTED, "input gradient: more than 16 stride-phase classes");
    cudaStream_t st = (cudaStream_t) stream;
    if (pl.has_empty_class && !accumulate) {
        // pixels no tap reaches receive zero (accumulating, they keep their value)
        if (convgemm_status_t e = cg_cuda_check(
                cudaMemsetAsync(dx, 0, sizeof(__nv_bfloat16) * (size_t) s.b * s.h * s.w * s.c, st), "zero dx"))
            return e;
    }
    TcTune t{0, 0};
    tc_tune_get(CONVGEMM_TUNE_DGRAD, *shape, &t);
    if (accumulate && ((uintptr_t) dx & 15))
        return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "convgemm_dgrad_bf16_ex: accumulating dx not 16-byte aligned");
    if (pl.has_empty_class && accumulate && mask) {
        // the pixels no tap reaches keep dx, masked like every other pixel
        const size_t n8 = (size_t) s.b * s.h * s.w * s.c / 8;
        const int blocks = (int) ((n8 + 255) / 256 < 4096 ? (n8 + 255) / 256 : 4096);
        relu_mask_bf16_kernel<<<blocks, 256, 0, st>>>((uint4 *) dx, (const uint4 *) mask, n8);
        cg_note_launch();
        if (convgemm_status_t e = cg_cuda_check(cudaGetLastError(), "relu mask of dx")) return e;
    }
    return tc_run(pl, s, dy, wpacked, dx, nullptr, nullptr, 0, st, 0, nullptr, nullptr, t.bn, t.splits, mask,
                  nullptr, accumulate != 0);
}

}  // namespace

extern "C" convgemm_status_t convgemm_dgrad_bf16(const convgemm_shape_t *shape, const void *dy, const void *wpacked,
                                                 void *dx, void *stream) {
    return dgrad_bf16(shape, dy, wpacked, dx, nullptr, 0, stream);
}

extern "C" convgemm_status_t convgemm_dgrad_bf16_relu(const convgemm_shape_t *shape, const void *dy,
                                                      const void *wpacked, void *dx, const void *x, void *stream) {
    if (!x || ((uintptr_t) x & 15))
        return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "convgemm_dgrad_bf16_relu: x NULL or not 16-byte aligned");
    return dgrad_bf16(shape, dy, wpacked, dx, x, 0, stream);
}

namespace {
long long dgrad_stat_groups(const TcPlan &pl, int b) {
    long long g = 0;
    for (int c = 0; c < pl.ncls; c++) g += ((long long) b * pl.cls[c].Hg * pl.cls[c].Wg + 31) / 32;
    return g;
}
}  // namespace

extern "C" size_t convgemm_dgrad_bf16_bias_grad_workspace_size(const convgemm_shape_t *shape) {
    if (tc_check_shape(shape, "convgemm_dgrad_bf16_bias_grad_workspace_size") || shape->c % 8) return 0;
    TcPlan pl;
    if (!tc_plan_dgrad(cg_from_public(*shape), pl)) return 0;
    return cg_colsum_ws_bytes(dgrad_stat_groups(pl, shape->b), shape->c);
}

extern "C" convgemm_status_t convgemm_dgrad_bf16_bias_grad(const convgemm_shape_t *shape, const void *dy,
                                                           const void *wpacked, void *dx, const void *relu_x,
                                                           float *db, void *workspace, size_t workspace_bytes,
                                                           void *stream) {
    const char *fn = "convgemm_dgrad_bf16_bias_grad";
    if (convgemm_status_t e = tc_check_shape(shape, fn)) return e;
    if (!dy || !wpacked || !dx || !db || !workspace)
        return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "%s: NULL argument", fn);
    if (shape->c % 8) return cg_set_error(CONVGEMM_ERROR_NOT_SUPPORTED, "%s: c must be a multiple of 8", fn);
    if (relu_x && ((uintptr_t) relu_x & 15))
        return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "%s: relu_x not 16-byte aligned", fn);
    const cg_shape s = cg_from_public(*shape);
    TcPlan pl;
    if (!tc_plan_dgrad(s, pl)) return cg_set_error(CONVGEMM_ERROR_NOT_SUPPORTED, "%s: more than 16 stride-phase classes", fn);
    const long long ng = dgrad_stat_groups(pl, s.b);
    const size_t need = cg_colsum_ws_bytes(ng, s.c);
    if (workspace_bytes < need || ((uintptr_t) workspace & 15))
        return cg_set_error(CONVGEMM_ERROR_WORKSPACE, "%s: workspace needs %zu bytes, 16-byte aligned", fn, need);
    cudaStream_t st = (cudaStream_t) stream;
    if (pl.has_empty_class)   // pixels no tap reaches: zero (and nothing to the sums)
        if (convgemm_status_t e = cg_cuda_check(
                cudaMemsetAsync(dx, 0, sizeof(__nv_bfloat16) * (size_t) s.b * s.h * s.w * s.c, st), "zero dx"))
            return e;
    TcTune t{0, 0};
    tc_tune_get(CONVGEMM_TUNE_DGRAD, *shape, &t);
    float *part = (float *) ((uint8_t *) workspace + cg_colsum_part_offset(ng, s.c));
    if (convgemm_status_t e = tc_run(pl, s, dy, wpacked, dx, nullptr, nullptr, 0, st, 0, nullptr, nullptr, t.bn,
                                     t.splits, relu_x, part, 0))
        return e;
    return cg_cuda_check(cg_colsum_reduce(workspace, (int) ng, s.c, db, st), "bias-gradient column sums");
}

extern "C" convgemm_status_t convgemm_dgrad_bf16_ex(const convgemm_shape_t *shape, const void *dy,
                                                    const void *wpacked, void *dx, const void *relu_x, int accumulate,
                                                    void *stream) {
    if (relu_x && ((uintptr_t) relu_x & 15))
        return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "convgemm_dgrad_bf16_ex: relu_x not 16-byte aligned");
    return dgrad_bf16(shape, dy, wpacked, dx, relu_x, accumulate, stream);
}

// ------------------------------------------------------- weight gradient
#include "tc_wgrad.h"

namespace {

struct WgPlan {
    int xa, bn, x2d, stem, mtiles, ntiles, splits, cps, nchunks, Nx, Cp, kn8;
    int csize, groups;   // grouped cluster reduction (groups > 1): splits = groups * csize
    int slab;            // the slab kernel (tc_wgrad_slab.cu) with `splits` partials
    int kb1;             // im2col path: one chunk per ring stage (twice the stages)
    int iss2;            // im2col path, two chunks per stage: two MMA-issuing warps
    int wide;            // im2col path: 128-pixel chunks (twice the bytes per TMA box), one per stage
    int pair;            // im2col path: CTA pairs, 256 x bn tiles (bn 128 / 256, mtiles even, wide chunks)
    int bk;              // pixels per chunk (64, or 128 when wide)
    size_t ws_bytes;
};

// Whether the weight gradient gathers X with im2col TMA (channels in 64-element atoms,
// padding and far-edge offsets within the im2col map's signed 8-bit corners).
bool wgrad_im2col_ok(const cg_shape &s, const ConvGeom &g) {
    const int up_h = -s.vpad + (g.ho - 1) * s.vstride - (s.h - 1), up_w = -s.hpad + (g.wo - 1) * s.hstride - (s.w - 1);
    return (round_up(s.c, 8) % 64) == 0 && s.vpad <= 128 && s.hpad <= 128 && up_h >= -128 && up_h <= 127 &&
           up_w >= -128 && up_w <= 127 && s.vstride <= 8 && s.hstride <= 8;
}

// Workspace of the one-cluster exchange of partial tiles: [tile][split][128 x bn] FP32.
size_t wgrad_xchg_bytes(const WgPlan &w) {
    return sizeof(float) * 128 * (size_t) w.bn * (size_t) w.mtiles * (size_t) w.ntiles * (size_t) w.splits;
}

WgPlan plan_wgrad(const convgemm_shape_t &ps) {
    const cg_shape s = cg_from_public(ps);
    const ConvGeom g = make_geom(s);
    TcTune t{0, 0};
    tc_tune_get(CONVGEMM_TUNE_WGRAD, ps, &t);
    WgPlan w;
    w.Cp = round_up(s.c, 8);
    w.kn8 = round_up(s.kn, 8);
    w.Nx = s.kh * s.kw * w.Cp;
    const bool im2col = wgrad_im2col_ok(s, g);
    const int aux_splits = t.splits & 0xffff;
    w.pair = im2col && (t.splits & CONVGEMM_WGRAD_PAIR) ? 1 : 0;
    w.wide = im2col && (w.pair || (t.splits & CONVGEMM_WGRAD_WIDE_CHUNKS)) ? 1 : 0;
    w.kb1 = im2col && !w.wide && (t.splits & CONVGEMM_WGRAD_STAGES1) ? 1 : 0;
    w.iss2 = im2col && !w.kb1 && !w.wide && (t.splits & CONVGEMM_WGRAD_TWO_ISSUERS) ? 1 : 0;
    w.bk = w.wide ? 128 : 64;
    // X on the A side: always for narrow layers, on request for wide ones (im2col path)
    const bool x_on_a = (t.splits & CONVGEMM_WGRAD_X_ON_A) && im2col;
    w.xa = s.kn < 128 || x_on_a;
    // X of a 1x1 stride-1 unpadded convolution is a plain [P][Cp] matrix: tiled boxes
    w.x2d = im2col && s.kh == 1 && s.kw == 1 && s.vstride == 1 && s.hstride == 1 && s.vpad == 0 && s.hpad == 0 &&
            !(t.splits & CONVGEMM_WGRAD_IM2COL_X);
    int Mext, Next;
    if (w.xa) {
        Mext = w.Nx;
        Next = s.kn;
        w.bn = s.kn <= 64 ? 64 : (s.kn >= 256 && x_on_a ? 256 : 128);
        if (t.bn == 64 || t.bn == 128 || (t.bn == 256 && x_on_a)) w.bn = t.bn;
    } else {
        Mext = s.kn;
        Next = w.Nx;
        w.bn = w.Nx >= 256 ? 256 : (w.Nx > 64 ? 128 : 64);
        if (t.bn) w.bn = t.bn;
    }
    if (w.pair) w.bn = t.bn == 128 ? 128 : 256;   // pair tiles: 256 x 128 or 256 x 256
    w.mtiles = (Mext + 127) / 128;
    if (w.pair) w.mtiles += w.mtiles & 1;   // the two CTAs of a pair take adjacent M tiles
    w.ntiles = (Next + w.bn - 1) / w.bn;
    w.nchunks = (int) ((g.P + w.bk - 1) / w.bk);
    const int base = w.mtiles * w.ntiles;
    const int per_sm = w.bn == 256 ? 1 : 2;
    int splits = tc_num_sms() * per_sm / base;   // one wave: no partial second wave
    const int max_splits = (int) ((g.P + 511) / 512);   // at least 512 pixels per split
    if (splits > max_splits) splits = max_splits;
    if (aux_splits) splits = aux_splits < w.nchunks ? aux_splits : w.nchunks;
    if (splits < 1) splits = 1;
    w.cps = (w.nchunks + splits - 1) / splits;
    w.splits = (w.nchunks + w.cps - 1) / w.cps;
    w.stem = tc_stem_wgrad_applicable(s);
    if (w.stem) {   // the slab kernel: one partial per CTA, tile settings do not apply
        w.bn = 64;
        w.splits = tc_stem_wgrad_splits(s);
    }
    // stride-1 layers with 128-channel input blocks: the slab kernel, by default (no tuning
    // entry) or when the tuning entry asks for it
    w.slab = 0;
    if (!w.stem && ((t.bn == 0 && t.splits == 0) || (t.splits & CONVGEMM_WGRAD_SLAB))) {
        const int sp = tc_wgrad_slab_splits(s, aux_splits, t.bn);
        if (sp > 0) {
            w.slab = 1;
            w.splits = sp;
            w.bn = tc_wgrad_slab_bn(s, t.bn);
            w.xa = 1;
        }
    }
    w.ws_bytes = sizeof(float) * (size_t) (w.splits + tc_wgrad_groups(w.splits)) * (size_t) w.Nx * (size_t) s.kn;
    w.csize = w.groups = 0;
    if (w.slab) return w;
    // 2..8 splits as one cluster exchange whole 128 x bn partial tiles through the workspace
    if (!w.stem && !w.pair && w.splits >= 2 && w.splits <= 8 && wgrad_xchg_bytes(w) > w.ws_bytes)
        w.ws_bytes = wgrad_xchg_bytes(w);
    // more splits than one cluster: clusters of up to 8 splits, reduced in the kernel (the
    // workspace is sized for the smallest cluster, so that it does not depend on the device)
    w.csize = w.groups = 0;
    if (!w.stem && !w.pair && w.splits > 8) {
        const size_t tile_bytes = sizeof(float) * 128 * (size_t) w.bn * (size_t) w.mtiles * (size_t) w.ntiles;
        const size_t grouped = tile_bytes * (size_t) ((w.splits + 1) / 2);
        if (grouped > w.ws_bytes) w.ws_bytes = grouped;
        const int code = (t.splits >> 20) & 3;   // CONVGEMM_WGRAD_GROUPS: 1, 2, 3 -> clusters of 2, 4, 8
        const int want = code ? 1 << code : 0;
        const int cs = want && cg_wgrad_cluster_enabled() && tc_wgrad_cluster_ok(w.bn, w.xa, im2col, want, w.kb1, w.iss2, w.wide) ? want : 0;
        if (cs) {
            w.csize = cs;
            w.groups = (w.splits + cs - 1) / cs;
            w.splits = w.groups * cs;
            w.cps = (w.nchunks + w.splits - 1) / w.splits;
            // a workspace that is not 16-byte aligned takes the reduction kernels at this split count
            const size_t planes =
                sizeof(float) * (size_t) (w.splits + tc_wgrad_groups(w.splits)) * (size_t) w.Nx * (size_t) s.kn;
            if (planes > w.ws_bytes) w.ws_bytes = planes;
        }
    }
    return w;
}

}  // namespace

extern "C" convgemm_status_t convgemm_wgrad_bf16_plan(const convgemm_shape_t *shape, int *bn, int *splits,
                                                      int *max_splits) {
    if (convgemm_status_t e = tc_check_shape(shape, "convgemm_wgrad_bf16_plan")) return e;
    const WgPlan w = plan_wgrad(*shape);
    if (bn) *bn = w.bn;
    if (splits) *splits = w.splits;
    if (max_splits) *max_splits = w.nchunks;
    return CONVGEMM_SUCCESS;
}

extern "C" size_t convgemm_wgrad_bf16_workspace_size(const convgemm_shape_t *shape) {
    if (tc_check_shape(shape, "convgemm_wgrad_bf16_workspace_size")) return 0;
    return plan_wgrad(*shape).ws_bytes;
}

extern "C" convgemm_status_t convgemm_wgrad_bf16(convgemm_layout_t layout, const convgemm_shape_t *shape,
                                                 const void *dy, const void *x, float *dw, void *workspace,
                                                 size_t workspace_bytes, void *stream) {
    if (convgemm_status_t e = tc_check_shape(shape, "convgemm_wgrad_bf16")) return e;
    if (!dy || !x || !dw || !workspace)
        return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "convgemm_wgrad_bf16: NULL tensor or workspace");
    if (layout != CONVGEMM_NHWC && layout != CONVGEMM_NCHW)
        return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "convgemm_wgrad_bf16: bad layout %d", (int) layout);
    const cg_shape s = cg_from_public(*shape);
    const ConvGeom g = make_geom(s);
    const WgPlan w = plan_wgrad(*shape);
    if (workspace_bytes < w.ws_bytes)
        return cg_set_error(CONVGEMM_ERROR_WORKSPACE, "convgemm_wgrad_bf16: workspace %zu bytes < %zu needed",
                            workspace_bytes, w.ws_bytes);
    if (w.stem)
        return tc_stem_wgrad_run(s, dy, x, (float *) workspace, dw, layout == CONVGEMM_NCHW, (cudaStream_t) stream);
    if (w.slab) {
        TcTune t{0, 0};
        tc_tune_get(CONVGEMM_TUNE_WGRAD, *shape, &t);
        return tc_wgrad_slab_run(s, t.splits & 0xffff, t.bn, dy, x, (float *) workspace, dw,
                                 layout == CONVGEMM_NCHW, (cudaStream_t) stream);
    }
    CUtensorMap map;
    if (convgemm_status_t e = tc_make_map_2d(&map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, dy, g.P, w.kn8, 64, w.bk))
        return e;
    TcWgradParams p;
    memset(&p, 0, sizeof(p));
    p.x = (const __nv_bfloat16 *) x;
    p.ws = (float *) workspace;
    p.B = s.b;
    p.H = s.h;
    p.W = s.w;
    p.Cp = w.Cp;
    p.kh = s.kh;
    p.kw = s.kw;
    p.kn = s.kn;
    p.Nx = w.Nx;
    p.P = (int) g.P;
    p.vstr = s.vstride;
    p.hstr = s.hstride;
    p.vpad = s.vpad;
    p.hpad = s.hpad;
    p.vdil = s.vdil;
    p.hdil = s.hdil;
    p.nchunks = w.nchunks;
    p.chunks_per_split = w.cps;
    p.dcp = FastDiv(w.Cp);
    p.dwo = FastDiv(g.wo);
    p.dho = FastDiv(g.ho);
    p.err = cg_device_error_word();
    if (!p.err) return cg_set_error(CONVGEMM_ERROR_CUDA, "device error word unavailable");
    CUtensorMap xmap;
    memset(&xmap, 0, sizeof(xmap));
    {
        const int up_h = -s.vpad + (g.ho - 1) * s.vstride - (s.h - 1), up_w = -s.hpad + (g.wo - 1) * s.hstride - (s.w - 1);
        p.im2col = wgrad_im2col_ok(s, g);
        p.x2d = w.x2d;
        if (p.x2d) {
            if (convgemm_status_t e = tc_make_map_2d(&xmap, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, x, g.P, p.Cp, 64, w.bk))
                return e;
        } else if (p.im2col) {
            if (convgemm_status_t e = tc_make_im2col_map(&xmap, x, s.b, s.h, s.w, p.Cp, -s.vpad, -s.hpad, up_h, up_w,
                                                         s.vstride, s.hstride, w.bk, 2, 64))
                return e;
        }
    }
    cudaStream_t st = (cudaStream_t) stream;
    // one split: the kernel writes dW itself
    p.dw = dw;
    p.direct = w.splits == 1;
    p.layout = layout == CONVGEMM_NCHW;
    p.C = s.c;
    p.kb1 = w.kb1;
    p.iss2 = w.iss2;
    p.wide = w.wide;
    p.pair = w.pair;
    if (w.pair) {
        p.cluster = 0;   // the cluster is the pair; several splits reduce through the workspace
    } else if (w.groups > 1 && !((uintptr_t) workspace & 15)) {
        // clusters of csize splits; the tile's last cluster adds the clusters' sums
        p.cluster = 1;
        p.groups = w.groups;
        p.csize = w.csize;
        p.gws = (float *) workspace;
        p.counters = tc_wgrad_counters(w.mtiles * w.ntiles * w.csize);
        if (!p.counters) return cg_set_error(CONVGEMM_ERROR_CUDA, "convgemm_wgrad_bf16: tile counters unavailable");
    } else {
        p.cluster = tc_wgrad_cluster_ok(w.bn, w.xa, p.im2col, w.splits, w.kb1, w.iss2, w.wide);
    }
    if ((p.direct || (p.cluster && p.groups <= 1)) && layout == CONVGEMM_NHWC && s.kn % 4 == 0 && w.Cp % 32 == 0 &&
        !((uintptr_t) dw & 15)) {
        // the kernel writes dW itself: [ci][tap][co] as (co, tap, ci), 32 x 1 x 32 FP32 boxes
        // (rows of 128 bytes, swizzled)
        const unsigned long long dims[3] = {(unsigned long long) s.kn, (unsigned long long) (s.kh * s.kw),
                                            (unsigned long long) s.c};
        const unsigned long long str[2] = {(unsigned long long) s.kn * 4, (unsigned long long) s.kn * s.kh * s.kw * 4};
        const unsigned box[3] = {32, 1, 32}, estr[3] = {1, 1, 1};
        if (convgemm_status_t e = tc_make_map_nd_dt(&p.dwmap, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, dw, dims, str, box, estr, 1))
            return e;
        p.dw_tma = 1;
        p.xchg = p.cluster && p.groups <= 1 && !((uintptr_t) workspace & 15) &&
                 workspace_bytes >= wgrad_xchg_bytes(w);
    }
    const int Mext = w.xa ? w.Nx : s.kn, Next = w.xa ? s.kn : w.Nx;
    if (!p.direct && !p.cluster && Next % 4 == 0 && !((uintptr_t) workspace & 15)) {
        // split partials [split][Mext][Next] written by TMA, clipped per split
        const unsigned long long dims[3] = {(unsigned long long) Next, (unsigned long long) Mext,
                                            (unsigned long long) w.splits};
        const unsigned long long str[2] = {(unsigned long long) Next * 4, (unsigned long long) Next * Mext * 4};
        const unsigned box[3] = {32, 32, 1}, estr[3] = {1, 1, 1};
        if (convgemm_status_t e =
                tc_make_map_nd_dt(&p.wsmap, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, workspace, dims, str, box, estr, 1))
            return e;
        p.ws_tma = 1;
    }
    if (convgemm_status_t e = cg_cuda_check(
            tc_wgrad_launch(p, map, xmap, w.bn, w.xa, w.mtiles, w.ntiles, w.splits, st), "weight-gradient launch"))
        return e;
    if (p.direct || p.cluster) return CONVGEMM_SUCCESS;
    return cg_cuda_check(tc_wgrad_reduce((float *) workspace, dw, w.splits, w.xa, w.Nx, s.kn, s.c, w.Cp, s.kh,
                                         s.kw, layout == CONVGEMM_NCHW, st),
                         "weight-gradient reduction");
}

// ---------------------------------------------------------- tuning report
// What the tuning table (or the heuristic) selects for one operation on one shape: the kernel
// (0 the general implicit GEMM, 1 a slab kernel, 2 the small-channel kernel), the tile width,
// the ring stages of the general kernels (slab and small-channel kernels size their buffers at
// run time: 0) and the cluster size (1, or the splits / cluster of a weight gradient).
extern "C" convgemm_status_t convgemm_tune_describe(int op, const convgemm_shape_t *shape, int *kernel, int *bn,
                                                    int *stages, int *cluster) {
    const char *fn = "convgemm_tune_describe";
    if (convgemm_status_t e = tc_check_shape(shape, fn)) return e;
    if (!kernel || !bn || !stages || !cluster) return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "%s: NULL output", fn);
    const cg_shape s = cg_from_public(*shape);
    TcTune t{0, 0};
    *kernel = 0;
    *bn = 0;
    *stages = 0;
    *cluster = 1;
    if (op == CONVGEMM_TUNE_WGRAD) {
        const WgPlan w = plan_wgrad(*shape);
        *bn = w.bn;
        if (w.stem || w.slab) {
            *kernel = w.stem ? 2 : 1;
            return CONVGEMM_SUCCESS;
        }
        const ConvGeom g = make_geom(s);
        const int im2col = wgrad_im2col_ok(s, g);
        *stages = tc_wgrad_stages(w.bn, im2col, w.kb1, w.wide, w.pair);
        if (w.pair) *cluster = 2;
        else if (w.groups > 1) *cluster = w.csize;
        else if (tc_wgrad_cluster_ok(w.bn, w.xa, im2col, w.splits, w.kb1, w.iss2, w.wide)) *cluster = w.splits;
        return CONVGEMM_SUCCESS;
    }
    if (op != CONVGEMM_TUNE_FWD && op != CONVGEMM_TUNE_DGRAD)
        return cg_set_error(CONVGEMM_ERROR_NOT_SUPPORTED, "%s: forward, input gradient or weight gradient only", fn);
    TcPlan pl;
    if (op == CONVGEMM_TUNE_FWD) {
        tc_plan_fwd(s, pl);
        if (tc_stem_applicable(s)) {
            *kernel = 2;
            *bn = s.kn;
            return CONVGEMM_SUCCESS;
        }
    } else if (!tc_plan_dgrad(s, pl)) {
        return cg_set_error(CONVGEMM_ERROR_NOT_SUPPORTED, "%s: more than 16 stride-phase classes", fn);
    }
    tc_tune_get(op, *shape, &t);
    if (!(t.splits & 8) && tc_slab_applicable(pl)) {
        *kernel = 1;
        *bn = 64;
        return CONVGEMM_SUCCESS;
    }
    TcPlan pi = pl;
    const int im2col = tc_plan_im2col(pi);
    *bn = t.bn ? t.bn : tc_pick_bn(pl, tc_num_sms());
    const int mt = ((t.splits & 3) == 2 && im2col) ? 2 : 1;
    bool ew8 = (t.splits & 4) != 0;
    if ((t.splits & 7) == 0) {
        int kmax = 0;
        for (int c = 0; c < pl.ncls; c++) kmax = pl.cls[c].ktiles > kmax ? pl.cls[c].ktiles : kmax;
        ew8 = kmax <= 8;
    }
    const int ew = (ew8 && im2col && (*bn >= 128 || mt == 2) && !(*bn == 256 && mt == 2)) ? 8 : 4;
    const int kb1 = (t.splits & 16) && im2col && mt == 1 && ew == 4 && *bn != 256;
    *stages = tc_conv_stages(*bn, im2col, mt, ew, kb1);
    return CONVGEMM_SUCCESS;
}

// ------------------------------------------------- grouped weight preparation
// The batch-norm folds and weight packings of many layers in one launch (a
// training step re-packs every layer's FP32 master weights): the host builds a
// job table once, the launch is capturable in a CUDA graph.

extern "C" size_t convgemm_prep_table_size(int n) {
    return n > 0 ? (size_t) 4 * n * (sizeof(PrepJob) + sizeof(int)) : 0;
}

extern "C" convgemm_status_t convgemm_prep_prepare(int n, const convgemm_prep_item_t *items, void *table,
                                                   size_t table_bytes, int *njobs, int *nblocks) {
    const char *fn = "convgemm_prep_prepare";
    if (n < 1 || !items || !table || !njobs || !nblocks)
        return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "%s: bad arguments", fn);
    if (table_bytes < convgemm_prep_table_size(n) || ((uintptr_t) table & 15))
        return cg_set_error(CONVGEMM_ERROR_WORKSPACE, "%s: table needs %zu bytes, 16-byte aligned", fn,
                            convgemm_prep_table_size(n));
    std::vector<PrepJob> jobs;
    long long blocks = 0;
    auto add = [&](PrepJob j, long long nb) {
        if (nb <= 0) return;
        j.block0 = (int) blocks;
        j.nblocks = (int) nb;
        jobs.push_back(j);
        blocks += nb;
    };
    for (int i = 0; i < n; i++) {
        const convgemm_prep_item_t &it = items[i];
        if (convgemm_status_t e = tc_check_shape(&it.shape, fn)) return e;
        if (it.layout != CONVGEMM_NHWC && it.layout != CONVGEMM_NCHW)
            return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "%s: item %d: bad layout", fn, i);
        if ((it.packed_fwd || it.packed_dgrad) && !it.weights)
            return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "%s: item %d: packing without weights", fn, i);
        if (!it.scale != !it.shift)
            return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "%s: item %d: scale and shift go together", fn, i);
        if (it.epi.mean && !(it.epi.inv_std && it.epi.gamma && it.epi.beta))
            return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "%s: item %d: batch-norm needs all parameters", fn, i);
        const cg_shape s = cg_from_public(it.shape);
        PrepJob j;
        memset(&j, 0, sizeof(j));
        j.nchw = it.layout == CONVGEMM_NCHW;
        j.C = s.c;
        j.kh = s.kh;
        j.kw = s.kw;
        j.kn = s.kn;
        j.w = it.weights;
        if (it.scale) {
            PrepJob f = j;
            f.type = PREP_FOLD;
            f.bias = it.epi.bias;
            f.mean = it.epi.mean;
            f.inv_std = it.epi.inv_std;
            f.gamma = it.epi.gamma;
            f.beta = it.epi.beta;
            f.scale = it.scale;
            f.shift = it.shift;
            add(f, (s.kn + 255) / 256);
        }
        if (it.packed_fwd) {
            TcPlan pl;
            tc_plan_fwd(s, pl);
            PrepJob f = j;
            f.Cp = pl.Cin;
            f.Kpad = pl.Ktot;
            f.out = it.packed_fwd;
            const int khw = s.kh * s.kw;
            if (j.nchw) {
                f.type = PREP_FWD_ELEM;
                add(f, (long long) s.kn * ((f.Kpad + 255) / 256));
            } else {
                f.type = PREP_FWD_TILED;
                add(f, (long long) khw * ((f.Cp + 63) / 64) * ((s.kn + 63) / 64));
                if (f.Kpad > khw * f.Cp) {
                    if ((long long) s.kn * (f.Kpad - khw * f.Cp) > (1LL << 31) - 256)
                        return cg_set_error(CONVGEMM_ERROR_NOT_SUPPORTED, "%s: item %d: weights too large", fn, i);
                    f.type = PREP_FWD_TAIL;
                    add(f, ((long long) s.kn * (f.Kpad - khw * f.Cp) + 255) / 256);
                }
            }
        }
        if (it.packed_dgrad) {
            TcPlan pl;
            if (!tc_plan_dgrad(s, pl))
                return cg_set_error(CONVGEMM_ERROR_NOT_SUPPORTED, "%s: item %d: more than 16 stride-phase classes", fn, i);
            if (pl.Ktot > 0) {
                PrepJob f = j;
                f.type = PREP_DGRAD;
                f.knp = pl.Cin;
                f.info = tc_pack_info(pl);
                f.dknp = FastDiv((uint32_t) f.knp);
                f.out = it.packed_dgrad;
                add(f, (long long) ((s.c + 3) / 4) * f.info.ncls);
            }
        }
        if (blocks > (1LL << 31) - 1) return cg_set_error(CONVGEMM_ERROR_NOT_SUPPORTED, "%s: too many blocks", fn);
    }
    if (jobs.empty()) return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "%s: nothing to prepare", fn);
    if (jobs.size() > 12288) return cg_set_error(CONVGEMM_ERROR_NOT_SUPPORTED, "%s: more than 12288 jobs", fn);
    *njobs = (int) jobs.size();
    *nblocks = (int) blocks;
    // [jobs][block0 of each job]
    std::vector<uint8_t> bytes(sizeof(PrepJob) * jobs.size() + sizeof(int) * jobs.size());
    memcpy(bytes.data(), jobs.data(), sizeof(PrepJob) * jobs.size());
    for (size_t j = 0; j < jobs.size(); j++)
        memcpy(bytes.data() + sizeof(PrepJob) * jobs.size() + sizeof(int) * j, &jobs[j].block0, sizeof(int));
    return cg_cuda_check(cudaMemcpy(table, bytes.data(), bytes.size(), cudaMemcpyHostToDevice),
                         "copy preparation table");
}

extern "C" convgemm_status_t convgemm_prep_launch(const void *table, int njobs, int nblocks, void *stream) {
    if (!table || njobs < 1 || nblocks < 1)
        return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "convgemm_prep_launch: bad arguments");
    return cg_cuda_check(prep_group_launch((const PrepJob *) table, njobs, nblocks, (cudaStream_t) stream),
                         "grouped preparation launch");
}

// ------------------------------------------------------------ bias gradient
extern "C" size_t convgemm_bias_grad_bf16_workspace_size(const convgemm_shape_t *shape) {
    if (tc_check_shape(shape, "convgemm_bias_grad_bf16_workspace_size")) return 0;
    const ConvGeom g = make_geom(cg_from_public(*shape));
    return sizeof(float) * (size_t) tc_bias_grad_groups(g.P) * shape->kn;
}

extern "C" convgemm_status_t convgemm_bias_grad_bf16(const convgemm_shape_t *shape, const void *dy, float *db,
                                                     void *workspace, size_t workspace_bytes, void *stream) {
    const char *fn = "convgemm_bias_grad_bf16";
    if (convgemm_status_t e = tc_check_shape(shape, fn)) return e;
    if (!dy || !db || !workspace) return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "%s: NULL argument", fn);
    const size_t need = convgemm_bias_grad_bf16_workspace_size(shape);
    if (workspace_bytes < need)
        return cg_set_error(CONVGEMM_ERROR_WORKSPACE, "%s: workspace %zu bytes < %zu needed", fn, workspace_bytes, need);
    const ConvGeom g = make_geom(cg_from_public(*shape));
    if (g.P > (1LL << 31) - 1) return cg_set_error(CONVGEMM_ERROR_NOT_SUPPORTED, "%s: too many pixels", fn);
    return cg_cuda_check(tc_bias_grad(dy, g.P, shape->kn, round_up(shape->kn, 8), db, (float *) workspace,
                                      (cudaStream_t) stream),
                         fn);
}

