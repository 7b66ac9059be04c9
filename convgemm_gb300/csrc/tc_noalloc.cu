// Weight gradient (BF16 tensor cores) that allocates nothing.
//
// convgemm_wgrad_bf16 needs a caller workspace for its FP32 split partials.
// Some callers cannot provide one: code that runs while a stream is being
// captured into a CUDA graph (cudaMalloc is not permitted during a capture), and
// services that fix their GPU memory footprint at start-up so that nothing can
// fail or fragment mid-run.  This entry point keeps the partials in a file-scope
// device array of fixed size instead, so it calls no cudaMalloc/cudaFree and no
// allocating routine.
//
// Limits and sharing:
//   * the scratch holds CONVGEMM_NOALLOC_SCRATCH_FLOATS FP32 values (16 MiB);
//     the number of pixel splits is capped so the partials (and the group sums
//     of the two-pass reduction) fit, and a layer
//     whose single partial tile (Nx*kn, Nx = kh*kw*c8) does not fit is
//     rejected with CONVGEMM_ERROR_NOT_SUPPORTED;
//   * every GPU that loads the library holds the 16 MiB until the process exits;
//   * all calls share the one array: calls that overlap on the GPU (different
//     streams without ordering) race on it.  The array keeps the last call's
//     partials; nothing in it needs to start at zero, because every element a
//     call reads back was written by that call's kernel first.
//   * a device-side wait that runs out is recorded in the library's device
//     error word, like every other kernel's, and reported by convgemm_check_device;
//   * the first call on a device looks up the array's device address
//     (cudaGetSymbolAddress) and sets kernel attributes; make that first call
//     before any stream capture.
#include <cstring>
#include <mutex>

#include "../../include/convgemm_gpu.h"
#include "cg_common.cuh"
#include "tc_host.h"
#include "tc_wgrad.h"

#define CONVGEMM_NOALLOC_SCRATCH_FLOATS (4u << 20)

namespace {

static __device__ __align__(256) float g_wgrad_scratch[CONVGEMM_NOALLOC_SCRATCH_FLOATS];

struct NoallocDevice {
    float *scratch = nullptr;
    int *err = nullptr;   // the library's device error word (convgemm_check_device reads it)
    bool ready = false;
};
std::mutex g_noalloc_mu;
NoallocDevice g_noalloc_dev[64];

// Device addresses of the file-scope arrays on the current device (host code
// cannot use the arrays' names as addresses).
convgemm_status_t noalloc_setup(NoallocDevice **out) {
    int dev = 0;
    if (convgemm_status_t e = cg_cuda_check(cudaGetDevice(&dev), "cudaGetDevice")) return e;
    if (dev < 0 || dev >= 64) return cg_set_error(CONVGEMM_ERROR_NOT_SUPPORTED, "device index %d out of range", dev);
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    NoallocDevice &d = g_noalloc_dev[dev];
    if (!d.ready) {
        void *p = nullptr;
        if (convgemm_status_t e = cg_cuda_check(cudaGetSymbolAddress(&p, g_wgrad_scratch), "cudaGetSymbolAddress"))
            return e;
        int *w = cg_device_error_word();
        if (!w) return cg_set_error(CONVGEMM_ERROR_CUDA, "device error word unavailable");
        d.scratch = (float *) p;
        d.err = w;
        d.ready = true;
    }
    *out = &d;
    return CONVGEMM_SUCCESS;
}

inline int rup(int v, int m) { return (v + m - 1) / m * m; }

}  // namespace

extern "C" convgemm_status_t convgemm_wgrad_bf16_noalloc(convgemm_layout_t layout, const convgemm_shape_t *shape,
                                                         const void *dy, const void *x, float *dw, void *stream) {
    const char *fn = "convgemm_wgrad_bf16_noalloc";
    if (!shape || !dy || !x || !dw) return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "%s: NULL argument", fn);
    if (layout != CONVGEMM_NHWC && layout != CONVGEMM_NCHW)
        return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "%s: bad layout %d", fn, (int) layout);
    // the geometry, size and filter-size checks of the workspace form
    if (convgemm_status_t e = tc_check_shape(shape, fn)) return e;
    const cg_shape s = cg_from_public(*shape);
    const ConvGeom g = make_geom(s);
    const int Cp = rup(s.c, 8), kn8 = rup(s.kn, 8), Nx = s.kh * s.kw * Cp;
    const long long tile = (long long) Nx * s.kn;
    if (tile > (long long) CONVGEMM_NOALLOC_SCRATCH_FLOATS)
        return cg_set_error(CONVGEMM_ERROR_NOT_SUPPORTED,
                            "%s: kh*kw*c8*kn = %lld FP32 partials exceed the fixed scratch of %u (16 MiB); "
                            "use convgemm_wgrad_bf16 with a workspace",
                            fn, tile, CONVGEMM_NOALLOC_SCRATCH_FLOATS);
    NoallocDevice *d = nullptr;
    if (convgemm_status_t e = noalloc_setup(&d)) return e;

    // the same tiling as the workspace form, with the pixel splits capped by the scratch
    const int xa = s.kn < 128;
    const int Mext = xa ? Nx : s.kn, Next = xa ? s.kn : Nx;
    const int bn = xa ? (s.kn <= 64 ? 64 : 128) : (Nx >= 256 ? 256 : (Nx > 64 ? 128 : 64));
    const int mtiles = (Mext + 127) / 128, ntiles = (Next + bn - 1) / bn;
    const int nchunks = (int) ((g.P + 63) / 64);
    const int base = mtiles * ntiles;
    // the workspace form's default: one wave of CTAs (no partial second wave), at least 8
    // chunks (512 pixels) per split
    int splits = tc_num_sms() * (bn == 256 ? 1 : 2) / base;
    splits = splits > (nchunks + 7) / 8 ? (nchunks + 7) / 8 : splits;
    const int fit = (int) ((long long) CONVGEMM_NOALLOC_SCRATCH_FLOATS / tile);
    if (splits > fit) splits = fit;
    if (splits < 1) splits = 1;
    int cps = (nchunks + splits - 1) / splits;
    splits = (nchunks + cps - 1) / cps;
    // the reduction's group planes follow the split planes in the scratch
    while (splits > 1 && (long long) (splits + tc_wgrad_groups(splits)) * tile > (long long) CONVGEMM_NOALLOC_SCRATCH_FLOATS) {
        splits--;
        cps = (nchunks + splits - 1) / splits;
        splits = (nchunks + cps - 1) / cps;
    }

    CUtensorMap map;
    if (convgemm_status_t e = tc_make_map_2d(&map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, dy, g.P, kn8, 64, 64)) return e;
    TcWgradParams p;
    memset(&p, 0, sizeof(p));
    p.x = (const __nv_bfloat16 *) x;
    p.ws = d->scratch;
    p.B = s.b;
    p.H = s.h;
    p.W = s.w;
    p.Cp = Cp;
    p.kh = s.kh;
    p.kw = s.kw;
    p.kn = s.kn;
    p.Nx = Nx;
    p.P = (int) g.P;
    p.vstr = s.vstride;
    p.hstr = s.hstride;
    p.vpad = s.vpad;
    p.hpad = s.hpad;
    p.vdil = s.vdil;
    p.hdil = s.hdil;
    p.nchunks = nchunks;
    p.chunks_per_split = cps;
    p.dcp = FastDiv(Cp);
    p.dwo = FastDiv(g.wo);
    p.dho = FastDiv(g.ho);
    p.err = d->err;
    CUtensorMap xmap;
    memset(&xmap, 0, sizeof(xmap));
    {
        const int up_h = -s.vpad + (g.ho - 1) * s.vstride - (s.h - 1), up_w = -s.hpad + (g.wo - 1) * s.hstride - (s.w - 1);
        p.im2col = (p.Cp % 64) == 0 && s.vpad <= 128 && s.hpad <= 128 && up_h >= -128 && up_h <= 127 && up_w >= -128 &&
                   up_w <= 127 && s.vstride <= 8 && s.hstride <= 8;
        if (p.im2col)
            if (convgemm_status_t e = tc_make_im2col_map(&xmap, x, s.b, s.h, s.w, p.Cp, -s.vpad, -s.hpad, up_h, up_w,
                                                         s.vstride, s.hstride, 64, 2))
                return e;
    }
    cudaStream_t st = (cudaStream_t) stream;
    p.dw = dw;
    p.direct = splits == 1;
    p.layout = layout == CONVGEMM_NCHW;
    p.C = s.c;
    p.cluster = tc_wgrad_cluster_ok(bn, xa, p.im2col, splits);
    if (convgemm_status_t e =
            cg_cuda_check(tc_wgrad_launch(p, map, xmap, bn, xa, mtiles, ntiles, splits, st), "weight-gradient launch"))
        return e;
    if (p.direct || p.cluster) return CONVGEMM_SUCCESS;
    return cg_cuda_check(
        tc_wgrad_reduce(d->scratch, dw, splits, xa, Nx, s.kn, s.c, Cp, s.kh, s.kw, layout == CONVGEMM_NCHW, st),
        "weight-gradient reduction");
}
