// Host runtime of the library: the C ABI of convGemm.h and convgemm_gpu.h,
// argument checks, error reporting, host-pointer staging and the cached
// device buffers the void drop-in entry points need.
#include <atomic>
#include <cstdlib>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include "../../include/convGemm.h"
#include "../../include/convgemm_gpu.h"
#include "cg_common.cuh"

// ------------------------------------------------------------------ errors
namespace {
thread_local convgemm_status_t tl_status = CONVGEMM_SUCCESS;
thread_local char tl_msg[512] = "";
}  // namespace

convgemm_status_t cg_set_error(convgemm_status_t st, const char *fmt, ...) {
    tl_status = st;
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(tl_msg, sizeof(tl_msg), fmt, ap);
    va_end(ap);
    return st;
}

convgemm_status_t cg_cuda_check(cudaError_t e, const char *what) {
    if (e == cudaSuccess) return CONVGEMM_SUCCESS;
    return cg_set_error(e == cudaErrorMemoryAllocation ? CONVGEMM_ERROR_ALLOC : CONVGEMM_ERROR_CUDA,
                        "%s: %s", what, cudaGetErrorString(e));
}

// Programmatic dependent launch for the persistent chain kernels: per host thread,
// default on unless the environment sets CONVGEMM_NO_PDL=1.
static thread_local int tl_pdl = -1;
bool cg_pdl_env_enabled() {
    static const bool env_on = [] {
        const char *e = getenv("CONVGEMM_NO_PDL");
        return !(e && e[0] == '1');
    }();
    return env_on;
}
bool cg_pdl_enabled() { return tl_pdl < 0 ? cg_pdl_env_enabled() : tl_pdl != 0; }
extern "C" int convgemm_set_pdl(int on) {
    const int prev = cg_pdl_enabled() ? 1 : 0;
    tl_pdl = on < 0 ? -1 : (on != 0);
    return prev;
}

bool cg_wgrad_cluster_enabled() {
    static const bool on = [] {
        const char *e = getenv("CONVGEMM_NO_WGRAD_CLUSTER");
        return !(e && e[0] == '1');
    }();
    return on;
}

static std::atomic<unsigned long long> g_launches{0};
void cg_note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
extern "C" unsigned long long convgemm_launch_count(void) { return g_launches.load(std::memory_order_relaxed); }

extern "C" convgemm_status_t convgemm_get_last_status(void) { return tl_status; }
extern "C" const char *convgemm_get_last_error(void) { return tl_msg; }
extern "C" void convgemm_clear_error(void) {
    tl_status = CONVGEMM_SUCCESS;
    tl_msg[0] = 0;
}

// ------------------------------------------------------- device error word
// One word per device for every kernel of the library: a file-scope device
// variable (zero when the module loads), so that no entry point allocates for it.
// Host code cannot use the variable's name as a device address; its address on
// the current device comes from cudaGetSymbolAddress, once per device.
namespace {
__device__ int g_dev_error_word;
std::mutex g_err_mu;
int *g_err_word[64] = {nullptr};
}  // namespace

int *cg_device_error_word() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
    std::lock_guard<std::mutex> lk(g_err_mu);
    if (!g_err_word[dev]) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_dev_error_word) != cudaSuccess) return nullptr;
        g_err_word[dev] = (int *) p;
    }
    return g_err_word[dev];
}

extern "C" convgemm_status_t convgemm_check_device(void *stream) {
    cudaStream_t st = (cudaStream_t) stream;
    if (convgemm_status_t s = cg_cuda_check(cudaStreamSynchronize(st), "cudaStreamSynchronize")) return s;
    int *w = cg_device_error_word();
    if (!w) return cg_set_error(CONVGEMM_ERROR_CUDA, "device error word unavailable");
    int v = 0;
    if (convgemm_status_t s = cg_cuda_check(cudaMemcpy(&v, w, sizeof(int), cudaMemcpyDeviceToHost), "read error word"))
        return s;
    if (v != 0) {
        cudaMemset(w, 0, sizeof(int));
        return cg_set_error(CONVGEMM_ERROR_TIMEOUT, "a device-side wait ran out (code %d)", v);
    }
    return CONVGEMM_SUCCESS;
}

// -------------------------------------------------------- argument checks
namespace {

convgemm_status_t check_shape(const convgemm_shape_t *s, const char *fn) {
    if (!s) return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "%s: shape is NULL", fn);
    if (s->b < 1 || s->h < 1 || s->w < 1 || s->c < 1 || s->kn < 1 || s->kh < 1 || s->kw < 1)
        return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "%s: sizes must be >= 1 (b=%d h=%d w=%d c=%d kn=%d kh=%d kw=%d)",
                            fn, s->b, s->h, s->w, s->c, s->kn, s->kh, s->kw);
    if (s->vstride < 1 || s->hstride < 1 || s->vdil < 1 || s->hdil < 1 || s->vpad < 0 || s->hpad < 0)
        return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE,
                            "%s: strides and dilations must be >= 1 and paddings >= 0", fn);
    const long long eh = (long long) s->h + 2LL * s->vpad - (long long) s->vdil * (s->kh - 1);
    const long long ew = (long long) s->w + 2LL * s->hpad - (long long) s->hdil * (s->kw - 1);
    if (eh < 1 || ew < 1)
        return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "%s: the filter does not fit the padded input", fn);
    const long long ho = (eh - 1) / s->vstride + 1, wo = (ew - 1) / s->hstride + 1;
    const long long lim = (1LL << 31) - 1;
    if ((long long) s->b * s->h * s->w * s->c > lim || (long long) s->b * ho * wo * s->kn > lim ||
        (long long) s->c * s->kh * s->kw * s->kn > lim || (long long) s->b * ho * wo > lim)
        return cg_set_error(CONVGEMM_ERROR_NOT_SUPPORTED, "%s: a tensor has more than 2^31-1 elements", fn);
    return CONVGEMM_SUCCESS;
}

convgemm_status_t check_epi(const convgemm_epilogue_t *e, const char *fn) {
    if (e && e->mean && !(e->inv_std && e->gamma && e->beta))
        return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE,
                            "%s: batch-norm needs mean, inv_std, gamma and beta", fn);
    return CONVGEMM_SUCCESS;
}

cg_epi to_epi(const convgemm_epilogue_t *e) {
    cg_epi r = {nullptr, nullptr, nullptr, nullptr, nullptr, 0};
    if (e) r = cg_epi{e->bias, e->mean, e->inv_std, e->gamma, e->beta, e->relu};
    return r;
}

long long out_elems(const convgemm_shape_t &s) {
    long long ho = (s.h + 2LL * s.vpad - (long long) s.vdil * (s.kh - 1) - 1) / s.vstride + 1;
    long long wo = (s.w + 2LL * s.hpad - (long long) s.hdil * (s.kw - 1) - 1) / s.hstride + 1;
    return (long long) s.b * ho * wo * s.kn;
}

}  // namespace

// ------------------------------------------------------- FP32 extended API
extern "C" convgemm_status_t convgemm_fwd_f32(convgemm_layout_t layout, const convgemm_shape_t *shape,
                                              const float *weights, const float *x, float *y,
                                              const convgemm_epilogue_t *epi, void *stream) {
    if (convgemm_status_t s = check_shape(shape, "convgemm_fwd_f32")) return s;
    if (convgemm_status_t s = check_epi(epi, "convgemm_fwd_f32")) return s;
    if (!weights || !x || !y) return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "convgemm_fwd_f32: NULL tensor");
    if (layout != CONVGEMM_NHWC && layout != CONVGEMM_NCHW)
        return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "convgemm_fwd_f32: bad layout %d", (int) layout);
    return cg_cuda_check(cg_fp32_fwd(layout == CONVGEMM_NCHW, cg_from_public(*shape), weights, x, y, to_epi(epi),
                                     (cudaStream_t) stream),
                         "convgemm_fwd_f32 launch");
}

extern "C" size_t convgemm_wgrad_f32_workspace_size(const convgemm_shape_t *shape) {
    if (check_shape(shape, "convgemm_wgrad_f32_workspace_size")) return 0;
    return cg_fp32_wgrad_ws_bytes(cg_from_public(*shape));
}

extern "C" convgemm_status_t convgemm_wgrad_f32(convgemm_layout_t layout, const convgemm_shape_t *shape,
                                                const float *dy, const float *x, float *dw, void *workspace,
                                                size_t workspace_bytes, void *stream) {
    if (convgemm_status_t s = check_shape(shape, "convgemm_wgrad_f32")) return s;
    if (!dy || !x || !dw || !workspace)
        return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "convgemm_wgrad_f32: NULL tensor or workspace");
    if (layout != CONVGEMM_NHWC && layout != CONVGEMM_NCHW)
        return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "convgemm_wgrad_f32: bad layout %d", (int) layout);
    const size_t need = cg_fp32_wgrad_ws_bytes(cg_from_public(*shape));
    if (workspace_bytes < need)
        return cg_set_error(CONVGEMM_ERROR_WORKSPACE, "convgemm_wgrad_f32: workspace %zu bytes < %zu needed",
                            workspace_bytes, need);
    return cg_cuda_check(cg_fp32_wgrad(layout == CONVGEMM_NCHW, cg_from_public(*shape), dy, x, dw, (float *) workspace,
                                       (cudaStream_t) stream),
                         "convgemm_wgrad_f32 launch");
}

extern "C" convgemm_status_t convgemm_dgrad_f32(convgemm_layout_t layout, const convgemm_shape_t *shape,
                                                const float *weights, const float *dy, float *dx, int accumulate,
                                                void *stream) {
    if (convgemm_status_t s = check_shape(shape, "convgemm_dgrad_f32")) return s;
    if (!weights || !dy || !dx) return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "convgemm_dgrad_f32: NULL tensor");
    if (layout != CONVGEMM_NHWC && layout != CONVGEMM_NCHW)
        return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "convgemm_dgrad_f32: bad layout %d", (int) layout);
    return cg_cuda_check(cg_fp32_dgrad(layout == CONVGEMM_NCHW, cg_from_public(*shape), weights, dy, dx, accumulate,
                                       (cudaStream_t) stream),
                         "convgemm_dgrad_f32 launch");
}

// ----------------------------------------------------------- drop-in ABI
namespace {

std::mutex g_dropin_mu;  // the drop-in entry points share staging buffers

// Grow-only device buffers, one per purpose, on the current device.
struct Slot {
    void *p = nullptr;
    size_t bytes = 0;
    int dev = -1;
};
enum { SLOT_IN, SLOT_X, SLOT_OUT, SLOT_BIAS, SLOT_MEAN, SLOT_ISTD, SLOT_GAMMA, SLOT_BETA, SLOT_WS, NSLOTS };
Slot g_slots[NSLOTS];

void *slot_get(int i, size_t bytes) {
    int dev = 0;
    cudaGetDevice(&dev);
    Slot &s = g_slots[i];
    if (s.p && s.dev == dev && s.bytes >= bytes) return s.p;
    if (s.p) {
        int cur = dev;
        cudaSetDevice(s.dev);
        cudaFree(s.p);
        cudaSetDevice(cur);
        s.p = nullptr;
        s.bytes = 0;
    }
    if (cudaMalloc(&s.p, bytes ? bytes : 16) != cudaSuccess) {
        s.p = nullptr;
        return nullptr;
    }
    s.bytes = bytes;
    s.dev = dev;
    return s.p;
}

bool is_device_ptr(const void *p) {
    if (!p) return true;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// A tensor argument of a drop-in call: the caller's pointer, and the device
// pointer the kernels use (a staging buffer when the caller's is host memory).
struct Arg {
    const void *user;
    void *dev;
    size_t bytes;
    bool staged;
};

bool stage_in(Arg &a, int slot, bool copy) {
    a.staged = false;
    a.dev = const_cast<void *>(a.user);
    if (!a.user || is_device_ptr(a.user)) return true;
    a.dev = slot_get(slot, a.bytes);
    if (!a.dev) {
        cg_set_error(CONVGEMM_ERROR_ALLOC, "cannot allocate %zu bytes of device staging memory", a.bytes);
        return false;
    }
    a.staged = true;
    if (copy) {
        cudaError_t e = cudaMemcpy(a.dev, a.user, a.bytes, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            cg_cuda_check(e, "host-to-device staging copy");
            return false;
        }
    }
    return true;
}

bool stage_out(const Arg &a) {
    if (!a.staged) return true;
    cudaError_t e = cudaMemcpy(const_cast<void *>(a.user), a.dev, a.bytes, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
        cg_cuda_check(e, "device-to-host staging copy");
        return false;
    }
    return true;
}

convgemm_shape_t mkshape(int b, int h, int w, int c, int kn, int kh, int kw, int vpad, int hpad, int vstr, int hstr,
                         int vdil, int hdil) {
    convgemm_shape_t s = {b, h, w, c, kn, kh, kw, vpad, hpad, vstr, hstr, vdil, hdil};
    return s;
}

void dropin_conv(int nchw, char trans, const convgemm_shape_t &s, const float *in, const float *x, float *out,
                 const float *bias, const float *mean, const float *inv_std, const float *gamma, const float *beta,
                 bool relu) {
    const char *fn = nchw ? "sconvGemmNCHW" : "sconvGemmNHWC";
    if (check_shape(&s, fn)) return;
    if (!in || !x || !out) {
        cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "%s: NULL tensor", fn);
        return;
    }
    std::lock_guard<std::mutex> lk(g_dropin_mu);
    const size_t K = (size_t) s.c * s.kh * s.kw;
    const size_t xb = sizeof(float) * (size_t) s.b * s.h * s.w * s.c;
    const size_t yb = sizeof(float) * (size_t) out_elems(s);
    const size_t wb = sizeof(float) * K * s.kn;
    const bool fwd = trans == 'N';
    Arg a_in{in, nullptr, fwd ? wb : yb, false};
    Arg a_x{x, nullptr, xb, false};
    Arg a_out{out, nullptr, fwd ? yb : wb, false};
    if (!stage_in(a_in, SLOT_IN, true) || !stage_in(a_x, SLOT_X, true) || !stage_in(a_out, SLOT_OUT, false)) return;
    if (fwd) {
        if (mean && !(inv_std && gamma && beta)) {
            cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "%s: batch-norm needs mean, inv_std, gamma and beta", fn);
            return;
        }
        const size_t pb = sizeof(float) * s.kn;
        Arg p[5] = {{bias, nullptr, pb, false}, {mean, nullptr, pb, false}, {inv_std, nullptr, pb, false},
                    {gamma, nullptr, pb, false}, {beta, nullptr, pb, false}};
        for (int i = 0; i < 5; i++)
            if (!stage_in(p[i], SLOT_BIAS + i, true)) return;
        cg_epi e = {(const float *) p[0].dev, (const float *) p[1].dev, (const float *) p[2].dev,
                    (const float *) p[3].dev, (const float *) p[4].dev, relu ? 1 : 0};
        if (cg_cuda_check(cg_fp32_fwd(nchw, cg_from_public(s), (const float *) a_in.dev, (const float *) a_x.dev,
                                      (float *) a_out.dev, e, 0),
                          fn))
            return;
    } else {
        const size_t wsb = cg_fp32_wgrad_ws_bytes(cg_from_public(s));
        void *ws = slot_get(SLOT_WS, wsb);
        if (!ws) {
            cg_set_error(CONVGEMM_ERROR_ALLOC, "%s: cannot allocate %zu bytes of workspace", fn, wsb);
            return;
        }
        if (cg_cuda_check(cg_fp32_wgrad(nchw, cg_from_public(s), (const float *) a_in.dev, (const float *) a_x.dev,
                                        (float *) a_out.dev, (float *) ws, 0),
                          fn))
            return;
    }
    if (a_out.staged) stage_out(a_out);
}

void dropin_back(int nchw, const convgemm_shape_t &s, const float *weights, const float *dy, float *dx) {
    const char *fn = nchw ? "sconvGemmNCHW_back" : "sconvGemmNHWC_back";
    if (check_shape(&s, fn)) return;
    if (!weights || !dy || !dx) {
        cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "%s: NULL tensor", fn);
        return;
    }
    std::lock_guard<std::mutex> lk(g_dropin_mu);
    const size_t K = (size_t) s.c * s.kh * s.kw;
    Arg a_w{weights, nullptr, sizeof(float) * K * s.kn, false};
    Arg a_dy{dy, nullptr, sizeof(float) * (size_t) out_elems(s), false};
    Arg a_dx{dx, nullptr, sizeof(float) * (size_t) s.b * s.h * s.w * s.c, false};
    // dx is accumulated into, so its old contents go to the device too
    if (!stage_in(a_w, SLOT_IN, true) || !stage_in(a_dy, SLOT_X, true) || !stage_in(a_dx, SLOT_OUT, true)) return;
    if (cg_cuda_check(cg_fp32_dgrad(nchw, cg_from_public(s), (const float *) a_w.dev, (const float *) a_dy.dev,
                                    (float *) a_dx.dev, 1, 0),
                      fn))
        return;
    if (a_dx.staged) stage_out(a_dx);
}

}  // namespace

// ------------------------------------------- explicit lowering helpers (drop-in)
// The reference's im2row_nhwc / row2im_nhwc / im2col_nchw / col2im_nchw /
// transpose_nchw (src/im2row_nhwc.h:20-29, src/im2col_nchw.h:20-38) on the GPU,
// with the same staging of host pointers as the convolution entry points.
namespace {

bool helper_geom_ok(const char *fn, int b, int h, int w, int c, int ho, int wo, int kh, int kw, int vpad, int hpad,
                    int vstr, int hstr, int vdil, int hdil) {
    if (b < 1 || h < 1 || w < 1 || c < 1 || ho < 1 || wo < 1 || kh < 1 || kw < 1 || vpad < 0 || hpad < 0 ||
        vstr < 1 || hstr < 1 || vdil < 1 || hdil < 1) {
        cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "%s: invalid geometry", fn);
        return false;
    }
    return true;
}

// in -> lowered (im2row / im2col); the lowered buffer is read too: padding entries stay as they were
void helper_lower(bool nchw, float *low, const float *in, int b, int h, int w, int c, int ho, int wo, int kh, int kw,
                  int vpad, int hpad, int vstr, int hstr, int vdil, int hdil) {
    const char *fn = nchw ? "im2col_nchw" : "im2row_nhwc";
    if (!helper_geom_ok(fn, b, h, w, c, ho, wo, kh, kw, vpad, hpad, vstr, hstr, vdil, hdil)) return;
    if (!low || !in) {
        cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "%s: NULL tensor", fn);
        return;
    }
    std::lock_guard<std::mutex> lk(g_dropin_mu);
    Arg a_low{low, nullptr, sizeof(float) * (size_t) b * ho * wo * c * kh * kw, false};
    Arg a_in{in, nullptr, sizeof(float) * (size_t) b * h * w * c, false};
    if (!stage_in(a_in, SLOT_IN, true) || !stage_in(a_low, SLOT_OUT, true)) return;
    cudaError_t e = nchw ? cg_helper_im2col((float *) a_low.dev, (const float *) a_in.dev, b, c, h, w, ho, wo, kh, kw,
                                            vpad, hpad, vstr, hstr, vdil, hdil, 0)
                         : cg_helper_im2row((float *) a_low.dev, (const float *) a_in.dev, b, h, w, c, ho, wo, kh, kw,
                                            vpad, hpad, vstr, hstr, vdil, hdil, 0);
    if (cg_cuda_check(e, fn)) return;
    if (a_low.staged) stage_out(a_low);
}

// lowered -> out, accumulated (row2im / col2im)
void helper_raise(bool nchw, const float *low, float *out, int b, int h, int w, int c, int ho, int wo, int kh, int kw,
                  int vpad, int hpad, int vstr, int hstr, int vdil, int hdil) {
    const char *fn = nchw ? "col2im_nchw" : "row2im_nhwc";
    if (!helper_geom_ok(fn, b, h, w, c, ho, wo, kh, kw, vpad, hpad, vstr, hstr, vdil, hdil)) return;
    if (!low || !out) {
        cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "%s: NULL tensor", fn);
        return;
    }
    std::lock_guard<std::mutex> lk(g_dropin_mu);
    Arg a_low{low, nullptr, sizeof(float) * (size_t) b * ho * wo * c * kh * kw, false};
    Arg a_out{out, nullptr, sizeof(float) * (size_t) b * h * w * c, false};
    if (!stage_in(a_low, SLOT_IN, true) || !stage_in(a_out, SLOT_OUT, true)) return;
    cudaError_t e = nchw ? cg_helper_col2im((const float *) a_low.dev, (float *) a_out.dev, b, c, h, w, ho, wo, kh, kw,
                                            vpad, hpad, vstr, hstr, vdil, hdil, 0)
                         : cg_helper_row2im((const float *) a_low.dev, (float *) a_out.dev, b, h, w, c, ho, wo, kh, kw,
                                            vpad, hpad, vstr, hstr, vdil, hdil, 0);
    if (cg_cuda_check(e, fn)) return;
    if (a_out.staged) stage_out(a_out);
}

}  // namespace

extern "C" void im2row_nhwc(float *rows, int ld, const float *in, int batches, int height, int width, int channels,
                            int oheight, int owidth, int kheight, int kwidth, int vpadding, int hpadding, int vstride,
                            int hstride, int vdilation, int hdilation) {
    (void) ld;   // the reference's active branch uses rows of channels*kheight*kwidth (im2row_nhwc.c:157-164)
    helper_lower(false, rows, in, batches, height, width, channels, oheight, owidth, kheight, kwidth, vpadding,
                 hpadding, vstride, hstride, vdilation, hdilation);
}

extern "C" void row2im_nhwc(int m, int n, const float *rows, int ld, float *out, int batches, int height, int width,
                            int channels, int oheight, int owidth, int kheight, int kwidth, int vpadding, int hpadding,
                            int vstride, int hstride, int vdilation, int hdilation) {
    (void) m, (void) n, (void) ld;   // as in the reference (im2row_nhwc.c:210-229)
    helper_raise(false, rows, out, batches, height, width, channels, oheight, owidth, kheight, kwidth, vpadding,
                 hpadding, vstride, hstride, vdilation, hdilation);
}

extern "C" void im2col_nchw(float *cols, int ld, const float *in, int batches, int channels, int height, int width,
                            int oheight, int owidth, int kheight, int kwidth, int vpadding, int hpadding, int vstride,
                            int hstride, int vdilation, int hdilation) {
    (void) ld;   // the reference's active branch uses rows of batches*oheight*owidth (im2col_nchw.c:151-166)
    helper_lower(true, cols, in, batches, height, width, channels, oheight, owidth, kheight, kwidth, vpadding,
                 hpadding, vstride, hstride, vdilation, hdilation);
}

extern "C" void col2im_nchw(int m, int n, const float *cols, int ld, float *out, int batches, int channels, int height,
                            int width, int oheight, int owidth, int kheight, int kwidth, int vpadding, int hpadding,
                            int vstride, int hstride, int vdilation, int hdilation) {
    (void) m, (void) n, (void) ld;   // as in the reference (im2col_nchw.c:337-359)
    helper_raise(true, cols, out, batches, height, width, channels, oheight, owidth, kheight, kwidth, vpadding,
                 hpadding, vstride, hstride, vdilation, hdilation);
}

extern "C" void transpose_nchw(int rows, int cols, const float *in, int ld, float beta, float *out, int kn, int ho,
                               int wo, int start_row, int start_col) {
    const char *fn = "transpose_nchw";
    if (rows < 0 || cols < 0 || ld < rows || kn < 1 || ho < 1 || wo < 1 || start_row < 0 || start_col < 0 ||
        start_col + cols > kn) {
        cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "%s: invalid arguments", fn);
        return;
    }
    if (rows == 0 || cols == 0) return;
    if (!in || !out) {
        cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "%s: NULL tensor", fn);
        return;
    }
    std::lock_guard<std::mutex> lk(g_dropin_mu);
    // extents: in[(cols-1)*ld + rows], out up to the last image the rows reach
    const long long last_b = ((long long) start_row + rows - 1) / ((long long) ho * wo);
    Arg a_in{in, nullptr, sizeof(float) * ((size_t) (cols - 1) * ld + rows), false};
    Arg a_out{out, nullptr, sizeof(float) * (size_t) ((last_b + 1) * kn * ho * wo), false};
    // out is copied in whole: the transpose writes only the entries of its rows and columns
    if (!stage_in(a_in, SLOT_IN, true) || !stage_in(a_out, SLOT_OUT, true)) return;
    if (cg_cuda_check(cg_helper_transpose(rows, cols, (const float *) a_in.dev, ld, beta, (float *) a_out.dev, kn, ho,
                                          wo, start_row, start_col, 0),
                      fn))
        return;
    if (a_out.staged) stage_out(a_out);
}

extern "C" int alloc_pack_buffs(float **Ac_pack, float **Bc_pack) {
    if (Ac_pack) *Ac_pack = nullptr;
    if (Bc_pack) *Bc_pack = nullptr;
    return 0;
}

extern "C" void sconvGemmNHWC(char trans, int b, int h, int w, int c, int kn, int kh, int kw, int vpadding,
                              int hpadding, int vstride, int hstride, int vdilation, int hdilation, const float *in,
                              const float *x, float *out, const float *bias_vector, const float *bn_running_mean,
                              const float *bn_inv_std, const float *bn_gamma, const float *bn_beta, bool relu,
                              float *ac_pack, float *bc_pack) {
    (void) ac_pack;
    (void) bc_pack;
    dropin_conv(0, trans, mkshape(b, h, w, c, kn, kh, kw, vpadding, hpadding, vstride, hstride, vdilation, hdilation),
                in, x, out, bias_vector, bn_running_mean, bn_inv_std, bn_gamma, bn_beta, relu);
}

extern "C" void sconvGemmNHWC_back(int b, int h, int w, int c, int kn, int kh, int kw, int vstride, int hstride,
                                   int vpadding, int hpadding, int vdilation, int hdilation, const float *weights,
                                   const float *dy, float *dx, float *ac_pack, float *bc_pack) {
    (void) ac_pack;
    (void) bc_pack;
    dropin_back(0, mkshape(b, h, w, c, kn, kh, kw, vpadding, hpadding, vstride, hstride, vdilation, hdilation),
                weights, dy, dx);
}

extern "C" void sconvGemmNCHW(char trans, int b, int c, int h, int w, int kn, int kh, int kw, int vpadding,
                              int hpadding, int vstride, int hstride, int vdilation, int hdilation, const float *in,
                              const float *x, float *out, const float *bias_vector, const float *bn_running_mean,
                              const float *bn_inv_std, const float *bn_gamma, const float *bn_beta, bool relu,
                              float *ac_pack, float *bc_pack) {
    (void) ac_pack;
    (void) bc_pack;
    dropin_conv(1, trans, mkshape(b, h, w, c, kn, kh, kw, vpadding, hpadding, vstride, hstride, vdilation, hdilation),
                in, x, out, bias_vector, bn_running_mean, bn_inv_std, bn_gamma, bn_beta, relu);
}

extern "C" void sconvGemmNCHW_back(int b, int c, int h, int w, int kn, int kh, int kw, int vstride, int hstride,
                                   int vpadding, int hpadding, int vdilation, int hdilation, const float *weights,
                                   const float *dy, float *dx, float *ac_pack, float *bc_pack) {
    (void) ac_pack;
    (void) bc_pack;
    dropin_back(1, mkshape(b, h, w, c, kn, kh, kw, vpadding, hpadding, vstride, hstride, vdilation, hdilation),
                weights, dy, dx);
}
