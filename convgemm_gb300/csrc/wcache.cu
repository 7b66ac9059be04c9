// Packed-weight cache: the tensor-core operands of a layer's FP32 weights, kept
// on the device and keyed on (device, weight pointer, layout, shape, operand kind),
// re-packed only when the caller's version number for those weights changes.
//
// The reference packs its weight operand on every call (pack_RB / pack_CB in
// src/gemm_blis.c:40-88, called for each MC x KC block from the loop nest of
// src/gemm_blis_B3A2C0.c).  For repeated calls on unchanged weights (inference,
// or the several uses of one weight version inside a training step) that packing
// is pure overhead; here a hit costs a hash lookup and no kernel launch.
//
// Concurrency: a host mutex guards the table.  A re-pack is ordered on the
// caller's stream: work already queued on other streams that still reads the old
// operand races with it, exactly as it would with any caller-owned buffer.
// Allocation happens only on a miss (cudaMalloc); a miss while the stream is being
// captured is refused, so a captured graph only ever sees hits.
#include <cstring>
#include <mutex>
#include <unordered_map>

#include "../../include/convgemm_gpu.h"
#include "cg_internal.h"

namespace {

struct Key {
    int dev, layout, kind;
    const float *w;
    convgemm_shape_t s;
    bool operator==(const Key &o) const {
        return dev == o.dev && layout == o.layout && kind == o.kind && w == o.w &&
               std::memcmp(&s, &o.s, sizeof(s)) == 0;
    }
};

struct KeyHash {
    size_t operator()(const Key &k) const {
        size_t h = std::hash<const void *>()(k.w);
        const int *v = reinterpret_cast<const int *>(&k.s);
        for (size_t i = 0; i < sizeof(k.s) / sizeof(int); i++) h = h * 1000003u ^ (size_t) (unsigned) v[i];
        return h ^ ((size_t) k.dev << 40) ^ ((size_t) k.layout << 48) ^ ((size_t) k.kind << 52);
    }
};

struct Entry {
    void *buf = nullptr;      // packed operand (then, for FP8, kn per-channel scales at scale_off)
    size_t bytes = 0, scale_off = 0;
    unsigned long long version = 0;
};

std::mutex g_mu;
std::unordered_map<Key, Entry, KeyHash> g_cache;
size_t g_bytes = 0;

size_t packed_bytes(const convgemm_shape_t &s, int kind) {
    switch (kind) {
        case CONVGEMM_CACHE_BF16_FWD: return convgemm_bf16_weights_size(&s, CONVGEMM_OPERAND_FWD);
        case CONVGEMM_CACHE_BF16_DGRAD: return convgemm_bf16_weights_size(&s, CONVGEMM_OPERAND_DGRAD);
        case CONVGEMM_CACHE_FP8_FWD: return convgemm_fp8_weights_size(&s);
        default: return 0;
    }
}

convgemm_status_t pack(const Key &k, const Entry &e, void *stream) {
    switch (k.kind) {
        case CONVGEMM_CACHE_BF16_FWD:
            return convgemm_bf16_pack_weights((convgemm_layout_t) k.layout, &k.s, CONVGEMM_OPERAND_FWD, k.w, e.buf,
                                              stream);
        case CONVGEMM_CACHE_BF16_DGRAD:
            return convgemm_bf16_pack_weights((convgemm_layout_t) k.layout, &k.s, CONVGEMM_OPERAND_DGRAD, k.w, e.buf,
                                              stream);
        default:
            return convgemm_fp8_pack_weights((convgemm_layout_t) k.layout, &k.s, k.w, e.buf,
                                             (float *) ((char *) e.buf + e.scale_off), stream);
    }
}

}  // namespace

extern "C" convgemm_status_t convgemm_weights_cached(convgemm_layout_t layout, const convgemm_shape_t *shape,
                                                     int kind, const float *weights, unsigned long long version,
                                                     const void **packed, const float **wscale, void *stream) {
    const char *fn = "convgemm_weights_cached";
    if (!shape || !weights || !packed) return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "%s: NULL argument", fn);
    if (layout != CONVGEMM_NHWC && layout != CONVGEMM_NCHW)
        return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "%s: bad layout %d", fn, (int) layout);
    if (kind < CONVGEMM_CACHE_BF16_FWD || kind > CONVGEMM_CACHE_FP8_FWD)
        return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "%s: bad operand kind %d", fn, kind);
    if (kind == CONVGEMM_CACHE_FP8_FWD && !wscale)
        return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "%s: the FP8 operand needs wscale", fn);
    const size_t pb = packed_bytes(*shape, kind);
    if (pb == 0) return cg_set_error(CONVGEMM_ERROR_NOT_SUPPORTED, "%s: no tensor-core kernel for this shape", fn);
    Key k;
    std::memset(&k, 0, sizeof(k));
    if (convgemm_status_t e = cg_cuda_check(cudaGetDevice(&k.dev), "cudaGetDevice")) return e;
    k.layout = (int) layout;
    k.kind = kind;
    k.w = weights;
    k.s = *shape;

    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_cache.find(k);
    if (it == g_cache.end()) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        if (convgemm_status_t e = cg_cuda_check(cudaStreamIsCapturing((cudaStream_t) stream, &cs), "cudaStreamIsCapturing"))
            return e;
        if (cs != cudaStreamCaptureStatusNone)
            return cg_set_error(CONVGEMM_ERROR_NOT_SUPPORTED,
                                "%s: cache miss while the stream is being captured (fill the cache before capture)", fn);
        Entry e;
        e.scale_off = (pb + 255) / 256 * 256;
        e.bytes = e.scale_off + (kind == CONVGEMM_CACHE_FP8_FWD ? sizeof(float) * (size_t) shape->kn : 0);
        if (cudaMalloc(&e.buf, e.bytes) != cudaSuccess) {
            cudaGetLastError();
            return cg_set_error(CONVGEMM_ERROR_ALLOC, "%s: cudaMalloc of %zu bytes failed", fn, e.bytes);
        }
        e.version = version;
        if (convgemm_status_t st = pack(k, e, stream)) {
            cudaFree(e.buf);
            return st;
        }
        it = g_cache.emplace(k, e).first;
        g_bytes += e.bytes;
    } else if (it->second.version != version) {
        if (convgemm_status_t st = pack(k, it->second, stream)) return st;
        it->second.version = version;
    }
    *packed = it->second.buf;
    if (wscale)
        *wscale = kind == CONVGEMM_CACHE_FP8_FWD ? (const float *) ((char *) it->second.buf + it->second.scale_off)
                                                 : nullptr;
    return CONVGEMM_SUCCESS;
}

extern "C" int convgemm_weights_cache_evict(const float *weights) {
    std::lock_guard<std::mutex> lk(g_mu);
    int n = 0;
    for (auto it = g_cache.begin(); it != g_cache.end();) {
        if (weights == nullptr || it->first.w == weights) {
            int cur = 0;
            cudaGetDevice(&cur);
            cudaSetDevice(it->first.dev);
            cudaFree(it->second.buf);   // waits for work still reading the operand
            cudaSetDevice(cur);
            g_bytes -= it->second.bytes;
            it = g_cache.erase(it);
            n++;
        } else {
            ++it;
        }
    }
    return n;
}

extern "C" size_t convgemm_weights_cache_bytes(void) {
    std::lock_guard<std::mutex> lk(g_mu);
    return g_bytes;
}
