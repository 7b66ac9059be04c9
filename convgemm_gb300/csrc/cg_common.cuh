// Shared device/host helpers for the convGemm GB300 kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "cg_internal.h"

// Unsigned division by a runtime constant with a multiply-high (valid for n < 2^31).
struct FastDiv {
    uint32_t d, mul, shift;
    __host__ __device__ FastDiv() : d(1), mul(0), shift(0) {}
    __host__ FastDiv(uint32_t div) : d(div) {
        shift = 0;
        while ((1u << shift) < div) shift++;
        uint64_t m = ((1ull << 32) * ((1ull << shift) - div)) / div + 1;
        mul = (uint32_t) m;
    }
    __device__ __forceinline__ uint32_t div(uint32_t n) const {
        return (__umulhi(n, mul) + n) >> shift;
    }
    __device__ __forceinline__ void divmod(uint32_t n, uint32_t &q, uint32_t &r) const {
        q = div(n);
        r = n - q * d;
    }
};

// Geometry of one convolution as the kernels see it.
struct ConvGeom {
    int b, h, w, c, kn, kh, kw;
    int vpad, hpad, vstr, hstr, vdil, hdil;
    int ho, wo;
    int K;          // c*kh*kw
    long long P;    // b*ho*wo
};

static inline ConvGeom make_geom(const cg_shape &s) {
    ConvGeom g;
    g.b = s.b; g.h = s.h; g.w = s.w; g.c = s.c; g.kn = s.kn; g.kh = s.kh; g.kw = s.kw;
    g.vpad = s.vpad; g.hpad = s.hpad; g.vstr = s.vstride; g.hstr = s.hstride; g.vdil = s.vdil; g.hdil = s.hdil;
    g.ho = (s.h + 2 * s.vpad - s.vdil * (s.kh - 1) - 1) / s.vstride + 1;
    g.wo = (s.w + 2 * s.hpad - s.hdil * (s.kw - 1) - 1) / s.hstride + 1;
    g.K = s.c * s.kh * s.kw;
    g.P = (long long) s.b * g.ho * g.wo;
    return g;
}
