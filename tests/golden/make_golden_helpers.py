"""Generates tests/golden/helpers.npz from the reference's own explicit lowering
helpers (im2row_nhwc, row2im_nhwc, im2col_nchw, col2im_nchw, transpose_nchw:
src/im2row_nhwc.c, src/im2col_nchw.c, compiled unmodified into
oracle/_ref/libconvgemm_ref.so).  Output buffers start from seeded random
values, so the fixtures also pin which entries the reference leaves untouched
(padding taps of im2row / im2col) and that row2im / col2im accumulate.

Run in the container that holds the reference checkout:
    make -C oracle ref && python tests/golden/make_golden_helpers.py
"""
from __future__ import annotations

import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import oracle as O  # noqa: E402

P = ctypes.c_void_p
I = ctypes.c_int
# (b, h, w, c, kh, kw, vpad, hpad, vstr, hstr, vdil, hdil)
GEOMS = {"g1": (2, 7, 6, 3, 3, 2, 1, 0, 2, 1, 1, 2), "g2": (1, 9, 8, 4, 3, 3, 1, 1, 1, 1, 1, 1),
         "g3": (2, 10, 7, 2, 5, 3, 2, 1, 3, 2, 1, 1)}
TRANSPOSES = {"t1": (35, 6, 40, 0.0, 10, 3, 4, 5, 2), "t2": (24, 5, 24, 0.5, 8, 2, 6, 12, 3)}
#            rows, cols, ld, beta, kn, ho, wo, start_row, start_col


def ohw(g):
    b, h, w, c, kh, kw, vp, hp, vs, hs, vd, hd = g
    return (h + 2 * vp - vd * (kh - 1) - 1) // vs + 1, (w + 2 * hp - hd * (kw - 1) - 1) // hs + 1


def ptr(a):
    return a.ctypes.data_as(P)


def main():
    os.environ.setdefault("OMP_NUM_THREADS", "1")
    if not O.ref_available():
        O.build(with_ref=True)
    R = O.ref()
    R.im2row_nhwc.argtypes = [P, I, P] + [I] * 14
    R.im2col_nchw.argtypes = [P, I, P] + [I] * 14
    R.row2im_nhwc.argtypes = [I, I, P, I, P] + [I] * 14
    R.col2im_nchw.argtypes = [I, I, P, I, P] + [I] * 14
    R.transpose_nchw.argtypes = [I, I, P, I, ctypes.c_float, P, I, I, I, I, I]
    rng = np.random.default_rng(20261203)
    out = {}
    for name, g in GEOMS.items():
        b, h, w, c, kh, kw, vp, hp, vs, hs, vd, hd = g
        ho, wo = ohw(g)
        K, Pn = c * kh * kw, b * ho * wo
        x = rng.uniform(-1, 1, b * h * w * c).astype(np.float32)
        low0 = rng.uniform(-1, 1, Pn * K).astype(np.float32)
        img0 = rng.uniform(-1, 1, b * h * w * c).astype(np.float32)
        r = low0.copy()
        R.im2row_nhwc(ptr(r), K, ptr(x), b, h, w, c, ho, wo, kh, kw, vp, hp, vs, hs, vd, hd)
        o = img0.copy()
        R.row2im_nhwc(Pn, K, ptr(low0), K, ptr(o), b, h, w, c, ho, wo, kh, kw, vp, hp, vs, hs, vd, hd)
        cl = low0.copy()
        R.im2col_nchw(ptr(cl), Pn, ptr(x), b, c, h, w, ho, wo, kh, kw, vp, hp, vs, hs, vd, hd)
        oc = img0.copy()
        R.col2im_nchw(K, Pn, ptr(low0), Pn, ptr(oc), b, c, h, w, ho, wo, kh, kw, vp, hp, vs, hs, vd, hd)
        out.update({f"{name}_x": x, f"{name}_low0": low0, f"{name}_img0": img0, f"{name}_im2row": r,
                    f"{name}_row2im": o, f"{name}_im2col": cl, f"{name}_col2im": oc})
    for name, t in TRANSPOSES.items():
        rows, cols, ld, beta, kn, ho, wo, sr, sc = t
        src = rng.uniform(-1, 1, (cols - 1) * ld + rows).astype(np.float32)
        nb = (sr + rows - 1) // (ho * wo) + 1
        dst0 = rng.uniform(-1, 1, nb * kn * ho * wo).astype(np.float32)
        d = dst0.copy()
        R.transpose_nchw(rows, cols, ptr(src), ld, beta, ptr(d), kn, ho, wo, sr, sc)
        out.update({f"{name}_src": src, f"{name}_dst0": dst0, f"{name}_out": d})
    np.savez_compressed(os.path.join(HERE, "helpers.npz"), **out)
    print("helpers.npz:", len(out), "arrays")


if __name__ == "__main__":
    main()
