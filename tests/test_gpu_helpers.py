"""GPU explicit lowering helpers (im2row_nhwc, row2im_nhwc, im2col_nchw,
col2im_nchw, transpose_nchw under the reference's names) against the golden
outputs of the reference's own helpers (tests/golden/helpers.npz, made by
tests/golden/make_golden_helpers.py): bit for bit, including the entries the
reference leaves untouched and the accumulation of row2im / col2im, with host
and with device pointers."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

HERE = os.path.dirname(os.path.abspath(__file__))
G = np.load(os.path.join(HERE, "golden", "helpers.npz"))
GEOMS = {"g1": (2, 7, 6, 3, 3, 2, 1, 0, 2, 1, 1, 2), "g2": (1, 9, 8, 4, 3, 3, 1, 1, 1, 1, 1, 1),
         "g3": (2, 10, 7, 2, 5, 3, 2, 1, 3, 2, 1, 1)}
TRANSPOSES = {"t1": (35, 6, 40, 0.0, 10, 3, 4, 5, 2), "t2": (24, 5, 24, 0.5, 8, 2, 6, 12, 3)}


def ohw(g):
    b, h, w, c, kh, kw, vp, hp, vs, hs, vd, hd = g
    return (h + 2 * vp - vd * (kh - 1) - 1) // vs + 1, (w + 2 * hp - hd * (kw - 1) - 1) // hs + 1


def _buf(a, on_dev):
    return torch.from_numpy(a.copy()).cuda() if on_dev else a.copy()


def _np(a):
    return a.cpu().numpy() if hasattr(a, "cpu") else a


@pytest.mark.parametrize("on_dev", [False, True], ids=["host", "device"])
@pytest.mark.parametrize("name", list(GEOMS))
def test_lowering_helpers_match_reference(cglib, name, on_dev):
    cg = cglib
    g = GEOMS[name]
    b, h, w, c, kh, kw, vp, hp, vs, hs, vd, hd = g
    ho, wo = ohw(g)
    K, P = c * kh * kw, b * ho * wo
    x, low0, img0 = G[f"{name}_x"], G[f"{name}_low0"], G[f"{name}_img0"]
    r = _buf(low0, on_dev)
    cg.im2row_nhwc(r, K, _buf(x, on_dev), b, h, w, c, ho, wo, kh, kw, vp, hp, vs, hs, vd, hd)
    o = _buf(img0, on_dev)
    cg.row2im_nhwc(P, K, _buf(low0, on_dev), K, o, b, h, w, c, ho, wo, kh, kw, vp, hp, vs, hs, vd, hd)
    cl = _buf(low0, on_dev)
    cg.im2col_nchw(cl, P, _buf(x, on_dev), b, c, h, w, ho, wo, kh, kw, vp, hp, vs, hs, vd, hd)
    oc = _buf(img0, on_dev)
    cg.col2im_nchw(K, P, _buf(low0, on_dev), P, oc, b, c, h, w, ho, wo, kh, kw, vp, hp, vs, hs, vd, hd)
    torch.cuda.synchronize()
    for got, key in ((r, "im2row"), (o, "row2im"), (cl, "im2col"), (oc, "col2im")):
        assert np.array_equal(_np(got), G[f"{name}_{key}"]), key


@pytest.mark.parametrize("on_dev", [False, True], ids=["host", "device"])
@pytest.mark.parametrize("name", list(TRANSPOSES))
def test_transpose_matches_reference(cglib, name, on_dev):
    rows, cols, ld, beta, kn, ho, wo, sr, sc = TRANSPOSES[name]
    d = _buf(G[f"{name}_dst0"], on_dev)
    cglib.transpose_nchw(rows, cols, _buf(G[f"{name}_src"], on_dev), ld, beta, d, kn, ho, wo, sr, sc)
    torch.cuda.synchronize()
    assert np.array_equal(_np(d), G[f"{name}_out"])
