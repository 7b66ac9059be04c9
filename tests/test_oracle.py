"""CPU tests of the oracle itself: pinned to the reference's own outputs.

The golden fixtures hold outputs of the reference's code (its convGemm.c, loop
nests, packers and epilogues, built against the project's BLIS shim) for every
case in tests/golden/cases.py.  These tests check that
  * the regenerated inputs are the ones the reference saw (hash),
  * the FP64 direct convolution agrees with the reference to FP32 rounding,
  * the FP32 restatement reproduces the reference bit for bit where the
    reference's own arithmetic is order-determined, and within 1e-5 elsewhere.
"""
import os

import numpy as np
import pytest

import cases as C
from parity import FP32_TOL, bitexact, componentwise, elementwise_ref_check, errors, magnitude

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")

# Cases where the reference's result is fully determined by its summation
# order (no batch-norm epilogue, which -Ofast reassociates, and no atomic scatter).
BITEXACT = {"config1_fwd_nhwc", "fwd_nhwc_bias_k432", "fwd_nhwc_none_dil2", "fwd_nchw_none_k900",
            "fwd_nchw_bias_relu_s2", "wgrad_nhwc_3x3", "wgrad_nhwc_s2_p1000", "wgrad_nchw_3x3",
            "wgrad_nchw_1x1_s2"}


def load(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


def f64_result(O, op, layout, g, inp):
    if op == "fwd":
        return O.fwd_f64(layout, g, inp["w"], inp["x"], inp["epi"]).ravel()
    if op == "wgrad":
        return O.wgrad_f64(layout, g, inp["dy"], inp["x"])
    return O.dgrad_f64(layout, g, inp["w"], inp["dy"]) + inp["dx0"]


def port_result(O, op, layout, g, inp, n_out):
    if op == "fwd":
        out = np.zeros(n_out, np.float32)
        return O.call_fwd("port", layout, g, inp["w"], inp["x"], out, inp["epi"])
    if op == "wgrad":
        out = np.zeros(n_out, np.float32)
        return O.call_fwd("port", layout, g, inp["dy"], inp["x"], out, None, trans="T")
    out = inp["dx0"].copy()
    return O.call_back("port", layout, g, inp["w"], inp["dy"], out)


@pytest.mark.parametrize("case", C.CASES, ids=[c[0] for c in C.CASES])
def test_oracle_against_reference_outputs(oracle_lib, case):
    O = oracle_lib
    name, op, layout, g, epi_kind, data = case
    inp = C.make_inputs(*case)
    gold = load(name)
    assert str(gold["in_sha256"]) == inp["hash"], "regenerated inputs differ from the reference's"
    ref = gold["out"]
    f64 = f64_result(O, op, layout, g, inp)
    nw, ew = errors(ref, f64)
    assert nw < 2e-6, f"reference vs FP64 normwise {nw}"
    mag = magnitude(O, op, layout, g, inp)
    assert componentwise(ref, f64, mag) < 1e-6
    port = port_result(O, op, layout, g, inp, ref.size)
    assert errors(port, ref)[0] <= FP32_TOL
    assert componentwise(port, ref, mag) <= FP32_TOL
    if data == "positive":
        assert elementwise_ref_check(port, ref) <= FP32_TOL
    if name in BITEXACT:
        assert bitexact(port, ref), "restatement must match the reference bit for bit"


def test_planted_mistake_is_caught(oracle_lib):
    """A one-ulp-scale shift is inside tolerance; a wrong tap is not."""
    O = oracle_lib
    case = next(c for c in C.CASES if c[0] == "fwd_nhwc_bn_relu_s2")
    name, op, layout, g, epi_kind, data = case
    inp = C.make_inputs(*case)
    ref = load(name)["out"]
    good = O.fwd_f64(layout, g, inp["w"], inp["x"], inp["epi"]).ravel()
    mag = magnitude(O, op, layout, g, inp)
    assert errors(good, ref)[0] <= FP32_TOL and componentwise(good, ref, mag) <= FP32_TOL
    bad = good.copy()
    bad[np.argmax(np.abs(bad))] *= 1.0001
    assert errors(bad, ref)[0] > FP32_TOL and componentwise(bad, ref, mag) > FP32_TOL
    # a mistake in the index semantics (padding taken on the wrong side) is far out
    g2 = dict(g, vpad=g["vpad"] + 1, h=g["h"] + 1)
    x2 = np.zeros((g["b"], g["h"] + 1, g["w"], g["c"]), np.float32)
    x2[:, 1:] = inp["x"].reshape(g["b"], g["h"], g["w"], g["c"])
    wrong = O.fwd_f64(layout, dict(g2, vpad=g["vpad"]), inp["w"], x2.ravel(), inp["epi"]).ravel()[:ref.size]
    assert errors(wrong, ref)[0] > 1e-2


def test_explicit_im2row_matches_direct(oracle_lib):
    """Explicit lowering (the reference tests' oracle path) x GEMM == direct convolution."""
    O = oracle_lib
    import ctypes
    g = C.geom(2, 9, 7, 5, 6, 3, 3, pad=1, stride=2)
    rng = np.random.default_rng(3)
    x = rng.uniform(-1, 1, g["b"] * g["h"] * g["w"] * g["c"]).astype(np.float32)
    K = g["c"] * 9
    w = rng.standard_normal(K * g["kn"]).astype(np.float32)
    ho, wo = C.out_hw(g)
    rows = np.zeros(g["b"] * ho * wo * K, np.float32)
    fp = ctypes.POINTER(ctypes.c_float)
    O.lib().oracle_im2row_nhwc(rows.ctypes.data_as(fp), x.ctypes.data_as(fp), g["b"], g["h"], g["w"], g["c"],
                               3, 3, 1, 1, 2, 2, 1, 1)
    y = rows.reshape(-1, K).astype(np.float64) @ w.reshape(K, g["kn"]).astype(np.float64)
    d = O.fwd_f64(0, g, w, x).reshape(-1, g["kn"])
    assert np.abs(y - d).max() < 1e-12
    cols = np.zeros(K * g["b"] * ho * wo, np.float32)
    xn = np.ascontiguousarray(x.reshape(g["b"], g["h"], g["w"], g["c"]).transpose(0, 3, 1, 2)).ravel()
    O.lib().oracle_im2col_nchw(cols.ctypes.data_as(fp), xn.ctypes.data_as(fp), g["b"], g["c"], g["h"], g["w"],
                               3, 3, 1, 1, 2, 2, 1, 1)
    wn = np.ascontiguousarray(w.reshape(K, g["kn"]).T)
    yn = wn.astype(np.float64) @ cols.reshape(K, -1).astype(np.float64)   # [kn][P]
    assert np.abs(yn.T - d).max() < 1e-12


def test_bn_fold(oracle_lib):
    O = oracle_lib
    rng = np.random.default_rng(4)
    kn = 17
    b, m, s, ga, be = (rng.uniform(0.5, 1.5, kn).astype(np.float32) for _ in range(5))
    scale, shift = O.bn_fold_f64(kn, b, m, s, ga, be)
    v = rng.standard_normal(kn)
    want = ((v + b - m) * s) * ga + be
    assert np.allclose(v * scale + shift, want, rtol=1e-12, atol=1e-12)


@pytest.mark.skipif(not os.path.isdir(os.path.join(os.environ.get("CONVGEMM_REFERENCE", "/root/reference"), "src")),
                    reason="reference checkout not present")
def test_port_matches_reference_random_shapes(oracle_lib):
    """Restatement vs the reference's own code on shapes outside the fixtures."""
    O = oracle_lib
    O.build(with_ref=True)
    rng = np.random.default_rng(11)
    for trial in range(6):
        g = C.geom(int(rng.integers(1, 4)), int(rng.integers(5, 14)), int(rng.integers(5, 14)),
                   int(rng.integers(1, 70)), int(rng.integers(1, 40)), int(rng.choice([1, 3, 5])),
                   int(rng.choice([1, 3])), pad=int(rng.integers(0, 3)), stride=int(rng.integers(1, 3)),
                   dil=int(rng.integers(1, 3)))
        ho, wo = C.out_hw(g)
        if ho < 1 or wo < 1:
            continue
        K = g["c"] * g["kh"] * g["kw"]
        for layout in (0, 1):
            x = rng.uniform(-1, 1, g["b"] * g["h"] * g["w"] * g["c"]).astype(np.float32)
            w = rng.standard_normal(K * g["kn"]).astype(np.float32)
            a = np.zeros(g["b"] * ho * wo * g["kn"], np.float32)
            b = np.zeros_like(a)
            O.call_fwd("ref", layout, g, w, x, a)
            O.call_fwd("port", layout, g, w, x, b)
            assert bitexact(a, b)
            dy = rng.uniform(-1, 1, a.size).astype(np.float32)
            a = np.zeros(K * g["kn"], np.float32)
            b = np.zeros_like(a)
            O.call_fwd("ref", layout, g, dy, x, a, trans="T")
            O.call_fwd("port", layout, g, dy, x, b, trans="T")
            assert bitexact(a, b)


@pytest.mark.parametrize("name", ["config1_fwd_nhwc", "fwd_nchw_bias_relu_s2", "fwd_nhwc_bias_k432",
                                  "wgrad_nhwc_3x3", "wgrad_nchw_1x1_s2", "wgrad_nhwc_s2_p1000"])
def test_port_sampled_points_equal_the_whole_layer_port(oracle_lib, name):
    """The port's sampled-point functions (used at full ResNet-50 size on the GPU machine) give the
    whole-layer port's values bit for bit, so a sampled FP32 check is as strict as a whole one."""
    O = oracle_lib
    case = next(c for c in C.CASES if c[0] == name)
    _, op, layout, g, _, _ = case
    inp = C.make_inputs(*case)
    n_out = load(name)["out"].size
    whole = port_result(O, op, layout, g, inp, n_out)
    idx = np.random.default_rng(5).choice(n_out, size=min(n_out, 500), replace=False)
    if op == "fwd":
        pts = O.port_fwd_points(layout, g, inp["w"], inp["x"], idx, inp["epi"])
    else:
        pts = O.port_wgrad_points(layout, g, inp["dy"], inp["x"], idx)
    assert np.array_equal(pts.view(np.int32), np.asarray(whole, np.float32)[idx].view(np.int32))
