"""Parity cases shared by the golden-fixture generator and the tests.

Inputs are regenerated from a seed with numpy's PCG64 (platform-independent
streams); each fixture stores a hash of its inputs so a test notices if they
ever differ from the ones the reference saw.
"""
from __future__ import annotations

import hashlib

import numpy as np

NHWC, NCHW = 0, 1


def geom(b, h, w, c, kn, kh, kw, pad=0, stride=1, dil=1, vpad=None, hpad=None, vstr=None, hstr=None,
         vdil=None, hdil=None):
    return {"b": b, "h": h, "w": w, "c": c, "kn": kn, "kh": kh, "kw": kw,
            "vpad": pad if vpad is None else vpad, "hpad": pad if hpad is None else hpad,
            "vstr": stride if vstr is None else vstr, "hstr": stride if hstr is None else hstr,
            "vdil": dil if vdil is None else vdil, "hdil": dil if hdil is None else hdil}


def out_hw(g):
    ho = (g["h"] + 2 * g["vpad"] - g["vdil"] * (g["kh"] - 1) - 1) // g["vstr"] + 1
    wo = (g["w"] + 2 * g["hpad"] - g["hdil"] * (g["kw"] - 1) - 1) // g["hstr"] + 1
    return ho, wo


# The CPU-runnable reference case: NHWC forward, batch 8, 28x28, 64->64, 3x3/s1/p1, bias+ReLU.
CONFIG1 = geom(8, 28, 28, 64, 64, 3, 3, pad=1)
CONFIG1_SEED = 20261203

# (name, op, layout, geometry, epilogue kind, data kind)
#   op: fwd | wgrad | dgrad;  epilogue: none | bias | bias_relu | bias_bn | bias_bn_relu
#   data: signed (uniform[-1,1] activations, normal weights) | positive (rand()/RAND_MAX style, as the
#   reference's tests draw, tests/test_base.h:12-17)
CASES = [
    ("config1_fwd_nhwc", "fwd", NHWC, CONFIG1, "bias_relu", "config1"),
    ("fwd_nhwc_bn_relu_s2", "fwd", NHWC, geom(2, 11, 9, 12, 20, 3, 3, pad=1, stride=2), "bias_bn_relu", "signed"),
    ("fwd_nhwc_bias_k432", "fwd", NHWC, geom(2, 8, 8, 48, 24, 3, 3, pad=1), "bias", "signed"),
    ("fwd_nhwc_none_dil2", "fwd", NHWC, geom(1, 12, 10, 7, 9, 3, 3, pad=2, dil=2), "none", "signed"),
    ("fwd_nhwc_positive", "fwd", NHWC, geom(2, 10, 10, 16, 32, 3, 3, pad=1), "bias_bn_relu", "positive"),
    ("fwd_nhwc_stem7x7", "fwd", NHWC, geom(2, 20, 20, 3, 16, 7, 7, pad=3, stride=2), "bias_bn", "signed"),
    ("fwd_nchw_bn_relu", "fwd", NCHW, geom(2, 9, 11, 12, 20, 3, 3, pad=1), "bias_bn_relu", "signed"),
    ("fwd_nchw_none_k900", "fwd", NCHW, geom(2, 6, 6, 100, 33, 3, 3, pad=1), "none", "signed"),
    ("fwd_nchw_bias_relu_s2", "fwd", NCHW, geom(3, 13, 13, 8, 16, 5, 5, pad=2, stride=2), "bias_relu", "signed"),
    ("fwd_nchw_positive", "fwd", NCHW, geom(2, 10, 10, 16, 32, 3, 3, pad=1), "bias_bn_relu", "positive"),
    ("wgrad_nhwc_3x3", "wgrad", NHWC, geom(4, 12, 12, 16, 24, 3, 3, pad=1), "none", "signed"),
    ("wgrad_nhwc_s2_p1000", "wgrad", NHWC, geom(10, 20, 20, 8, 12, 3, 3, pad=1, stride=2), "none", "signed"),
    ("wgrad_nchw_3x3", "wgrad", NCHW, geom(4, 12, 12, 16, 24, 3, 3, pad=1), "none", "signed"),
    ("wgrad_nchw_1x1_s2", "wgrad", NCHW, geom(3, 14, 14, 32, 16, 1, 1, stride=2), "none", "signed"),
    ("dgrad_nhwc_3x3", "dgrad", NHWC, geom(2, 10, 10, 16, 24, 3, 3, pad=1), "none", "signed"),
    ("dgrad_nhwc_s2_kn400", "dgrad", NHWC, geom(2, 9, 9, 8, 400, 3, 3, pad=1, stride=2), "none", "signed"),
    ("dgrad_nchw_3x3_dil2", "dgrad", NCHW, geom(2, 11, 11, 8, 12, 3, 3, pad=2, dil=2), "none", "signed"),
    ("dgrad_nchw_1x1_s2", "dgrad", NCHW, geom(2, 10, 10, 16, 32, 1, 1, stride=2), "none", "signed"),
]


def _hash(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        if a is not None:
            h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def make_inputs(name, op, layout, g, epi_kind, data, seed=None):
    """Returns dict(arrays...) of float32 inputs for one case."""
    if data == "config1":
        rng = np.random.Generator(np.random.PCG64(CONFIG1_SEED))
    else:
        rng = np.random.Generator(np.random.PCG64(int.from_bytes(hashlib.sha256(name.encode()).digest()[:8], "little")))
    b, h, w, c, kn, kh, kw = (g[k] for k in ("b", "h", "w", "c", "kn", "kh", "kw"))
    ho, wo = out_hw(g)
    K = c * kh * kw
    n_x, n_w, n_y = b * h * w * c, K * kn, b * ho * wo * kn
    if data == "positive":
        u = lambda n: rng.random(n, dtype=np.float32)  # noqa: E731
        x, wts, dy = u(n_x), u(n_w), u(n_y)
        bias, mean, inv_std, gamma, beta = u(kn), u(kn), u(kn), u(kn), u(kn)
    else:
        x = rng.uniform(-1.0, 1.0, n_x).astype(np.float32)
        wts = (rng.standard_normal(n_w) * np.sqrt(2.0 / K)).astype(np.float32)
        dy = rng.uniform(-1.0, 1.0, n_y).astype(np.float32)
        bias = rng.uniform(-0.1, 0.1, kn).astype(np.float32)
        gamma = rng.uniform(0.5, 1.5, kn).astype(np.float32)
        beta = rng.uniform(-0.1, 0.1, kn).astype(np.float32)
        mean = rng.normal(0.0, 0.1, kn).astype(np.float32)
        var = rng.uniform(0.5, 2.0, kn)
        inv_std = (1.0 / np.sqrt(var + 1e-5)).astype(np.float32)
    dx0 = rng.uniform(-1.0, 1.0, n_x).astype(np.float32)
    epi = {}
    if "bias" in epi_kind:
        epi["bias"] = bias
    if "bn" in epi_kind:
        epi.update(mean=mean, inv_std=inv_std, gamma=gamma, beta=beta)
    if "relu" in epi_kind:
        epi["relu"] = True
    inp = {"x": x, "w": wts, "dy": dy, "dx0": dx0, "epi": epi}
    inp["hash"] = _hash(x, wts, dy, dx0, *(epi.get(k) for k in ("bias", "mean", "inv_std", "gamma", "beta")))
    return inp
