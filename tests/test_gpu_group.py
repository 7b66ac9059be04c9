"""GPU tests of the persistent grouped BF16 forward launch.

One launch runs many convolutions of uneven shapes (channels that are not a
multiple of 64, ragged output channels, 1x1 to 5x5 filters, strides,
dilations, padding) with per-convolution tile widths.  Each output is compared
with the FP64 oracle on the BF16-rounded inputs and on the original FP32
inputs, as for the single-convolution BF16 form.
"""
import numpy as np
import pytest

import cases as C
from parity import rel_max_rms

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

BF16_TOL = 1e-2
BF16_SELF_TOL = 6e-3


def bf16r(a):
    return torch.from_numpy(np.ascontiguousarray(a)).to(torch.bfloat16).float().numpy()


def random_convs(n, seed, max_hw=18):
    """Seeded uneven convolution shapes: (b, h, w, c, kn, k, pad, stride, dil, bn, epilogue)."""
    rng = np.random.default_rng(seed)
    out = []
    while len(out) < n:
        k = int(rng.choice([1, 1, 3, 3, 5]))
        dil = int(rng.choice([1, 1, 2])) if k > 1 else 1
        stride = int(rng.choice([1, 1, 2]))
        pad = int(rng.integers(0, k // 2 * dil + 1))
        h, w = int(rng.integers(4, max_hw)), int(rng.integers(4, max_hw))
        if h + 2 * pad - dil * (k - 1) < 1 or w + 2 * pad - dil * (k - 1) < 1:
            continue
        c = int(rng.choice([8, 16, 24, 40, 64, 72, 128, 136, 256]))
        kn = int(rng.choice([8, 24, 64, 72, 120, 128, 200, 256, 264]))
        bn = int(rng.choice([0, 64, 128, 256]))
        out.append((int(rng.integers(1, 4)), h, w, c, kn, k, pad, stride, dil, bn, bool(rng.integers(0, 2))))
    return out


def build(cg, tc, convs, seed):
    rng = np.random.default_rng(seed)
    items, host = [], []
    for (b, h, w, c, kn, k, pad, stride, dil, bn, with_epi) in convs:
        s = cg.Shape.of(b, h, w, c, kn, k, k, pad, pad, stride, stride, dil, dil)
        K = c * k * k
        x = rng.standard_normal(b * h * w * c).astype(np.float32)
        wt = (rng.standard_normal(K * kn) * np.sqrt(2.0 / K)).astype(np.float32)
        xd = torch.from_numpy(x).cuda().to(torch.bfloat16)
        wp = torch.empty(tc.group_weights_size(s) // 2, dtype=torch.bfloat16, device="cuda")
        tc.group_pack_weights(cg.NHWC, s, torch.from_numpy(wt).cuda(), wp)
        y = torch.full((b, s.ho, s.wo, kn), float("nan"), dtype=torch.bfloat16, device="cuda")
        epi = {"relu": False}
        item = {"shape": s, "x": xd, "w": wp, "y": y, "bn": bn}
        if with_epi:
            epi = {"bias": rng.uniform(-.1, .1, kn).astype(np.float32), "mean": rng.normal(0, .1, kn).astype(np.float32),
                   "inv_std": (1 / np.sqrt(rng.uniform(.5, 2, kn) + 1e-5)).astype(np.float32),
                   "gamma": rng.uniform(.5, 1.5, kn).astype(np.float32),
                   "beta": rng.uniform(-.1, .1, kn).astype(np.float32), "relu": True}
            scale, shift = torch.empty(kn, device="cuda"), torch.empty(kn, device="cuda")
            tc.fold_epilogue(kn, scale, shift, **{k_: torch.from_numpy(v).cuda() for k_, v in epi.items()
                                                  if k_ != "relu"})
            item.update(scale=scale, shift=shift, relu=True)
        items.append(item)
        host.append((C.geom(b, h, w, c, kn, k, k, pad=pad, stride=stride, dil=dil), x, wt, epi))
    return items, host


@pytest.mark.parametrize("seed", [1, 2])
def test_group_uneven_against_fp64(cglib, oracle_lib, seed):
    from convgemm_gb300 import tc
    cg, O = cglib, oracle_lib
    convs = random_convs(10, seed)
    items, host = build(cg, tc, convs, 100 + seed)
    grp = tc.Group(items)
    grp.launch()
    torch.cuda.synchronize()
    cg.check_device()
    for cv, it, (g, x, wt, epi) in zip(convs, items, host):
        got = it["y"].float().cpu().numpy().ravel()
        assert np.isfinite(got).all(), cv
        ref_r = O.fwd_f64(C.NHWC, g, bf16r(wt), bf16r(x), epi).ravel()
        ref = O.fwd_f64(C.NHWC, g, wt, x, epi).ravel()
        assert rel_max_rms(got, ref_r)[0] <= BF16_SELF_TOL, cv
        assert rel_max_rms(got, ref)[0] <= BF16_TOL, cv


def test_group_graph_replay_is_deterministic(cglib):
    from convgemm_gb300 import tc
    cg = cglib
    convs = random_convs(24, 7, max_hw=30)
    items, _ = build(cg, tc, convs, 7)
    grp = tc.Group(items)
    grp.launch()
    torch.cuda.synchronize()
    first = [it["y"].clone() for it in items]
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        grp.launch(s)   # warm the stream before capture
        s.synchronize()
        for it in items:
            it["y"].fill_(float("nan"))
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=s):
            grp.launch(s)
    for _ in range(2):
        g.replay()
    torch.cuda.synchronize()
    cg.check_device()
    for a, it in zip(first, items):
        assert torch.equal(a, it["y"])


def test_group_matches_single_convolution_form(cglib):
    """Where channels are multiples of 64 the K order is that of convgemm_fwd_bf16."""
    from convgemm_gb300 import tc
    cg = cglib
    convs = [(2, 14, 14, 64, 128, 3, 1, 1, 1, 128, True), (2, 9, 9, 128, 256, 3, 1, 2, 1, 256, False),
             (1, 8, 8, 256, 64, 1, 0, 1, 1, 64, True)]
    items, _ = build(cg, tc, convs, 11)
    tc.Group(items).launch()
    for it in items:
        s = it["shape"]
        wp = torch.empty(tc.weights_size(s, tc.OPERAND_FWD) // 2, dtype=torch.bfloat16, device="cuda")
        # the grouped packing of c % 64 == 0 is the single-convolution packing
        assert wp.numel() == it["w"].numel()
        y = torch.empty_like(it["y"])
        tc.fwd_bf16(s, it["x"], it["w"], y, it.get("scale"), it.get("shift"), relu=it.get("relu", False))
        torch.cuda.synchronize()
        d = (y.float() - it["y"].float()).abs().max().item()
        assert d <= 2 ** -7 * y.float().abs().max().item(), d
