"""Per-layer precision of every ResNet-50 convolution at the benchmark's batch sizes.

For all 53 convolutions of ResNet-50 v1.5 (224x224 NHWC input; activations
N(0,1), Kaiming-normal weights, batch-norm folded from gamma U[0.5,1.5], beta
U[-0.1,0.1], mean N(0,0.1), var U[0.5,2]; ReLU after every conv1/conv2, none
after conv3 / the downsample; upstream gradients N(0, 1e-2)):

* BF16 tensor-core forward, input gradient and weight gradient at batch 64,
  max relative error <= 1e-2 against the FP64 direct convolution of the FP32
  inputs (the stated target);
* FP8-E4M3 and 3xBF16 forward at batch 128 (every layer with 64-channel
  blocks; the 3-channel stem has no FP8 / 3xBF16 kernel and stays BF16):
  FP8 max <= 8e-2 and RMS <= 5e-2, 3xBF16 max <= 1e-4;
* the FP32 drop-in (forward with the reference epilogue, weight gradient, input
  gradient) at batch 64: forward and weight gradient against the reference-order
  FP32 port, input gradient against FP64, each <= 1e-5 normwise.

Each layer is checked on 1024 output elements drawn at random across the whole
output (so across the images of the batch): max relative error is max|d| /
max|ref| over those elements, RMS relative error RMS(d) / RMS(ref).  Setting
CONVGEMM_PRECISION_REPORT=<file> writes the per-layer table as markdown.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

BF16_TOL = 1e-2
FP8_TOL_MAX, FP8_TOL_RMS = 8e-2, 5e-2
X3_TOL = 1e-4
FP32_TOL = 1e-5
NPTS = 1024


def rel(got, ref):
    got = np.asarray(got, np.float64)
    ref = np.asarray(ref, np.float64)
    d = got - ref
    return (float(np.abs(d).max() / max(np.abs(ref).max(), 1e-300)),
            float(np.sqrt(np.mean(d * d)) / max(np.sqrt(np.mean(ref * ref)), 1e-300)))


def _layers():
    from convgemm_gb300.workloads import resnet50_layers
    return resnet50_layers()


def _data(cg, layer, b, seed):
    """FP32 device tensors of one layer: x NHWC, weights [c][kh][kw][kn], dY NHWC, BN parameters."""
    l = layer
    s = cg.Shape.of(b, l["h"], l["w"], l["c"], l["kn"], l["k"], l["k"], l["pad"], l["pad"], l["stride"],
                    l["stride"], 1, 1)
    gen = torch.Generator(device="cuda").manual_seed(seed)
    K = l["c"] * l["k"] * l["k"]
    kn = l["kn"]
    x = torch.randn(b, l["h"], l["w"], l["c"], device="cuda", generator=gen)
    w = torch.randn(K, kn, device="cuda", generator=gen) * np.sqrt(2.0 / K)
    dy = torch.randn(b, s.ho, s.wo, kn, device="cuda", generator=gen) * 0.1
    var = torch.rand(kn, device="cuda", generator=gen) * 1.5 + 0.5
    epi = {"mean": torch.randn(kn, device="cuda", generator=gen) * 0.1,
           "inv_std": 1.0 / torch.sqrt(var + 1e-5),
           "gamma": torch.rand(kn, device="cuda", generator=gen) + 0.5,
           "beta": torch.rand(kn, device="cuda", generator=gen) * 0.2 - 0.1}
    relu = not (l["name"].endswith("conv3") or l["name"].endswith("down"))
    return s, x, w, dy, epi, relu


def _np(t):
    return np.ascontiguousarray(t.detach().float().cpu().numpy()).ravel()


def _report(title, header, rows):
    path = os.environ.get("CONVGEMM_PRECISION_REPORT")
    lines = [f"### {title}", "", "| " + " | ".join(header) + " |", "|" + "---|" * len(header)]
    lines += ["| " + " | ".join(r) + " |" for r in rows]
    print("\n".join(lines))
    if path:
        with open(path, "a") as f:
            f.write("\n".join(lines) + "\n\n")


def _fmt(e):
    return f"{e[0]:.2e} / {e[1]:.2e}"


def test_resnet50_bf16_every_layer_batch64(cglib, oracle_lib):
    from convgemm_gb300 import tc
    cg, O = cglib, oracle_lib
    b = 64
    rng = np.random.default_rng(20261204)
    rows, bad = [], []
    for i, l in enumerate(_layers()):
        s, x, w, dy, epi, relu = _data(cg, l, b, 1000 + i)
        g, kn, c = s.as_dict(), s.kn, s.c
        xb = torch.empty(b, s.h, s.w, tc.c8(c), dtype=torch.bfloat16, device="cuda")
        tc.to_bf16_nhwc(cg.NHWC, b, c, s.h, s.w, x, xb)
        dyb = torch.empty(b, s.ho, s.wo, tc.c8(kn), dtype=torch.bfloat16, device="cuda")
        tc.to_bf16_nhwc(cg.NHWC, b, kn, s.ho, s.wo, dy, dyb)
        wp = torch.empty(tc.weights_size(s, tc.OPERAND_FWD) // 2, dtype=torch.bfloat16, device="cuda")
        tc.pack_weights(cg.NHWC, s, tc.OPERAND_FWD, w, wp)
        scale, shift = torch.empty(kn, device="cuda"), torch.empty(kn, device="cuda")
        tc.fold_epilogue(kn, scale, shift, **epi)
        y = torch.empty(b, s.ho, s.wo, kn, dtype=torch.bfloat16, device="cuda")
        tc.fwd_bf16(s, xb, wp, y, scale, shift, relu=relu)
        ws = torch.empty(tc.wgrad_bf16_workspace_size(s) // 4 + 1, device="cuda")
        dw = torch.empty(c * s.kh * s.kw * kn, device="cuda")
        tc.wgrad_bf16(cg.NHWC, s, dyb, xb, dw, ws)
        dx = None
        if c % 8 == 0:   # the stem's input gradient is not part of a training step
            wpd = torch.empty(tc.weights_size(s, tc.OPERAND_DGRAD) // 2, dtype=torch.bfloat16, device="cuda")
            tc.pack_weights(cg.NHWC, s, tc.OPERAND_DGRAD, w, wpd)
            dx = torch.empty(b, s.h, s.w, c, dtype=torch.bfloat16, device="cuda")
            tc.dgrad_bf16(s, dyb, wpd, dx)
        torch.cuda.synchronize()
        cg.check_device()
        xn, wn, dyn = _np(x), _np(w), _np(dy)
        en = {k: _np(v) for k, v in epi.items()}
        iy = rng.choice(y.numel(), NPTS, replace=False)
        ef = rel(_np(y)[iy], O.fwd_points_f64(O.NHWC, g, wn, xn, iy, dict(en, relu=relu)))
        iw = rng.choice(dw.numel(), min(NPTS, dw.numel()), replace=False)
        ew = rel(_np(dw)[iw], O.wgrad_points_f64(O.NHWC, g, dyn, xn, iw))
        ed = None
        if dx is not None:
            ix = rng.choice(dx.numel(), NPTS, replace=False)
            ed = rel(_np(dx)[ix], O.dgrad_points_f64(O.NHWC, g, wn, dyn, ix))
        rows.append([l["name"], _fmt(ef), _fmt(ed) if ed else "-", _fmt(ew)])
        for what, e in (("fwd", ef), ("dgrad", ed), ("wgrad", ew)):
            if e is not None and e[0] > BF16_TOL:
                bad.append((l["name"], what, e[0]))
        del x, xb, y, dy, dyb, dx, dw, ws
    _report("BF16 tensor cores, ResNet-50 batch 64 (max / RMS relative error vs FP64 of the FP32 inputs)",
            ["layer", "forward", "input gradient", "weight gradient"], rows)
    assert not bad, bad


def test_resnet50_fp8_and_bf16x3_every_layer_batch128(cglib, oracle_lib):
    from convgemm_gb300 import tc
    cg, O = cglib, oracle_lib
    b = 128
    rng = np.random.default_rng(20261205)
    rows, bad = [], []
    for i, l in enumerate(_layers()):
        if l["c"] % 64:
            continue   # the stem: no FP8 / 3xBF16 kernel, it runs in BF16
        s, x, w, dy, epi, relu = _data(cg, l, b, 2000 + i)
        del dy
        g, kn = s.as_dict(), s.kn
        scale, shift = torch.empty(kn, device="cuda"), torch.empty(kn, device="cuda")
        tc.fold_epilogue(kn, scale, shift, **epi)
        # FP8-E4M3: per-tensor activation scale, per-output-channel weight scales
        xq = torch.empty(x.numel(), dtype=torch.uint8, device="cuda")
        xs = torch.zeros(2, device="cuda")
        tc.fp8_quantize(x, xq, xs)
        wp8 = torch.empty(tc.fp8_weights_size(s), dtype=torch.uint8, device="cuda")
        wsc = torch.empty(kn, device="cuda")
        tc.fp8_pack_weights(cg.NHWC, s, w, wp8, wsc)
        sc8, sh8 = torch.empty(kn, device="cuda"), torch.empty(kn, device="cuda")
        tc.fp8_epilogue_scales(kn, scale, shift, wsc, xs, sc8, sh8)
        y8 = torch.empty(b, s.ho, s.wo, kn, dtype=torch.bfloat16, device="cuda")
        tc.fwd_fp8(s, xq, wp8, y8, sc8, sh8, relu=relu)
        # 3xBF16 split products, FP32 output
        xh = torch.empty(x.numel(), dtype=torch.bfloat16, device="cuda")
        xl = torch.empty_like(xh)
        tc.split_bf16x2(x, xh, xl)
        nw = tc.weights_size(s, tc.OPERAND_FWD) // 2
        wh = torch.empty(nw, dtype=torch.bfloat16, device="cuda")
        wl = torch.empty_like(wh)
        tc.bf16x3_pack_weights(cg.NHWC, s, w, wh, wl)
        y3 = torch.empty(b, s.ho, s.wo, kn, device="cuda")
        tc.fwd_bf16x3(s, xh, xl, wh, wl, y3, scale, shift, relu=relu)
        torch.cuda.synchronize()
        cg.check_device()
        del xq, xh, xl
        xn, wn = _np(x), _np(w)
        en = dict({k: _np(v) for k, v in epi.items()}, relu=relu)
        idx = rng.choice(y8.numel(), NPTS, replace=False)
        ref = O.fwd_points_f64(O.NHWC, g, wn, xn, idx, en)
        e8 = rel(_np(y8)[idx], ref)
        e3 = rel(_np(y3)[idx], ref)
        rows.append([l["name"], _fmt(e8), _fmt(e3), f"{float(xs[0]):.3g}"])
        if e8[0] > FP8_TOL_MAX or e8[1] > FP8_TOL_RMS:
            bad.append((l["name"], "fp8", e8))
        if e3[0] > X3_TOL:
            bad.append((l["name"], "bf16x3", e3))
        del x, y8, y3
    _report("FP8-E4M3 and 3xBF16 forward, ResNet-50 batch 128 (max / RMS relative error vs FP64 of the FP32 inputs)",
            ["layer", "FP8-E4M3", "3xBF16", "activation scale"], rows)
    assert not bad, bad


def test_resnet50_fp32_every_layer_batch64(cglib, oracle_lib):
    cg, O = cglib, oracle_lib
    b = 64
    rng = np.random.default_rng(20261206)
    rows, bad = [], []
    for i, l in enumerate(_layers()):
        s, x, w, dy, epi, relu = _data(cg, l, b, 3000 + i)
        g, kn, c = s.as_dict(), s.kn, s.c
        y = torch.empty(b, s.ho, s.wo, kn, device="cuda")
        cg.fwd_f32(cg.NHWC, s, w, x, y, relu=relu, **epi)
        ws = torch.empty(cg.wgrad_f32_workspace_size(s) // 4 + 1, device="cuda")
        dw = torch.empty(c * s.kh * s.kw, kn, device="cuda")
        cg.wgrad_f32(cg.NHWC, s, dy, x, dw, ws)
        dx = None
        if c % 8 == 0:
            dx = torch.empty_like(x)
            cg.dgrad_f32(cg.NHWC, s, w, dy, dx, accumulate=False)
        torch.cuda.synchronize()
        cg.check_device()
        xn, wn, dyn = _np(x), _np(w), _np(dy)
        en = dict({k: _np(v) for k, v in epi.items()}, relu=relu)
        iy = rng.choice(y.numel(), NPTS, replace=False)
        gy = _np(y)[iy]
        py = O.port_fwd_points(O.NHWC, g, wn, xn, iy, en)
        ef = rel(gy, py)
        same_f = float(np.mean(gy.view(np.uint32) == py.view(np.uint32)))
        iw = rng.choice(dw.numel(), min(NPTS, dw.numel()), replace=False)
        gw = _np(dw)[iw]
        pw = O.port_wgrad_points(O.NHWC, g, dyn, xn, iw)
        ew = rel(gw, pw)
        same_w = float(np.mean(gw.view(np.uint32) == pw.view(np.uint32)))
        ed = None
        if dx is not None:
            ix = rng.choice(dx.numel(), NPTS, replace=False)
            ed = rel(_np(dx)[ix], O.dgrad_points_f64(O.NHWC, g, wn, dyn, ix))
        rows.append([l["name"], _fmt(ef), f"{same_f:.3f}", _fmt(ew), f"{same_w:.3f}", _fmt(ed) if ed else "-"])
        for what, e in (("fwd", ef), ("wgrad", ew), ("dgrad", ed)):
            if e is not None and e[0] > FP32_TOL:
                bad.append((l["name"], what, e[0]))
        del x, y, dy, dx, dw, ws
    _report("FP32 drop-in, ResNet-50 batch 64 (forward / weight gradient vs the reference-order port, "
            "input gradient vs FP64; max / RMS relative error; share of sampled values bit-identical to the port)",
            ["layer", "forward", "fwd bit-identical", "weight gradient", "wgrad bit-identical", "input gradient"],
            rows)
    assert not bad, bad
