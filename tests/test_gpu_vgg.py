"""VGG-16-shaped NCHW training step (forward with bias + ReLU, input gradient,
split-K weight gradient) on reduced spatial sizes, in both forms.

FP32 plain (the drop-in's NCHW layouts: x [b][c][h][w], W [kn][c][kh][kw]):
forward and weight gradient bit for bit against the FP32 restatement of the
reference (its KC=384 summation order), input gradient within 1e-5.
BF16 (x and dY converted from the NCHW FP32 tensors, OIHW weights packed,
dW written OIHW): within 1e-2 of FP64.  dW is bit-reproducible run to run in
both forms.
"""
import numpy as np
import pytest

import cases as C
from parity import FP32_TOL, bitexact, errors, rel_max_rms

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

# (h, c, kn) of VGG-16 layers, spatial reduced 8x (224 -> 28 ...), batch 2
LAYERS = [(28, 3, 64), (28, 64, 64), (14, 64, 128), (7, 256, 256), (4, 512, 512)]


@pytest.mark.parametrize("layer", LAYERS, ids=[f"{h}x{h}_{c}-{kn}" for h, c, kn in LAYERS])
def test_vgg_layer_nchw_step(cglib, oracle_lib, layer):
    from convgemm_gb300 import tc
    cg, O = cglib, oracle_lib
    h, c, kn = layer
    b = 2
    g = C.geom(b, h, h, c, kn, 3, 3, pad=1, stride=1, dil=1)
    s = cg.Shape.of(b, h, h, c, kn, 3, 3, 1, 1, 1, 1, 1, 1)
    rng = np.random.default_rng(h * 1000 + c + kn)
    K = c * 9
    x = rng.standard_normal(b * c * h * h).astype(np.float32)
    w = (rng.standard_normal(kn * K) * np.sqrt(2.0 / K)).astype(np.float32)          # OIHW
    dy = (rng.standard_normal(b * kn * h * h) * 0.1).astype(np.float32)
    bias = rng.uniform(-.1, .1, kn).astype(np.float32)
    epi = {"bias": bias, "relu": True}
    xd, wd, dyd, bd = (torch.from_numpy(a).cuda() for a in (x, w, dy, bias))

    # FP32 plain, NCHW
    y = torch.empty(b * kn * h * h, device="cuda")
    cg.fwd_f32(cg.NCHW, s, wd, xd, y, bias=bd, relu=True)
    dx = torch.empty(b * c * h * h, device="cuda")
    cg.dgrad_f32(cg.NCHW, s, wd, dyd, dx, accumulate=False)
    ws = torch.empty(cg.wgrad_f32_workspace_size(s) // 4 + 1, device="cuda")
    dws = []
    for _ in range(2):
        dw = torch.full((kn * K,), float("nan"), device="cuda")
        cg.wgrad_f32(cg.NCHW, s, dyd, xd, dw, ws)
        dws.append(dw)
    torch.cuda.synchronize()
    cg.check_device()
    assert torch.equal(dws[0], dws[1])
    want_y = O.call_fwd("port", C.NCHW, g, w, x, np.zeros(b * kn * h * h, np.float32), epi)
    want_dw = O.call_fwd("port", C.NCHW, g, dy, x, np.zeros(kn * K, np.float32), None, trans="T")
    want_dx = O.call_back("port", C.NCHW, g, w, dy, np.zeros(b * c * h * h, np.float32))
    assert bitexact(y.cpu().numpy(), want_y)
    assert bitexact(dws[0].cpu().numpy(), want_dw)
    assert errors(dx.cpu().numpy(), want_dx)[0] <= FP32_TOL

    # BF16 form fed from the same NCHW FP32 tensors
    xb = torch.empty(b, h, h, tc.c8(c), dtype=torch.bfloat16, device="cuda")
    tc.to_bf16_nhwc(cg.NCHW, b, c, h, h, xd, xb)
    dyb = torch.empty(b, h, h, kn, dtype=torch.bfloat16, device="cuda")
    tc.to_bf16_nhwc(cg.NCHW, b, kn, h, h, dyd, dyb)
    scale, shift = torch.empty(kn, device="cuda"), torch.empty(kn, device="cuda")
    tc.fold_epilogue(kn, scale, shift, bias=bd)
    wp = torch.empty(tc.weights_size(s, tc.OPERAND_FWD) // 2, dtype=torch.bfloat16, device="cuda")
    tc.pack_weights(cg.NCHW, s, tc.OPERAND_FWD, wd, wp)
    yb = torch.empty(b, h, h, kn, dtype=torch.bfloat16, device="cuda")
    tc.fwd_bf16(s, xb, wp, yb, scale, shift, relu=True)
    wsb = torch.empty(tc.wgrad_bf16_workspace_size(s) // 4 + 1, device="cuda")
    dwb = []
    for _ in range(2):
        d = torch.full((kn * K,), float("nan"), device="cuda")
        tc.wgrad_bf16(cg.NCHW, s, dyb, xb, d, wsb)
        dwb.append(d)
    dxb = None
    if c % 8 == 0:
        wpd = torch.empty(tc.weights_size(s, tc.OPERAND_DGRAD) // 2, dtype=torch.bfloat16, device="cuda")
        tc.pack_weights(cg.NCHW, s, tc.OPERAND_DGRAD, wd, wpd)
        dxb = torch.empty(b, h, h, c, dtype=torch.bfloat16, device="cuda")
        tc.dgrad_bf16(s, dyb, wpd, dxb)
    torch.cuda.synchronize()
    cg.check_device()
    assert torch.equal(dwb[0], dwb[1])
    ref_y = O.fwd_f64(C.NCHW, g, w, x, epi).reshape(b, kn, h, h).transpose(0, 2, 3, 1).ravel()
    assert rel_max_rms(yb.float().cpu().numpy(), ref_y)[0] <= 1e-2
    assert rel_max_rms(dwb[0].cpu().numpy(), O.wgrad_f64(C.NCHW, g, dy, x))[0] <= 1e-2
    if dxb is not None:
        ref_dx = O.dgrad_f64(C.NCHW, g, w, dy).reshape(b, c, h, h).transpose(0, 2, 3, 1).ravel()
        assert rel_max_rms(dxb.float().cpu().numpy(), ref_dx)[0] <= 1e-2
