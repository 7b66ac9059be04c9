"""GPU tests of the FP8-E4M3 and 3xBF16 forward forms against the FP64 oracle.

FP8: per-tensor activation scale, per-output-channel weight scales, FP32
accumulation.  The kernel is checked tightly against FP64 of the dequantised
E4M3 inputs (only FP32 accumulation and the BF16 output rounding remain), and
its max / RMS error against FP64 of the original FP32 inputs is bounded.
3xBF16: hi*hi + hi*lo + lo*hi in FP32, FP32 output, close to FP32 accuracy.
"""
import numpy as np
import pytest

import cases as C
from parity import rel_max_rms

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

SHAPES = [
    # b, h, w, c, kn, k, pad, stride, dil
    (2, 14, 14, 64, 64, 3, 1, 1, 1),
    (2, 9, 9, 128, 256, 3, 1, 2, 1),
    (2, 8, 8, 256, 512, 1, 0, 1, 1),
    (1, 13, 11, 64, 72, 3, 2, 1, 2),
]
FP8_TOL_MAX, FP8_TOL_RMS = 8e-2, 5e-2   # E4M3 carries 3 mantissa bits
FP8_SELF_TOL = 6e-3                      # vs FP64 of the dequantised operands
X3_TOL = 1e-4                            # 3xBF16 vs FP64 of the FP32 inputs


def _setup(cg, shape, seed):
    b, h, w, c, kn, k, pad, stride, dil = shape
    g = C.geom(b, h, w, c, kn, k, k, pad=pad, stride=stride, dil=dil)
    s = cg.Shape.of(b, h, w, c, kn, k, k, pad, pad, stride, stride, dil, dil)
    rng = np.random.default_rng(seed)
    K = c * k * k
    x = rng.standard_normal(b * h * w * c).astype(np.float32)
    wt = (rng.standard_normal(K * kn) * np.sqrt(2.0 / K)).astype(np.float32)
    epi = {"bias": rng.uniform(-.1, .1, kn).astype(np.float32), "mean": rng.normal(0, .1, kn).astype(np.float32),
           "inv_std": (1 / np.sqrt(rng.uniform(.5, 2, kn) + 1e-5)).astype(np.float32),
           "gamma": rng.uniform(.5, 1.5, kn).astype(np.float32), "beta": rng.uniform(-.1, .1, kn).astype(np.float32)}
    return g, s, x, wt, epi


def _fold(tc, kn, epi):
    scale = torch.empty(kn, device="cuda")
    shift = torch.empty(kn, device="cuda")
    tc.fold_epilogue(kn, scale, shift, **{k: torch.from_numpy(v).cuda() for k, v in epi.items()})
    return scale, shift


@pytest.mark.parametrize("shape", SHAPES, ids=[str(s) for s in SHAPES])
def test_fwd_fp8_against_fp64(cglib, oracle_lib, shape):
    from convgemm_gb300 import tc
    cg, O = cglib, oracle_lib
    g, s, x, wt, epi = _setup(cg, shape, 21 + sum(shape))
    kn = s.kn
    xd = torch.from_numpy(x).cuda()
    xq = torch.empty(x.size, dtype=torch.uint8, device="cuda")
    xs = torch.zeros(2, device="cuda")
    tc.fp8_quantize(xd, xq, xs)
    wp = torch.empty(tc.fp8_weights_size(s), dtype=torch.uint8, device="cuda")
    ws = torch.empty(kn, device="cuda")
    tc.fp8_pack_weights(cg.NHWC, s, torch.from_numpy(wt).cuda(), wp, ws)
    scale, shift = _fold(tc, kn, epi)
    sc8, sh8 = torch.empty(kn, device="cuda"), torch.empty(kn, device="cuda")
    tc.fp8_epilogue_scales(kn, scale, shift, ws, xs, sc8, sh8)
    y = torch.empty(s.b, s.ho, s.wo, kn, dtype=torch.bfloat16, device="cuda")
    tc.fwd_fp8(s, xq, wp, y, sc8, sh8, relu=True)
    torch.cuda.synchronize()
    cg.check_device()
    got = y.float().cpu().numpy().ravel()
    e = dict(epi, relu=True)
    # dequantised operands: what the tensor cores actually multiplied
    f8 = torch.float8_e4m3fn
    xdq = (xq.view(f8).float() * xs[0]).cpu().numpy()
    K = s.c * s.kh * s.kw
    wpk = wp.view(f8).float().reshape(kn, -1)[:, :K] * ws[:, None]          # [kn][tap*c + ci]
    wdq = wpk.reshape(kn, s.kh * s.kw, s.c).permute(2, 1, 0).reshape(K, kn)  # -> [c][kh][kw][kn]
    ref_q = O.fwd_f64(C.NHWC, g, np.ascontiguousarray(wdq.cpu().numpy()), np.ascontiguousarray(xdq), e).ravel()
    assert rel_max_rms(got, ref_q)[0] <= FP8_SELF_TOL
    e_max, e_rms = rel_max_rms(got, O.fwd_f64(C.NHWC, g, wt, x, e).ravel())
    assert e_max <= FP8_TOL_MAX and e_rms <= FP8_TOL_RMS, (e_max, e_rms)


@pytest.mark.parametrize("shape", SHAPES, ids=[str(s) for s in SHAPES])
def test_fwd_bf16x3_against_fp64(cglib, oracle_lib, shape):
    from convgemm_gb300 import tc
    cg, O = cglib, oracle_lib
    g, s, x, wt, epi = _setup(cg, shape, 31 + sum(shape))
    kn = s.kn
    xd = torch.from_numpy(x).cuda()
    xh = torch.empty(x.size, dtype=torch.bfloat16, device="cuda")
    xl = torch.empty_like(xh)
    tc.split_bf16x2(xd, xh, xl)
    nw = tc.weights_size(s, tc.OPERAND_FWD) // 2
    wh = torch.empty(nw, dtype=torch.bfloat16, device="cuda")
    wl = torch.empty_like(wh)
    tc.bf16x3_pack_weights(cg.NHWC, s, torch.from_numpy(wt).cuda(), wh, wl)
    scale, shift = _fold(tc, kn, epi)
    y = torch.full((s.b, s.ho, s.wo, kn), float("nan"), device="cuda")
    tc.fwd_bf16x3(s, xh, xl, wh, wl, y, scale, shift, relu=True)
    torch.cuda.synchronize()
    cg.check_device()
    got = y.cpu().numpy().ravel()
    e_max, e_rms = rel_max_rms(got, O.fwd_f64(C.NHWC, g, wt, x, dict(epi, relu=True)).ravel())
    assert e_max <= X3_TOL, (e_max, e_rms)
