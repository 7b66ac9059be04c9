"""GPU tests of the BF16 tensor-core form (tcgen05 + TMEM + TMA).

Each result is compared with the FP64 direct-convolution oracle run on the
same BF16-rounded inputs (so the only differences left are FP32 accumulation
and the BF16 rounding of the output) and with the FP64 result of the original
FP32 inputs, where the stated target is max relative error <= 1e-2.
"""
import numpy as np
import pytest

import cases as C
from parity import rel_max_rms

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

BF16_TOL = 1e-2        # stated target vs FP64 of the FP32 inputs (normwise max relative error)
BF16_SELF_TOL = 6e-3   # vs FP64 of the BF16-rounded inputs: output rounding (2^-9) + FP32 accumulation


def bf16r(a):
    return torch.from_numpy(np.ascontiguousarray(a)).to(torch.bfloat16).float().numpy()


def to_dev_bf16_nhwc(cg, tc, x_nhwc, b, c, h, w):
    xt = torch.from_numpy(x_nhwc).cuda()
    out = torch.empty(b, h, w, tc.c8(c), dtype=torch.bfloat16, device="cuda")
    tc.to_bf16_nhwc(cg.NHWC, b, c, h, w, xt, out)
    return out


def pack(cg, tc, s, kind, w):
    nbytes = tc.weights_size(s, kind)
    assert nbytes > 0
    packed = torch.empty(nbytes // 2, dtype=torch.bfloat16, device="cuda")
    tc.pack_weights(cg.NHWC, s, kind, torch.from_numpy(w).cuda(), packed)
    return packed


FWD_SHAPES = [
    # b, h, w, c, kn, k, pad, stride, dil
    (2, 14, 14, 64, 64, 3, 1, 1, 1),
    (2, 14, 14, 64, 256, 1, 0, 1, 1),
    (2, 9, 9, 128, 128, 3, 1, 2, 1),
    (3, 7, 7, 512, 512, 3, 1, 1, 1),
    (2, 20, 20, 3, 64, 7, 3, 2, 1),      # stem-like: 3 channels padded to 8
    (1, 13, 11, 40, 72, 3, 2, 1, 2),     # ragged channels, dilation
    (2, 8, 8, 256, 1024, 1, 0, 1, 1),
    (1, 15, 15, 96, 192, 3, 1, 2, 1),
    (1, 17, 19, 8, 72, 5, 2, 1, 1),      # small-channel path: 25 taps (7 padded), one 128-wide N tile for 72 channels
    (2, 11, 9, 5, 64, 3, 1, 2, 2),       # small-channel path: stride 2, dilation 2
    (3, 30, 30, 3, 128, 7, 3, 2, 1),     # small-channel path: stem with 128 output channels
]


@pytest.mark.parametrize("shape", FWD_SHAPES, ids=[str(s) for s in FWD_SHAPES])
def test_fwd_bf16_against_fp64(cglib, oracle_lib, shape):
    from convgemm_gb300 import tc
    cg, O = cglib, oracle_lib
    b, h, w, c, kn, k, pad, stride, dil = shape
    g = C.geom(b, h, w, c, kn, k, k, pad=pad, stride=stride, dil=dil)
    s = cg.Shape.of(b, h, w, c, kn, k, k, pad, pad, stride, stride, dil, dil)
    rng = np.random.default_rng(sum(shape))
    K = c * k * k
    x = rng.standard_normal(b * h * w * c).astype(np.float32)
    wt = (rng.standard_normal(K * kn) * np.sqrt(2.0 / K)).astype(np.float32)
    epi = {"bias": rng.uniform(-.1, .1, kn).astype(np.float32), "mean": rng.normal(0, .1, kn).astype(np.float32),
           "inv_std": (1 / np.sqrt(rng.uniform(.5, 2, kn) + 1e-5)).astype(np.float32),
           "gamma": rng.uniform(.5, 1.5, kn).astype(np.float32), "beta": rng.uniform(-.1, .1, kn).astype(np.float32),
           "relu": True}
    xd = to_dev_bf16_nhwc(cg, tc, x, b, c, h, w)
    wp = pack(cg, tc, s, tc.OPERAND_FWD, wt)
    scale = torch.empty(kn, device="cuda")
    shift = torch.empty(kn, device="cuda")
    dev = {k_: torch.from_numpy(v).cuda() for k_, v in epi.items() if k_ != "relu"}
    tc.fold_epilogue(kn, scale, shift, **dev)
    y = torch.empty(b, s.ho, s.wo, kn, dtype=torch.bfloat16, device="cuda")
    tc.fwd_bf16(s, xd, wp, y, scale, shift, relu=True)
    torch.cuda.synchronize()
    cg.check_device()
    got = y.float().cpu().numpy().ravel()
    ref_r = O.fwd_f64(C.NHWC, g, bf16r(wt), bf16r(x), epi).ravel()
    ref = O.fwd_f64(C.NHWC, g, wt, x, epi).ravel()
    e_self, _ = rel_max_rms(got, ref_r)
    e_max, e_rms = rel_max_rms(got, ref)
    assert e_self <= BF16_SELF_TOL, e_self
    assert e_max <= BF16_TOL, (e_max, e_rms)
    # deterministic
    y2 = torch.empty_like(y)
    tc.fwd_bf16(s, xd, wp, y2, scale, shift, relu=True)
    torch.cuda.synchronize()
    assert torch.equal(y.view(torch.int16), y2.view(torch.int16))


DGRAD_SHAPES = [
    (2, 14, 14, 64, 64, 3, 1, 1, 1),
    (2, 14, 14, 64, 128, 3, 1, 2, 1),    # four stride-phase classes
    (2, 14, 14, 256, 512, 1, 0, 2, 1),   # 1x1/s2: three classes receive no tap -> zeros
    (2, 13, 13, 64, 64, 7, 3, 2, 1),
    (1, 12, 10, 32, 48, 3, 2, 1, 2),
    (3, 7, 7, 512, 512, 3, 1, 1, 1),
    (2, 9, 9, 128, 64, 3, 0, 2, 1),      # no padding, odd size
    (2, 7, 9, 64, 128, 1, 0, 2, 1),      # 1x1/s2, odd sizes: the unreached pixels are zero
    (1, 12, 12, 128, 64, 1, 0, 3, 1),    # 1x1/s3: eight zero pixels per reached one
]


@pytest.mark.parametrize("shape", DGRAD_SHAPES, ids=[str(s) for s in DGRAD_SHAPES])
def test_dgrad_bf16_against_fp64(cglib, oracle_lib, shape):
    from convgemm_gb300 import tc
    cg, O = cglib, oracle_lib
    b, h, w, c, kn, k, pad, stride, dil = shape
    g = C.geom(b, h, w, c, kn, k, k, pad=pad, stride=stride, dil=dil)
    s = cg.Shape.of(b, h, w, c, kn, k, k, pad, pad, stride, stride, dil, dil)
    rng = np.random.default_rng(7 + sum(shape))
    K = c * k * k
    wt = (rng.standard_normal(K * kn) * np.sqrt(2.0 / K)).astype(np.float32)
    dy = rng.standard_normal(b * s.ho * s.wo * kn).astype(np.float32)
    dyd = to_dev_bf16_nhwc(cg, tc, dy, b, kn, s.ho, s.wo)
    wp = pack(cg, tc, s, tc.OPERAND_DGRAD, wt)
    dx = torch.full((b, h, w, c), float("nan"), dtype=torch.bfloat16, device="cuda")
    tc.dgrad_bf16(s, dyd, wp, dx)
    torch.cuda.synchronize()
    cg.check_device()
    got = dx.float().cpu().numpy().ravel()
    assert np.isfinite(got).all(), "every input-gradient pixel must be written"
    ref_r = O.dgrad_f64(C.NHWC, g, bf16r(wt), bf16r(dy))
    ref = O.dgrad_f64(C.NHWC, g, wt, dy)
    assert rel_max_rms(got, ref_r)[0] <= BF16_SELF_TOL
    assert rel_max_rms(got, ref)[0] <= BF16_TOL


WGRAD_SHAPES = [
    (2, 14, 14, 64, 64, 3, 1, 1, 1),      # kn < 128: X is the A operand, BN = 64
    (2, 14, 14, 64, 128, 3, 1, 2, 1),     # dY is the A operand, BN = 256
    (4, 7, 7, 256, 512, 1, 0, 1, 1),      # P = 196: ragged pixel chunks
    (2, 20, 20, 3, 64, 7, 3, 2, 1),       # stem-like: channels padded to 8, Nx = 392
    (1, 12, 10, 40, 96, 3, 2, 1, 2),      # kn = 96, dilation
    (8, 28, 28, 128, 128, 3, 1, 1, 1),    # several pixel splits
    (2, 9, 9, 16, 256, 1, 0, 2, 1),       # Nx = 16: BN = 64 on the X side
    (8, 56, 56, 64, 256, 1, 0, 1, 1),     # 49 splits: two-pass grouped reduction, dY is A
    (8, 56, 56, 256, 64, 1, 0, 1, 1),     # 49 splits, X is A
    (2, 17, 19, 8, 96, 3, 1, 1, 1),       # 8 channels: one 8-channel im2col box per tap, BN = 128
    (2, 16, 16, 5, 64, 5, 2, 1, 2),       # 5 channels padded to 8, dilation 2
    (1, 9, 9, 8, 64, 1, 0, 1, 1),         # 8 channels, 1x1: Nx = 8, one tap
    (1, 224, 224, 3, 64, 7, 3, 2, 1),     # the ResNet-50 stem: slab kernel, 28 bands of 4 output rows
    (2, 30, 26, 8, 64, 5, 2, 2, 1),       # slab kernel: even padding, 3 tap pairs, last band of 3 rows
    (1, 19, 17, 6, 64, 3, 1, 2, 1),       # slab kernel: 3x3, 2 tap pairs
]


@pytest.mark.parametrize("shape", WGRAD_SHAPES, ids=[str(s) for s in WGRAD_SHAPES])
def test_wgrad_bf16_against_fp64(cglib, oracle_lib, shape):
    from convgemm_gb300 import tc
    cg, O = cglib, oracle_lib
    b, h, w, c, kn, k, pad, stride, dil = shape
    g = C.geom(b, h, w, c, kn, k, k, pad=pad, stride=stride, dil=dil)
    s = cg.Shape.of(b, h, w, c, kn, k, k, pad, pad, stride, stride, dil, dil)
    rng = np.random.default_rng(11 + sum(shape))
    x = rng.standard_normal(b * h * w * c).astype(np.float32)
    dy = rng.standard_normal(b * s.ho * s.wo * kn).astype(np.float32)
    xd = to_dev_bf16_nhwc(cg, tc, x, b, c, h, w)
    dyd = to_dev_bf16_nhwc(cg, tc, dy, b, kn, s.ho, s.wo)
    ws = torch.empty(tc.wgrad_bf16_workspace_size(s) // 4 + 1, device="cuda")
    K = c * k * k
    dws = []
    for layout in (cg.NHWC, cg.NCHW, cg.NHWC):
        dw = torch.full((K * kn,), float("nan"), device="cuda")
        tc.wgrad_bf16(layout, s, dyd, xd, dw, ws)
        dws.append(dw)
    torch.cuda.synchronize()
    cg.check_device()
    assert torch.equal(dws[0], dws[2]), "weight gradient must be bit-reproducible"
    got = dws[0].cpu().numpy()
    ref_r = O.wgrad_f64(C.NHWC, g, bf16r(dy), bf16r(x))
    ref = O.wgrad_f64(C.NHWC, g, dy, x)
    assert rel_max_rms(got, ref_r)[0] <= 1e-4       # only FP32 accumulation differs
    assert rel_max_rms(got, ref)[0] <= BF16_TOL
    got_nchw = dws[1].cpu().numpy()
    assert rel_max_rms(got_nchw, O.wgrad_f64(C.NCHW, g, np.ascontiguousarray(
        bf16r(dy).reshape(b, s.ho, s.wo, kn).transpose(0, 3, 1, 2)).ravel(), np.ascontiguousarray(
        bf16r(x).reshape(b, h, w, c).transpose(0, 3, 1, 2)).ravel()))[0] <= 1e-4


def test_wgrad_stem_uses_slab_kernel(cglib):
    """The ResNet-50 stem's weight gradient plans one FP32 partial per CTA of the slab kernel
    (bands of 4 output rows), whatever tile configuration is set for it."""
    from convgemm_gb300 import tc
    cg = cglib
    s = cg.Shape.of(64, 224, 224, 3, 64, 7, 7, 3, 3, 2, 2)
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    try:
        tc.tune_set(tc.TUNE_WGRAD, s, 128, 7)
        assert tc.wgrad_bf16_plan(s)[:2] == (64, min(sms, 64 * 28))
    finally:
        tc.tune_clear()


def test_wgrad_bf16_rejects_small_workspace(cglib):
    from convgemm_gb300 import tc
    cg = cglib
    s = cg.Shape.of(2, 8, 8, 64, 64, 3, 3, 1, 1)
    ws = torch.empty(16, device="cuda")
    x = torch.zeros(2, 8, 8, 64, dtype=torch.bfloat16, device="cuda")
    dy = torch.zeros(2, 8, 8, 64, dtype=torch.bfloat16, device="cuda")
    dw = torch.empty(64 * 9 * 64, device="cuda")
    with pytest.raises(cg.ConvGemmError) as ei:
        tc.wgrad_bf16(cg.NHWC, s, dy, x, dw, ws)
    assert ei.value.status == 6


def test_tuned_tile_configurations_agree(cglib, oracle_lib):
    """Every tile width and M-tile count of the tuning table gives the same forward /
    input-gradient result (the K order of an output does not depend on them; 7 M tiles
    leave the last pair with an empty tile); every weight-gradient
    split count stays within tolerance of FP64 and is reproducible."""
    from convgemm_gb300 import tc
    cg, O = cglib, oracle_lib
    b, h, w, c, kn = 4, 14, 14, 128, 192
    s = cg.Shape.of(b, h, w, c, kn, 3, 3, 1, 1, 1, 1)
    g = C.geom(b, h, w, c, kn, 3, 3, pad=1)
    rng = np.random.default_rng(77)
    x = rng.standard_normal(b * h * w * c).astype(np.float32)
    wt = (rng.standard_normal(9 * c * kn) * np.sqrt(2.0 / (9 * c))).astype(np.float32)
    dy = rng.standard_normal(b * h * w * kn).astype(np.float32)
    xd = to_dev_bf16_nhwc(cg, tc, x, b, c, h, w)
    dyd = to_dev_bf16_nhwc(cg, tc, dy, b, kn, h, w)
    wp = pack(cg, tc, s, tc.OPERAND_FWD, wt)
    wpd = pack(cg, tc, s, tc.OPERAND_DGRAD, wt)
    try:
        ys, dxs = [], []
        # aux + 4: the kernel form with eight epilogue warps ((64, 5) is not a valid pairing and
        # falls back to four)
        for bn, mt in ((64, 1), (128, 1), (256, 1), (64, 2), (128, 2), (256, 2), (128, 5), (256, 5), (64, 6),
                       (128, 6), (64, 5)):
            tc.tune_set(tc.TUNE_FWD, s, bn, mt)
            tc.tune_set(tc.TUNE_DGRAD, s, bn, mt)
            y = torch.empty(b, h, w, kn, dtype=torch.bfloat16, device="cuda")
            tc.fwd_bf16(s, xd, wp, y)
            dx = torch.empty(b, h, w, c, dtype=torch.bfloat16, device="cuda")
            tc.dgrad_bf16(s, dyd, wpd, dx)
            ys.append(y)
            dxs.append(dx)
        torch.cuda.synchronize()
        cg.check_device()
        assert all(torch.equal(ys[0], y) for y in ys[1:])
        assert all(torch.equal(dxs[0], d) for d in dxs[1:])
        ref = O.wgrad_f64(C.NHWC, g, dy, x)
        for bn, splits in ((64, 1), (256, 3), (128, 7)):
            tc.tune_set(tc.TUNE_WGRAD, s, bn, splits)
            assert tc.wgrad_bf16_plan(s)[:2] == (bn, splits)
            ws = torch.empty(tc.wgrad_bf16_workspace_size(s) // 4 + 1, device="cuda")
            d1, d2 = torch.empty(9 * c * kn, device="cuda"), torch.empty(9 * c * kn, device="cuda")
            tc.wgrad_bf16(cg.NHWC, s, dyd, xd, d1, ws)
            tc.wgrad_bf16(cg.NHWC, s, dyd, xd, d2, ws)
            torch.cuda.synchronize()
            cg.check_device()
            assert torch.equal(d1, d2)
            assert rel_max_rms(d1.cpu().numpy(), ref)[0] <= BF16_TOL
    finally:
        tc.tune_clear()


@pytest.mark.gpu
@pytest.mark.parametrize("b,h,w,c,kn,k,st,pad", [(4, 14, 14, 128, 192, 3, 1, 1), (4, 14, 14, 128, 256, 1, 1, 0),
                                                 (8, 9, 9, 256, 320, 1, 2, 0), (4, 15, 13, 64, 64, 1, 1, 0)])
def test_wgrad_operand_forms(cglib, oracle_lib, b, h, w, c, kn, k, st, pad):
    """The weight gradient's operand forms: X of a 1x1 stride-1 layer by tiled boxes (the
    default) or by im2col boxes gives the same bits; X as the A operand of a wide layer, with
    N tiles of 128 / 256 channels (partial last tile included), stays within the BF16 bound."""
    from convgemm_gb300 import tc
    cg, O = cglib, oracle_lib
    s = cg.Shape.of(b, h, w, c, kn, k, k, pad, pad, st, st)
    g = C.geom(b, h, w, c, kn, k, k, stride=st, pad=pad)
    ho, wo = C.out_hw(g)
    rng = np.random.default_rng(79)
    x = rng.standard_normal(b * h * w * c).astype(np.float32)
    dy = rng.standard_normal(b * ho * wo * kn).astype(np.float32)
    xd = to_dev_bf16_nhwc(cg, tc, x, b, c, h, w)
    dyd = to_dev_bf16_nhwc(cg, tc, dy, b, kn, ho, wo)
    ref = O.wgrad_f64(C.NHWC, g, dy, x)
    one = k == 1 and st == 1 and pad == 0

    def run(bn, aux):
        tc.tune_set(tc.TUNE_WGRAD, s, bn, aux)
        plan = tc.wgrad_bf16_plan(s)[:2]
        ws = torch.empty(tc.wgrad_bf16_workspace_size(s) // 4 + 1, device="cuda")
        d = torch.empty(k * k * c * kn, device="cuda")
        tc.wgrad_bf16(cg.NHWC, s, dyd, xd, d, ws)
        torch.cuda.synchronize()
        cg.check_device()
        return plan, d.cpu().numpy()

    try:
        for splits in (1, 3, 64):   # 64: one 64-pixel chunk per split (capped by the chunk count)
            p0, d0 = run(0, splits)
            assert rel_max_rms(d0, ref)[0] <= BF16_TOL
            if one:
                p1, d1 = run(0, splits | tc.WGRAD_IM2COL_X)
                assert p1 == p0 and np.array_equal(d0, d1), (splits, p0)
            if kn >= 128:
                for bn in (128, 256):
                    p2, d2 = run(bn, splits | tc.WGRAD_X_ON_A)
                    assert p2[0] == bn
                    assert rel_max_rms(d2, ref)[0] <= BF16_TOL, (bn, p2)
    finally:
        tc.tune_clear()


@pytest.mark.parametrize("b,h,w,c,kn,k,st,pad,splits", [
    (8, 56, 56, 64, 64, 1, 1, 0, 143),    # 64-wide tiles, X is A: 18 clusters of 8, last one partly empty
    (8, 28, 28, 128, 128, 3, 1, 1, 16),   # two clusters of 8 per tile
    (4, 28, 28, 512, 256, 1, 1, 0, 19),   # 19 splits -> 3 clusters of 8 (5 empty splits)
    (8, 28, 28, 256, 96, 3, 2, 1, 12),    # strided, kn = 96, ragged N tile
])
def test_wgrad_grouped_cluster_reduction(cglib, oracle_lib, b, h, w, c, kn, k, st, pad, splits):
    """More than 8 pixel splits, reduced by the separate fixed-order kernels (the default) or inside
    the kernel: clusters of 2 / 4 / 8 splits summed in distributed shared memory, the clusters'
    sums added by the last cluster of each tile to arrive (no reduction launch).  Each within FP32
    accumulation of FP64 on the same BF16 inputs, in both dW layouts, and bit-reproducible."""
    from convgemm_gb300 import tc
    cg, O = cglib, oracle_lib
    s = cg.Shape.of(b, h, w, c, kn, k, k, pad, pad, st, st)
    g = C.geom(b, h, w, c, kn, k, k, stride=st, pad=pad)
    ho, wo = C.out_hw(g)
    rng = np.random.default_rng(83 + splits)
    x = rng.standard_normal(b * h * w * c).astype(np.float32)
    dy = rng.standard_normal(b * ho * wo * kn).astype(np.float32)
    xd = to_dev_bf16_nhwc(cg, tc, x, b, c, h, w)
    dyd = to_dev_bf16_nhwc(cg, tc, dy, b, kn, ho, wo)
    ref = O.wgrad_f64(C.NHWC, g, bf16r(dy), bf16r(x))
    ref_nchw = O.wgrad_f64(C.NCHW, g, np.ascontiguousarray(bf16r(dy).reshape(b, ho, wo, kn).transpose(0, 3, 1, 2)).ravel(),
                           np.ascontiguousarray(bf16r(x).reshape(b, h, w, c).transpose(0, 3, 1, 2)).ravel())
    K = c * k * k
    n0 = cg.lib().convgemm_launch_count()

    def run(aux, layout):
        tc.tune_set(tc.TUNE_WGRAD, s, 0, aux)
        ws = torch.empty(tc.wgrad_bf16_workspace_size(s) // 4 + 1, device="cuda")
        d = torch.full((K * kn,), float("nan"), device="cuda")
        c0 = cg.lib().convgemm_launch_count()
        tc.wgrad_bf16(layout, s, dyd, xd, d, ws)
        launches = cg.lib().convgemm_launch_count() - c0
        torch.cuda.synchronize()
        cg.check_device()
        return d, launches

    try:
        kern, nk = run(splits, cg.NHWC)   # default: the separate reduction kernels
        assert tc.wgrad_bf16_plan(s)[1] > 8
        assert nk >= 2
        assert rel_max_rms(kern.cpu().numpy(), ref)[0] <= 1e-4
        for cs in (2, 4, 8):
            grouped, nl = run(splits | tc.WGRAD_GROUPS(cs), cg.NHWC)
            plan = tc.wgrad_bf16_plan(s)
            assert plan[1] % cs == 0 and plan[1] >= splits // 2, (cs, plan)
            assert nl == 1, "the grouped reduction needs no reduction launch"
            again, _ = run(splits | tc.WGRAD_GROUPS(cs), cg.NHWC)
            assert torch.equal(grouped, again), "bit-reproducible"
            assert rel_max_rms(grouped.cpu().numpy(), ref)[0] <= 1e-4, cs
            nchw, _ = run(splits | tc.WGRAD_GROUPS(cs), cg.NCHW)
            assert rel_max_rms(nchw.cpu().numpy(), ref_nchw)[0] <= 1e-4, cs
    finally:
        tc.tune_clear()
    assert cg.lib().convgemm_launch_count() > n0


@pytest.mark.parametrize("b,h,w,c,kn,k,pad,dil,splits", [
    (8, 28, 28, 128, 128, 3, 1, 1, 0),    # ResNet-50 stage 2 3x3: heuristic split count
    (4, 14, 14, 256, 256, 3, 1, 1, 0),    # stage 3: two input-block pairs, two output tiles
    (4, 7, 7, 512, 512, 3, 1, 1, 0),      # stage 4: one band per image
    (2, 20, 18, 128, 96, 3, 1, 1, 5),     # kn = 96: partial output tile, W != H
    (2, 16, 16, 124, 64, 3, 2, 2, 3),     # 124 channels padded to 128, 64-wide tile, dilation 2
    (2, 12, 11, 128, 128, 2, 0, 1, 2),    # even filter, no padding
    (1, 9, 9, 256, 128, 3, 1, 1, 1),      # one split: dW written by the kernel
])
def test_wgrad_slab_kernel(cglib, oracle_lib, b, h, w, c, kn, k, pad, dil, splits):
    """The slab weight gradient (stride 1, 128-channel input blocks): within FP32 accumulation of
    FP64 on the same BF16 inputs in both dW layouts, bit-reproducible, and within the same bound
    of the general kernel's result."""
    from convgemm_gb300 import tc
    cg, O = cglib, oracle_lib
    s = cg.Shape.of(b, h, w, c, kn, k, k, pad, pad, 1, 1, dil, dil)
    g = C.geom(b, h, w, c, kn, k, k, pad=pad, dil=dil)
    ho, wo = C.out_hw(g)
    rng = np.random.default_rng(91 + c + kn + k)
    x = rng.standard_normal(b * h * w * c).astype(np.float32)
    dy = rng.standard_normal(b * ho * wo * kn).astype(np.float32)
    xd = to_dev_bf16_nhwc(cg, tc, x, b, c, h, w)
    dyd = to_dev_bf16_nhwc(cg, tc, dy, b, kn, ho, wo)
    ref = O.wgrad_f64(C.NHWC, g, bf16r(dy), bf16r(x))
    ref_nchw = O.wgrad_f64(C.NCHW, g, np.ascontiguousarray(bf16r(dy).reshape(b, ho, wo, kn).transpose(0, 3, 1, 2)).ravel(),
                           np.ascontiguousarray(bf16r(x).reshape(b, h, w, c).transpose(0, 3, 1, 2)).ravel())
    K = c * k * k

    def run(bn, aux, layout):
        tc.tune_set(tc.TUNE_WGRAD, s, bn, aux)
        ws = torch.empty(tc.wgrad_bf16_workspace_size(s) // 4 + 1, device="cuda")
        d = torch.full((K * kn,), float("nan"), device="cuda")
        tc.wgrad_bf16(layout, s, dyd, xd, d, ws)
        torch.cuda.synchronize()
        cg.check_device()
        return d

    try:
        aux = tc.WGRAD_SLAB | splits
        d0 = run(0, aux, cg.NHWC)
        if splits:   # at most the requested split count (whole bands per split)
            assert 1 <= tc.wgrad_bf16_plan(s)[1] <= splits
        d1 = run(0, aux, cg.NHWC)
        assert torch.equal(d0, d1), "bit-reproducible"
        assert rel_max_rms(d0.cpu().numpy(), ref)[0] <= 1e-4
        dn = run(0, aux, cg.NCHW)
        assert rel_max_rms(dn.cpu().numpy(), ref_nchw)[0] <= 1e-4
        general = run(128 if kn > 64 else 64, 4, cg.NHWC)
        assert rel_max_rms(general.cpu().numpy(), ref)[0] <= 1e-4
    finally:
        tc.tune_clear()


def test_ring_stage_forms_give_identical_results(cglib):
    """The tuned ring-stage forms (one K block or one 64-pixel chunk per stage, twice the stages)
    issue the same MMAs in the same order: forward, input gradient and weight gradient are bit-
    identical to the default forms, and tune_describe reports the stage count of each form."""
    from convgemm_gb300 import tc
    cg = cglib
    b, h, w, c, kn = 4, 14, 14, 128, 128
    s = cg.Shape.of(b, h, w, c, kn, 3, 3, 1, 1)
    rng = np.random.default_rng(5)
    x = rng.standard_normal(b * h * w * c).astype(np.float32)
    wt = (rng.standard_normal(9 * c * kn) * np.sqrt(2.0 / (9 * c))).astype(np.float32)
    dy = rng.standard_normal(b * h * w * kn).astype(np.float32)
    xd = to_dev_bf16_nhwc(cg, tc, x, b, c, h, w)
    dyd = to_dev_bf16_nhwc(cg, tc, dy, b, kn, h, w)
    wp = pack(cg, tc, s, tc.OPERAND_FWD, wt)
    wpd = pack(cg, tc, s, tc.OPERAND_DGRAD, wt)
    try:
        outs = {}
        for bn in (64, 128):
            for aux in (1, 1 | tc.CONV_STAGES1):
                tc.tune_set(tc.TUNE_FWD, s, bn, aux)
                tc.tune_set(tc.TUNE_DGRAD, s, bn, aux)
                kern, bnd, stages, cl = tc.tune_describe(tc.TUNE_FWD, s)
                assert (kern, bnd, cl) == (0, bn, 1)
                assert stages == {64: 4, 128: 3}[bn] * (2 if aux & tc.CONV_STAGES1 else 1)
                y = torch.empty(b, h, w, kn, dtype=torch.bfloat16, device="cuda")
                dx = torch.empty(b, h, w, c, dtype=torch.bfloat16, device="cuda")
                tc.fwd_bf16(s, xd, wp, y)
                tc.dgrad_bf16(s, dyd, wpd, dx)
                outs[(bn, aux)] = (y, dx)
        torch.cuda.synchronize()
        cg.check_device()
        ref_y, ref_dx = outs[(64, 1)]
        for y, dx in outs.values():
            assert torch.equal(y, ref_y) and torch.equal(dx, ref_dx)
        for bn, splits in ((128, 4), (256, 3), (64, 12)):
            dws = []
            for flag in (0, tc.WGRAD_STAGES1):
                tc.tune_set(tc.TUNE_WGRAD, s, bn, splits | tc.WGRAD_X_ON_A * (bn != 64) | flag)
                kern, bnd, stages, cl = tc.tune_describe(tc.TUNE_WGRAD, s)
                assert kern == 0 and bnd == bn
                assert stages == {64: 2, 128: 3, 256: 2}[bn] * (2 if flag else 1)
                ws = torch.empty(tc.wgrad_bf16_workspace_size(s) // 4 + 1, device="cuda")
                d = torch.empty(9 * c * kn, device="cuda")
                tc.wgrad_bf16(cg.NHWC, s, dyd, xd, d, ws)
                dws.append(d)
            torch.cuda.synchronize()
            cg.check_device()
            assert torch.equal(dws[0], dws[1]), (bn, splits)
            # two MMA issuers (odd chunks into a second accumulator): another FP32 summation order,
            # reproducible and within FP32 accumulation of the one-issuer result
            two = []
            for _ in range(2):
                tc.tune_set(tc.TUNE_WGRAD, s, bn, splits | tc.WGRAD_X_ON_A * (bn != 64) | tc.WGRAD_TWO_ISSUERS)
                ws = torch.empty(tc.wgrad_bf16_workspace_size(s) // 4 + 1, device="cuda")
                d = torch.empty(9 * c * kn, device="cuda")
                tc.wgrad_bf16(cg.NHWC, s, dyd, xd, d, ws)
                two.append(d)
            torch.cuda.synchronize()
            cg.check_device()
            assert torch.equal(two[0], two[1]), (bn, splits)
            assert ((two[0] - dws[0]).abs().max() / dws[0].abs().max()).item() <= 1e-5, (bn, splits)
    finally:
        tc.tune_clear()


@pytest.mark.parametrize("b,h,w,c,kn,k,st,pad,bn,splits", [
    (4, 14, 14, 128, 256, 3, 1, 1, 128, 4),     # X on A, 3x3 im2col boxes, cluster of 4
    (4, 15, 13, 64, 64, 1, 1, 0, 64, 3),        # 1x1 tiled X boxes, odd pixel count, cluster of 3
    (2, 28, 28, 256, 128, 3, 2, 1, 256, 9),     # strided, dY on A, reduction kernel (9 splits)
    (2, 7, 7, 512, 512, 3, 1, 1, 256, 1),       # one split: dW written directly
])
def test_wgrad_wide_chunks_bit_identical(cglib, b, h, w, c, kn, k, st, pad, bn, splits):
    """128-pixel chunks (TMA boxes of twice the bytes, one chunk per stage) issue the MMAs in the
    same pixel order as two 64-pixel chunks per stage: the same split count gives the same bits."""
    from convgemm_gb300 import tc
    cg = cglib
    s = cg.Shape.of(b, h, w, c, kn, k, k, pad, pad, st, st)
    g = C.geom(b, h, w, c, kn, k, k, stride=st, pad=pad)
    ho, wo = C.out_hw(g)
    rng = np.random.default_rng(17 + c + kn)
    xd = to_dev_bf16_nhwc(cg, tc, rng.standard_normal(b * h * w * c).astype(np.float32), b, c, h, w)
    dyd = to_dev_bf16_nhwc(cg, tc, rng.standard_normal(b * ho * wo * kn).astype(np.float32), b, kn, ho, wo)
    xa = tc.WGRAD_X_ON_A if kn >= 128 and bn != 64 and k == 3 and st == 1 else 0
    outs = []
    try:
        for flag in (0, tc.WGRAD_WIDE_CHUNKS):
            tc.tune_set(tc.TUNE_WGRAD, s, bn, splits | xa | flag)
            plan = tc.wgrad_bf16_plan(s)
            kern, bnd, stages, cl = tc.tune_describe(tc.TUNE_WGRAD, s)
            assert kern == 0
            ws = torch.empty(tc.wgrad_bf16_workspace_size(s) // 4 + 1, device="cuda")
            d = torch.full((c * k * k * kn,), float("nan"), device="cuda")
            tc.wgrad_bf16(cg.NHWC, s, dyd, xd, d, ws)
            outs.append((plan, d))
        torch.cuda.synchronize()
        cg.check_device()
    finally:
        tc.tune_clear()
    (p0, d0), (p1, d1) = outs
    assert torch.isfinite(d1).all()
    P = b * ho * wo
    cps64 = -(-(-(-P // 64)) // splits)            # 64-pixel chunks per split
    cps128 = -(-(-(-P // 128)) // splits)          # 128-pixel chunks per split
    if cps64 * 64 == cps128 * 128 or (cps64 * 64 >= P and cps128 * 128 >= P):
        # the same partition of the pixels into splits: the same MMAs in the same order
        assert torch.equal(d0, d1), (p0, p1)
    else:
        assert ((d1 - d0).abs().max() / d0.abs().max()).item() <= 1e-5, (p0, p1)


@pytest.mark.parametrize("b,h,w,c,kn,k,st,pad,bn,aux", [
    (2, 7, 7, 512, 512, 3, 1, 1, 128, 1),             # one split, dY on A: blocks transposed into the boxes
    (2, 7, 7, 512, 512, 3, 1, 1, 128, 1 | 0x1000000),  # the same with 128-pixel chunks
    (2, 7, 7, 512, 512, 3, 1, 1, 256, 1 | 0x10000),    # one split, X on A
    (4, 14, 14, 256, 256, 3, 1, 1, 128, 4),           # cluster of 4: blocks pushed to their owners
    (4, 14, 14, 128, 256, 3, 1, 1, 128, 3 | 0x10000),  # cluster of 3, X on A (uneven block ownership)
    (16, 7, 7, 2048, 512, 1, 1, 0, 256, 8),           # 13 chunks: cluster of 7, 256-wide tiles
    (4, 14, 14, 128, 100, 3, 1, 1, 0, 2),             # kn = 100: the last channel block clipped
    (2, 11, 11, 30, 100, 3, 1, 1, 0, 1),              # 30 channels padded to 32: rows past C clipped
])
def test_wgrad_tma_epilogue_matches_scalar_layout(cglib, b, h, w, c, kn, k, st, pad, bn, aux):
    """dW of the NHWC API is staged in 32 x 32 blocks and written by TMA (one split, or one
    cluster of 2-8 splits whose blocks meet at their owner rank); the NCHW API writes the same
    sums element by element.  The two must hold the same bits."""
    from convgemm_gb300 import tc
    cg = cglib
    s = cg.Shape.of(b, h, w, c, kn, k, k, pad, pad, st, st)
    g = C.geom(b, h, w, c, kn, k, k, stride=st, pad=pad)
    ho, wo = C.out_hw(g)
    rng = np.random.default_rng(23 + c + kn + bn)
    xd = to_dev_bf16_nhwc(cg, tc, rng.standard_normal(b * h * w * c).astype(np.float32), b, c, h, w)
    dyd = to_dev_bf16_nhwc(cg, tc, rng.standard_normal(b * ho * wo * kn).astype(np.float32), b, kn, ho, wo)
    try:
        tc.tune_set(tc.TUNE_WGRAD, s, bn, aux)
        kern, _, _, cl = tc.tune_describe(tc.TUNE_WGRAD, s)
        sp = tc.wgrad_bf16_plan(s)[1]
        assert kern == 0 and sp <= (aux & 0xffff) and cl == (sp if sp <= 8 else 1), (kern, sp, cl)
        ws = torch.empty(tc.wgrad_bf16_workspace_size(s) // 4 + 1, device="cuda")
        out = {}
        for layout in (cg.NHWC, cg.NCHW):
            d = torch.full((c * k * k * kn,), float("nan"), device="cuda")
            tc.wgrad_bf16(layout, s, dyd, xd, d, ws)
            out[layout] = d
        torch.cuda.synchronize()
        cg.check_device()
    finally:
        tc.tune_clear()
    nhwc = out[cg.NHWC].view(c, k * k, kn).permute(2, 0, 1).contiguous()
    nchw = out[cg.NCHW].view(kn, c, k * k)
    assert torch.isfinite(nhwc).all()
    assert torch.equal(nhwc, nchw)


@pytest.mark.parametrize("b,h,w,c,kn,k,st,pad,xa", [
    (8, 7, 7, 256, 256, 3, 1, 1, 0),       # dY on A: 2 M tiles (one pair), 9 N tiles
    (4, 14, 14, 128, 384, 1, 1, 0, 0),     # 1x1 tiled X boxes, 3 M tiles padded to 4, N tile past Nx
    (4, 9, 9, 192, 256, 3, 1, 1, 1),       # X on A: 14 M tiles (the last one partly past Nx)
    (8, 10, 12, 128, 320, 3, 2, 1, 1),     # strided, X on A, 320 channels: second N tile partly past kn
])
def test_wgrad_cta_pairs(cglib, oracle_lib, b, h, w, c, kn, k, st, pad, xa):
    """CTA pairs (cta_group::2 MMAs on 256 x 256 and 256 x 128 tiles, each CTA loading its A rows and
    half of the B columns):
    within FP32 accumulation of FP64 on the same BF16 inputs, bit-reproducible, and the NHWC (TMA
    store) and NCHW (element stores) results hold the same bits, for one split and for several."""
    from convgemm_gb300 import tc
    cg, O = cglib, oracle_lib
    s = cg.Shape.of(b, h, w, c, kn, k, k, pad, pad, st, st)
    g = C.geom(b, h, w, c, kn, k, k, stride=st, pad=pad)
    ho, wo = C.out_hw(g)
    rng = np.random.default_rng(31 + c + kn + k)
    x = rng.standard_normal(b * h * w * c).astype(np.float32)
    dy = rng.standard_normal(b * ho * wo * kn).astype(np.float32)
    xd = to_dev_bf16_nhwc(cg, tc, x, b, c, h, w)
    dyd = to_dev_bf16_nhwc(cg, tc, dy, b, kn, ho, wo)
    ref = O.wgrad_f64(C.NHWC, g, bf16r(dy), bf16r(x))
    try:
        for bn, splits in ((256, 1), (256, 3), (128, 1), (128, 3)):
            tc.tune_set(tc.TUNE_WGRAD, s, bn, splits | tc.WGRAD_PAIR | (tc.WGRAD_X_ON_A if xa else 0))
            kern, bnd, stages, cl = tc.tune_describe(tc.TUNE_WGRAD, s)
            assert (kern, bnd, stages, cl) == (0, bn, 3 if bn == 256 else 4, 2)
            _, sp, mx = tc.wgrad_bf16_plan(s)
            assert 1 <= sp <= splits and (sp > 1) == (splits > 1 and mx > 1), (sp, mx)
            ws = torch.empty(tc.wgrad_bf16_workspace_size(s) // 4 + 1, device="cuda")
            out = []
            for layout in (cg.NHWC, cg.NHWC, cg.NCHW):
                d = torch.full((c * k * k * kn,), float("nan"), device="cuda")
                tc.wgrad_bf16(layout, s, dyd, xd, d, ws)
                out.append(d)
            torch.cuda.synchronize()
            cg.check_device()
            assert torch.equal(out[0], out[1]), (bn, splits)
            assert torch.equal(out[0].view(c, k * k, kn).permute(2, 0, 1).contiguous(), out[2].view(kn, c, k * k)), (bn, splits)
            assert rel_max_rms(out[0].cpu().numpy(), ref)[0] <= 1e-4, (bn, splits)
    finally:
        tc.tune_clear()


def test_grouped_preparation_matches_per_layer_calls(cglib):
    """One grouped launch of folds and packings gives the bytes of the per-layer calls."""
    from convgemm_gb300 import tc
    cg = cglib
    rng = np.random.default_rng(5)
    shapes = [(cg.NHWC, cg.Shape.of(2, 20, 20, 3, 64, 7, 7, 3, 3, 2, 2)),       # stem: K tail
              (cg.NHWC, cg.Shape.of(2, 14, 14, 128, 256, 3, 3, 1, 1, 2, 2)),    # stride-2 dgrad classes
              (cg.NCHW, cg.Shape.of(2, 9, 9, 40, 72, 3, 3, 1, 1, 1, 1)),        # NCHW, ragged
              (cg.NHWC, cg.Shape.of(2, 8, 8, 256, 64, 1, 1)),
              (cg.NHWC, cg.Shape.of(2, 9, 9, 40, 72, 3, 3, 1, 1, 2, 2)),       # partial 64 x 64 tiles
              (cg.NHWC, cg.Shape.of(1, 6, 6, 16, 6, 3, 3, 1, 1))]              # kn % 4 != 0: scalar paths
    items, ref = [], []
    for li, (layout, s) in enumerate(shapes):
        K = s.c * s.kh * s.kw
        wt = torch.from_numpy(rng.standard_normal(K * s.kn).astype(np.float32)).cuda()
        bn = li % 2 == 0
        ep = {k: torch.from_numpy(rng.uniform(.5, 1.5, s.kn).astype(np.float32)).cuda()
              for k in ("bias", "mean", "inv_std", "gamma", "beta")} if bn else {
            "bias": torch.from_numpy(rng.uniform(-.1, .1, s.kn).astype(np.float32)).cuda()}
        it = dict(layout=layout, shape=s, weights=wt, **ep)
        want = {}
        for kind, key in ((tc.OPERAND_FWD, "packed_fwd"), (tc.OPERAND_DGRAD, "packed_dgrad")):
            it[key] = torch.full((tc.weights_size(s, kind) // 2,), float("nan"), dtype=torch.bfloat16, device="cuda")
            want[key] = torch.empty_like(it[key])
            tc.pack_weights(layout, s, kind, wt, want[key])
        it["scale"], it["shift"] = torch.empty(s.kn, device="cuda"), torch.empty(s.kn, device="cuda")
        want["scale"], want["shift"] = torch.empty(s.kn, device="cuda"), torch.empty(s.kn, device="cuda")
        tc.fold_epilogue(s.kn, want["scale"], want["shift"], **ep)
        items.append(it)
        ref.append(want)
    p = tc.Prep(items)
    p.launch()
    torch.cuda.synchronize()
    cg.check_device()
    for it, want in zip(items, ref):
        for k, v in want.items():
            assert torch.equal(it[k].view(torch.int16) if v.dtype == torch.bfloat16 else it[k],
                               v.view(torch.int16) if v.dtype == torch.bfloat16 else v), k


def test_two_m_tiles_strided_input_gradient(cglib, oracle_lib):
    """Stride-2 input gradient (4 stride-phase classes with odd M-tile counts) with two M tiles
    per weight tile: identical to one M tile, and within tolerance of FP64."""
    from convgemm_gb300 import tc
    cg, O = cglib, oracle_lib
    b, h, w, c, kn = 3, 15, 15, 128, 128
    s = cg.Shape.of(b, h, w, c, kn, 3, 3, 1, 1, 2, 2)
    g = C.geom(b, h, w, c, kn, 3, 3, pad=1, stride=2)
    rng = np.random.default_rng(78)
    wt = (rng.standard_normal(9 * c * kn) * np.sqrt(2.0 / (9 * c))).astype(np.float32)
    x = rng.standard_normal(b * h * w * c).astype(np.float32)
    dy = rng.standard_normal(b * s.ho * s.wo * kn).astype(np.float32)
    dyd = to_dev_bf16_nhwc(cg, tc, dy, b, kn, s.ho, s.wo)
    xd = to_dev_bf16_nhwc(cg, tc, x, b, c, h, w)
    wpd = pack(cg, tc, s, tc.OPERAND_DGRAD, wt)
    wp = pack(cg, tc, s, tc.OPERAND_FWD, wt)
    try:
        outs = []
        for mt in (1, 2, 5, 6):
            tc.tune_set(tc.TUNE_DGRAD, s, 128, mt)
            tc.tune_set(tc.TUNE_FWD, s, 128, mt)
            dx = torch.empty(b, h, w, c, dtype=torch.bfloat16, device="cuda")
            tc.dgrad_bf16(s, dyd, wpd, dx)
            y = torch.empty(b, s.ho, s.wo, kn, dtype=torch.bfloat16, device="cuda")
            tc.fwd_bf16(s, xd, wp, y)
            outs.append((dx, y))
        torch.cuda.synchronize()
        cg.check_device()
        for o in outs[1:]:
            assert torch.equal(outs[0][0], o[0]) and torch.equal(outs[0][1], o[1])
        ref = O.dgrad_f64(C.NHWC, g, wt, dy)
        assert rel_max_rms(outs[1][0].float().cpu().numpy(), ref)[0] <= BF16_TOL
    finally:
        tc.tune_clear()


@pytest.mark.parametrize("shape", [(2, 14, 14, 64, 128, 3, 1, 1, 1), (2, 9, 9, 128, 64, 3, 1, 2, 1),
                                   (2, 8, 8, 256, 512, 1, 0, 2, 1)], ids=str)
def test_dgrad_relu_mask_fused(cglib, shape):
    """The ReLU-backward mask fused into the input-gradient epilogue equals the unmasked
    input gradient with the entries where x <= 0 zeroed, bit for bit."""
    from convgemm_gb300 import tc
    cg = cglib
    b, h, w, c, kn, k, pad, stride, dil = shape
    s = cg.Shape.of(b, h, w, c, kn, k, k, pad, pad, stride, stride, dil, dil)
    rng = np.random.default_rng(c + kn)
    wt = (rng.standard_normal(k * k * c * kn) * 0.1).astype(np.float32)
    x = torch.from_numpy(rng.standard_normal(b * h * w * c).astype(np.float32)).cuda().to(torch.bfloat16)
    x = torch.relu(x) - (torch.rand(x.shape, device="cuda") < 0.1).to(torch.bfloat16)   # zeros, and some negatives
    dy = to_dev_bf16_nhwc(cg, tc, rng.standard_normal(b * s.ho * s.wo * kn).astype(np.float32), b, kn, s.ho, s.wo)
    wpd = pack(cg, tc, s, tc.OPERAND_DGRAD, wt)
    dx = torch.empty(b, h, w, c, dtype=torch.bfloat16, device="cuda")
    tc.dgrad_bf16(s, dy, wpd, dx)
    dxm = torch.full_like(dx, float("nan"))
    tc.dgrad_bf16_relu(s, dy, wpd, dxm, x.reshape(b, h, w, c).contiguous())
    torch.cuda.synchronize()
    cg.check_device()
    want = torch.where(x.reshape(b, h, w, c) > 0, dx, torch.zeros_like(dx))
    assert torch.equal(dxm.view(torch.int16), want.view(torch.int16))


ACC_SHAPES = [(2, 14, 14, 64, 64, 3, 1, 1, 1),    # stride 1, 64 channels (otherwise the slab kernel's shape)
              (2, 14, 14, 256, 512, 1, 0, 2, 1),  # 1x1/s2: three classes receive no tap and keep dx
              (2, 9, 9, 128, 64, 3, 1, 2, 1),     # four stride-phase classes, direct stores
              (1, 12, 10, 32, 48, 3, 2, 1, 2)]    # ragged channels: cp.async gather path


@pytest.mark.parametrize("shape", ACC_SHAPES, ids=str)
@pytest.mark.parametrize("masked", [False, True], ids=["plain", "relu"])
def test_dgrad_bf16_accumulates_like_the_reference(cglib, oracle_lib, shape, masked):
    """accumulate=1 adds the input gradient into dx (sconvGemmNHWC_back's dx += ..., src/convGemm.c:94-95):
    FP64 oracle of dx0 + dgrad on the same BF16 inputs, within the BF16 output tolerance; with the ReLU
    mask the sum is zeroed where x <= 0."""
    from convgemm_gb300 import tc
    cg, O = cglib, oracle_lib
    b, h, w, c, kn, k, pad, stride, dil = shape
    g = C.geom(b, h, w, c, kn, k, k, pad=pad, stride=stride, dil=dil)
    s = cg.Shape.of(b, h, w, c, kn, k, k, pad, pad, stride, stride, dil, dil)
    rng = np.random.default_rng(31 + sum(shape))
    K = c * k * k
    wt = (rng.standard_normal(K * kn) * np.sqrt(2.0 / K)).astype(np.float32)
    dy = rng.standard_normal(b * s.ho * s.wo * kn).astype(np.float32)
    dyd = to_dev_bf16_nhwc(cg, tc, dy, b, kn, s.ho, s.wo)
    wp = pack(cg, tc, s, tc.OPERAND_DGRAD, wt)
    dx0 = torch.from_numpy(rng.standard_normal(b * h * w * c).astype(np.float32)).cuda().to(torch.bfloat16)
    dx0 = dx0.reshape(b, h, w, c)
    x = None
    if masked:
        x = (torch.rand(b, h, w, c, device="cuda") - 0.3).to(torch.bfloat16)
    dx = dx0.clone()
    tc.dgrad_bf16_ex(s, dyd, wp, dx, relu_x=x, accumulate=True)
    torch.cuda.synchronize()
    cg.check_device()
    want = dx0.double().cpu().numpy().ravel() + O.dgrad_f64(C.NHWC, g, bf16r(wt), bf16r(dy))
    if masked:
        want = np.where(x.float().cpu().numpy().ravel() > 0, want, 0.0)
    got = dx.float().cpu().numpy().ravel()
    assert rel_max_rms(got, want)[0] <= BF16_SELF_TOL
    # accumulate = 0 through the same entry point is the overwriting input gradient, bit for bit
    over = torch.full_like(dx, float("nan"))
    tc.dgrad_bf16_ex(s, dyd, wp, over, relu_x=x, accumulate=False)
    ref_over = torch.empty_like(dx)
    if masked:
        tc.dgrad_bf16_relu(s, dyd, wp, ref_over, x)
    else:
        tc.dgrad_bf16(s, dyd, wp, ref_over)
    torch.cuda.synchronize()
    assert torch.equal(over.view(torch.int16), ref_over.view(torch.int16))


@pytest.mark.parametrize("shape", [(2, 14, 14, 64, 96, 3, 1, 1, 1), (8, 28, 28, 64, 256, 1, 0, 1, 1)], ids=str)
def test_bias_grad_against_fp64(cglib, shape):
    """db = sum over output pixels of dY: within FP32 rounding of FP64, and reproducible."""
    from convgemm_gb300 import tc
    cg = cglib
    b, h, w, c, kn, k, pad, stride, dil = shape
    s = cg.Shape.of(b, h, w, c, kn, k, k, pad, pad, stride, stride, dil, dil)
    rng = np.random.default_rng(kn)
    dy = rng.standard_normal(b * s.ho * s.wo * kn).astype(np.float32)
    dyd = to_dev_bf16_nhwc(cg, tc, dy, b, kn, s.ho, s.wo)
    db1, db2 = torch.empty(kn, device="cuda"), torch.empty(kn, device="cuda")
    tc.bias_grad_bf16(s, dyd, db1)
    tc.bias_grad_bf16(s, dyd, db2)
    torch.cuda.synchronize()
    cg.check_device()
    assert torch.equal(db1, db2)
    ref = bf16r(dy).astype(np.float64).reshape(-1, kn).sum(0)
    assert np.abs(db1.cpu().numpy() - ref).max() <= 1e-5 * np.abs(bf16r(dy)).reshape(-1, kn).sum(0).max()


BGRAD_SHAPES = [(4, 14, 14, 64, 128, 3, 1, 1, 1),    # stride 1, one stride-phase class
                (2, 14, 14, 128, 64, 1, 0, 2, 1),    # 1x1/s2: three classes receive no tap (zero, nothing summed)
                (2, 9, 9, 64, 96, 3, 1, 2, 1),       # four stride-phase classes
                (1, 12, 10, 32, 48, 3, 2, 1, 2)]     # ragged channels: cp.async gather path, dilation 2


@pytest.mark.parametrize("shape", BGRAD_SHAPES, ids=str)
@pytest.mark.parametrize("masked", [False, True], ids=["plain", "relu"])
def test_dgrad_with_fused_bias_grad(cglib, oracle_lib, shape, masked):
    """convgemm_dgrad_bf16_bias_grad: dx bit-identical to the input gradient of
    convgemm_dgrad_bf16_ex (same mask), and db = the per-channel sum of the masked input gradient
    within FP32 accumulation of the FP64 oracle's, bit-reproducible run to run."""
    from convgemm_gb300 import tc
    cg, O = cglib, oracle_lib
    b, h, w, c, kn, k, pad, stride, dil = shape
    g = C.geom(b, h, w, c, kn, k, k, pad=pad, stride=stride, dil=dil)
    s = cg.Shape.of(b, h, w, c, kn, k, k, pad, pad, stride, stride, dil, dil)
    rng = np.random.default_rng(41 + sum(shape))
    K = c * k * k
    wt = (rng.standard_normal(K * kn) * np.sqrt(2.0 / K)).astype(np.float32)
    dy = rng.standard_normal(b * s.ho * s.wo * kn).astype(np.float32)
    dyd = to_dev_bf16_nhwc(cg, tc, dy, b, kn, s.ho, s.wo)
    wp = pack(cg, tc, s, tc.OPERAND_DGRAD, wt)
    x = (torch.rand(b, h, w, c, device="cuda") - 0.3).to(torch.bfloat16) if masked else None
    dx = torch.full((b, h, w, c), float("nan"), dtype=torch.bfloat16, device="cuda")
    db1, db2 = torch.empty(c, device="cuda"), torch.empty(c, device="cuda")
    tc.dgrad_bf16_bias_grad(s, dyd, wp, dx, db1, relu_x=x)
    dx2 = torch.empty_like(dx)
    tc.dgrad_bf16_bias_grad(s, dyd, wp, dx2, db2, relu_x=x)
    want = torch.full_like(dx, float("nan"))
    tc.dgrad_bf16_ex(s, dyd, wp, want, relu_x=x)
    torch.cuda.synchronize()
    cg.check_device()
    assert torch.equal(dx.view(torch.int16), want.view(torch.int16))
    assert torch.equal(db1, db2) and torch.equal(dx, dx2)
    ref = O.dgrad_f64(C.NHWC, g, bf16r(wt), bf16r(dy)).reshape(-1, c)
    if masked:
        ref = np.where(x.float().cpu().numpy().reshape(-1, c) > 0, ref, 0.0)
    want_db = ref.sum(0)
    got = db1.cpu().numpy().astype(np.float64)
    assert np.abs(got - want_db).max() <= 1e-5 * np.abs(ref).sum(0).max()


SLAB_SHAPES = [
    # b, h, w, c, kn, k, pad, dil: stride 1, 64-channel blocks -> the slab kernel
    (2, 14, 14, 64, 64, 3, 1, 1),       # 8 rows of 16 per tile
    (1, 20, 150, 64, 72, 3, 1, 1),      # two column chunks per row, two N tiles (72 = 64 + 8)
    (2, 12, 12, 128, 64, 2, 0, 1),      # two channel blocks, 2x2 taps, no padding
    (1, 16, 40, 64, 64, 3, 2, 2),       # dilation 2
    (2, 10, 33, 64, 128, 3, 1, 1),      # partial row group at the image bottom (3 + 3 + 3 + 1 rows)
]


@pytest.mark.parametrize("shape", SLAB_SHAPES, ids=[str(s) for s in SLAB_SHAPES])
def test_slab_kernel_matches_general_kernel_and_fp64(cglib, oracle_lib, shape):
    """Stride-1 forward and input gradient through the slab kernel are bit-identical to the
    general kernel (aux + 8 selects it) and within tolerance of FP64."""
    from convgemm_gb300 import tc
    cg, O = cglib, oracle_lib
    b, h, w, c, kn, k, pad, dil = shape
    s = cg.Shape.of(b, h, w, c, kn, k, k, pad, pad, 1, 1, dil, dil)
    g = C.geom(b, h, w, c, kn, k, k, pad=pad, dil=dil)
    rng = np.random.default_rng(sum(shape) + 5)
    K = c * k * k
    x = rng.standard_normal(b * h * w * c).astype(np.float32)
    wt = (rng.standard_normal(K * kn) * np.sqrt(2.0 / K)).astype(np.float32)
    dy = rng.standard_normal(b * s.ho * s.wo * kn).astype(np.float32)
    bias = rng.uniform(-.1, .1, kn).astype(np.float32)
    xd = to_dev_bf16_nhwc(cg, tc, x, b, c, h, w)
    dyd = to_dev_bf16_nhwc(cg, tc, dy, b, kn, s.ho, s.wo)
    wp = pack(cg, tc, s, tc.OPERAND_FWD, wt)
    wpd = pack(cg, tc, s, tc.OPERAND_DGRAD, wt)
    shift = torch.from_numpy(bias).cuda()
    outs = []
    try:
        for aux in (0, 9):   # default (slab), general kernel
            tc.tune_set(tc.TUNE_FWD, s, 64 if aux else 0, aux)
            tc.tune_set(tc.TUNE_DGRAD, s, 64 if aux else 0, aux)
            y = torch.empty(b, s.ho, s.wo, kn, dtype=torch.bfloat16, device="cuda")
            dx = torch.empty(b, h, w, c, dtype=torch.bfloat16, device="cuda")
            tc.fwd_bf16(s, xd, wp, y, None, shift, relu=True)
            tc.dgrad_bf16(s, dyd, wpd, dx)
            outs.append((y, dx))
        torch.cuda.synchronize()
        cg.check_device()
    finally:
        tc.tune_clear()
    assert torch.equal(outs[0][0].view(torch.int16), outs[1][0].view(torch.int16))
    assert torch.equal(outs[0][1].view(torch.int16), outs[1][1].view(torch.int16))
    ref = O.fwd_f64(C.NHWC, g, wt, x, {"bias": bias, "relu": True}).ravel()
    assert rel_max_rms(outs[0][0].float().cpu().numpy().ravel(), ref)[0] <= BF16_TOL
    ref = O.dgrad_f64(C.NHWC, g, wt, dy).ravel()
    assert rel_max_rms(outs[0][1].float().cpu().numpy().ravel(), ref)[0] <= BF16_TOL
