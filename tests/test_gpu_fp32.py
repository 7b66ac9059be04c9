"""GPU parity of the FP32 plain form (the drop-in) against the reference.

Each case runs through the reference-facing C ABI (sconvGemm* with host
pointers, as a C caller of the reference would, and with device pointers) and
through the extended API, and is compared with
  * the reference's own outputs (golden fixtures): normwise and componentwise
    relative error <= 1e-5, and the reference's own element-wise ratio on its
    all-positive data (tests/parity.py);
  * the FP32 restatement of the reference's summation order (oracle, built on
    this host): bit for bit for the forward pass and the weight gradient;
  * the FP64 direct convolution at larger sizes.
"""
import os

import numpy as np
import pytest

import cases as C
from parity import FP32_TOL, bitexact, componentwise, elementwise_ref_check, errors, magnitude

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")

torch = pytest.importorskip("torch")


def gold(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))["out"]


def dropin(cg, op, layout, g, inp, out, to_dev=False):
    """Calls the reference-named entry point exactly as the reference's callers do."""
    conv = cg.sconvGemmNHWC if layout == C.NHWC else cg.sconvGemmNCHW
    back = cg.sconvGemmNHWC_back if layout == C.NHWC else cg.sconvGemmNCHW_back
    dims = (g["b"], g["h"], g["w"], g["c"]) if layout == C.NHWC else (g["b"], g["c"], g["h"], g["w"])
    cv = (lambda a: None if a is None else torch.from_numpy(a).cuda()) if to_dev else (lambda a: a)
    e = inp["epi"]
    if to_dev:
        out_t = torch.from_numpy(out).cuda()
    else:
        out_t = out
    if op == "fwd":
        conv("N", *dims, g["kn"], g["kh"], g["kw"], g["vpad"], g["hpad"], g["vstr"], g["hstr"], g["vdil"], g["hdil"],
             cv(inp["w"]), cv(inp["x"]), out_t, cv(e.get("bias")), cv(e.get("mean")), cv(e.get("inv_std")),
             cv(e.get("gamma")), cv(e.get("beta")), e.get("relu", False))
    elif op == "wgrad":
        conv("T", *dims, g["kn"], g["kh"], g["kw"], g["vpad"], g["hpad"], g["vstr"], g["hstr"], g["vdil"], g["hdil"],
             cv(inp["dy"]), cv(inp["x"]), out_t)
    else:
        back(*dims, g["kn"], g["kh"], g["kw"], g["vstr"], g["hstr"], g["vpad"], g["hpad"], g["vdil"], g["hdil"],
             cv(inp["w"]), cv(inp["dy"]), out_t)
    if to_dev:
        torch.cuda.synchronize()
        return out_t.cpu().numpy()
    return out_t


def port(O, op, layout, g, inp, n):
    if op == "fwd":
        return O.call_fwd("port", layout, g, inp["w"], inp["x"], np.zeros(n, np.float32), inp["epi"])
    if op == "wgrad":
        return O.call_fwd("port", layout, g, inp["dy"], inp["x"], np.zeros(n, np.float32), None, trans="T")
    return O.call_back("port", layout, g, inp["w"], inp["dy"], inp["dx0"].copy())


@pytest.mark.parametrize("case", C.CASES, ids=[c[0] for c in C.CASES])
def test_dropin_matches_reference(cglib, oracle_lib, case):
    name, op, layout, g, epi_kind, data = case
    inp = C.make_inputs(*case)
    ref = gold(name)
    out0 = inp["dx0"].copy() if op == "dgrad" else np.full(ref.size, np.nan, np.float32)
    host = dropin(cglib, op, layout, g, inp, out0.copy(), to_dev=False)
    assert errors(host, ref)[0] <= FP32_TOL
    assert componentwise(host, ref, magnitude(oracle_lib, op, layout, g, inp)) <= FP32_TOL
    if data == "positive":
        assert elementwise_ref_check(host, ref) <= FP32_TOL
    dev = dropin(cglib, op, layout, g, inp, out0.copy(), to_dev=True)
    assert bitexact(host, dev), "host-staged and device-pointer calls must agree"
    if op != "dgrad":
        assert bitexact(host, port(oracle_lib, op, layout, g, inp, ref.size)), \
            "forward / weight gradient must follow the reference's summation order exactly"


def test_config1_bitexact_with_reference(cglib):
    """Config 1 (NHWC fwd, b=8 28x28 64->64 3x3 bias+ReLU): identical bits to the reference's output."""
    case = C.CASES[0]
    inp = C.make_inputs(*case)
    ref = gold(case[0])
    out = dropin(cglib, "fwd", C.NHWC, case[3], inp, np.zeros(ref.size, np.float32))
    assert bitexact(out, ref)


def _rand_geom(rng):
    while True:
        g = C.geom(int(rng.integers(1, 4)), int(rng.integers(3, 20)), int(rng.integers(3, 20)),
                   int(rng.integers(1, 70)), int(rng.integers(1, 150)), int(rng.choice([1, 2, 3, 5])),
                   int(rng.choice([1, 3, 4])), vpad=int(rng.integers(0, 3)), hpad=int(rng.integers(0, 3)),
                   vstr=int(rng.integers(1, 4)), hstr=int(rng.integers(1, 3)), vdil=int(rng.integers(1, 3)),
                   hdil=int(rng.integers(1, 3)))
        ho, wo = C.out_hw(g)
        if ho >= 1 and wo >= 1:
            return g


@pytest.mark.parametrize("seed", range(6))
def test_random_shapes_against_restatement(cglib, oracle_lib, seed):
    """Ragged sizes (partial tiles in every dimension, odd strides/dilations/paddings)."""
    rng = np.random.default_rng(100 + seed)
    g = _rand_geom(rng)
    ho, wo = C.out_hw(g)
    K = g["c"] * g["kh"] * g["kw"]
    for layout in (C.NHWC, C.NCHW):
        inp = {"x": rng.uniform(-1, 1, g["b"] * g["h"] * g["w"] * g["c"]).astype(np.float32),
               "w": rng.standard_normal(K * g["kn"]).astype(np.float32),
               "dy": rng.uniform(-1, 1, g["b"] * ho * wo * g["kn"]).astype(np.float32),
               "dx0": rng.uniform(-1, 1, g["b"] * g["h"] * g["w"] * g["c"]).astype(np.float32),
               "epi": {"bias": rng.uniform(-.1, .1, g["kn"]).astype(np.float32), "relu": True}}
        for op, n in (("fwd", g["b"] * ho * wo * g["kn"]), ("wgrad", K * g["kn"]), ("dgrad", None)):
            out0 = inp["dx0"].copy() if op == "dgrad" else np.zeros(n, np.float32)
            got = dropin(cglib, op, layout, g, inp, out0, to_dev=True)
            want = port(oracle_lib, op, layout, g, inp, n)
            if op == "dgrad":
                assert errors(got, want)[0] <= FP32_TOL, (g, layout)
                assert componentwise(got, want, magnitude(oracle_lib, op, layout, g, inp)) <= FP32_TOL
            else:
                assert bitexact(got, want), (g, layout, op)


@pytest.mark.parametrize("b,h,w,c,kn", [
    (2, 7, 7, 512, 512),     # 4 tiles: one CTA per (tile, KC block) in both operations, ordered reduction
    (4, 64, 76, 64, 512),    # forward: 608 tiles (4 full waves on 152 SMs), fused, 2 KC blocks folded;
                             # input gradient: 76 tiles of 256 x 64, split into 18 segments
    (8, 64, 76, 128, 64),    # forward: 152 tiles of 256 x 64, split into 3 KC blocks;
                             # input gradient: 304 tiles (one full wave), fused, 9 taps folded
])
def test_block_split_and_fused_forms_follow_reference_order(cglib, oracle_lib, b, h, w, c, kn):
    """Grids that leave SMs idle or end in a thin last wave run the forward and input gradient one
    CTA per reduction segment and add the segments in order in a second kernel; grids of full
    waves fold them inside one kernel.  The forward keeps the reference's bits in both forms (both
    layouts, with the epilogue); the input gradient, plain and accumulating, stays within FP32
    tolerance of the port and is reproducible."""
    g = C.geom(b, h, w, c, kn, 3, 3, pad=1)
    rng = np.random.default_rng(b * 1000 + kn)
    K = 9 * c
    inp = {"x": rng.uniform(-1, 1, b * h * w * c).astype(np.float32),
           "w": (rng.standard_normal(K * kn) * np.sqrt(2 / K)).astype(np.float32),
           "dy": rng.uniform(-1, 1, b * h * w * kn).astype(np.float32),
           "dx0": rng.uniform(-1, 1, b * h * w * c).astype(np.float32),
           "epi": {"bias": rng.uniform(-.1, .1, kn).astype(np.float32), "relu": True}}
    for layout in (C.NHWC, C.NCHW):
        n = b * h * w * kn
        got = dropin(cglib, "fwd", layout, g, inp, np.zeros(n, np.float32), to_dev=True)
        assert bitexact(got, port(oracle_lib, "fwd", layout, g, inp, n)), layout
        got = dropin(cglib, "dgrad", layout, g, inp, inp["dx0"].copy(), to_dev=True)
        want = port(oracle_lib, "dgrad", layout, g, inp, None)
        assert errors(got, want)[0] <= FP32_TOL, layout
        again = dropin(cglib, "dgrad", layout, g, inp, inp["dx0"].copy(), to_dev=True)
        assert bitexact(got, again), layout


def test_extended_api_streams_and_determinism(cglib):
    """convgemm_*_f32 on a side stream; weight and input gradients are bit-reproducible."""
    cg = cglib
    g = C.geom(4, 28, 28, 64, 96, 3, 3, pad=1, stride=2)
    s = cg.Shape.of(g["b"], g["h"], g["w"], g["c"], g["kn"], 3, 3, 1, 1, 2, 2, 1, 1)
    gen = torch.Generator(device="cuda").manual_seed(0)
    x = torch.rand(g["b"], g["h"], g["w"], g["c"], device="cuda", generator=gen) * 2 - 1
    w = torch.randn(g["c"] * 9, g["kn"], device="cuda", generator=gen)
    dy = torch.randn(g["b"], s.ho, s.wo, g["kn"], device="cuda", generator=gen)
    ws = torch.empty(cg.wgrad_f32_workspace_size(s) // 4, device="cuda")
    st = torch.cuda.Stream()
    outs = []
    with torch.cuda.stream(st):
        for _ in range(2):
            dw = torch.empty(g["c"] * 9, g["kn"], device="cuda")
            dx = torch.empty_like(x)
            cg.wgrad_f32(cg.NHWC, s, dy, x, dw, ws, stream=st)
            cg.dgrad_f32(cg.NHWC, s, w, dy, dx, accumulate=False, stream=st)
            outs.append((dw.clone(), dx.clone()))
    st.synchronize()
    cg.check_device(st)
    assert torch.equal(outs[0][0], outs[1][0]) and torch.equal(outs[0][1], outs[1][1])
    # against torch's own FP64 convolution
    xd = x.double().permute(0, 3, 1, 2)
    wd = w.double().reshape(g["c"], 3, 3, g["kn"]).permute(3, 0, 1, 2)
    dyd = dy.double().permute(0, 3, 1, 2)
    dx_ref = torch.nn.grad.conv2d_input(xd.shape, wd, dyd, stride=2, padding=1)
    dw_ref = torch.nn.grad.conv2d_weight(xd, wd.shape, dyd, stride=2, padding=1)
    assert errors(outs[0][1].permute(0, 3, 1, 2).cpu().numpy(), dx_ref.cpu().numpy())[0] < FP32_TOL
    assert errors(outs[0][0].reshape(g["c"], 3, 3, g["kn"]).permute(3, 0, 1, 2).cpu().numpy(),
                  dw_ref.cpu().numpy())[0] < FP32_TOL


def test_resnet_layer_against_fp64(cglib, oracle_lib):
    """A ResNet-50 stage-2 3x3 layer at batch 4, checked on sampled outputs in FP64."""
    cg = cglib
    O = oracle_lib
    g = C.geom(4, 56, 56, 64, 64, 3, 3, pad=1)
    rng = np.random.default_rng(5)
    x = rng.standard_normal(4 * 56 * 56 * 64).astype(np.float32)
    w = (rng.standard_normal(576 * 64) * np.sqrt(2 / 576)).astype(np.float32)
    y = np.zeros(4 * 56 * 56 * 64, np.float32)
    cg.sconvGemmNHWC("N", 4, 56, 56, 64, 64, 3, 3, 1, 1, 1, 1, 1, 1, w, x, y)
    idx = rng.choice(y.size, 4000, replace=False)
    want = O.fwd_points_f64(0, g, w, x, idx)
    assert errors(y[idx], want)[0] < FP32_TOL


def _offset_copy(a, off):
    """A device copy of numpy array `a` whose first element sits `off` floats into its allocation
    (off = 1: 4-byte aligned only, so the kernels' 16-byte vector paths are not taken)."""
    buf = torch.zeros(a.size + off, dtype=torch.float32, device="cuda")
    buf[off:] = torch.from_numpy(a).cuda()
    return buf, buf[off:]


@pytest.mark.parametrize("b,h,w,c,kn,k,stride,dil,pad", [
    (2, 9, 9, 64, 48, 1, 1, 1, 0),     # single tap: 16-byte channel rows of x and dy, 16-byte B rows
    (2, 9, 7, 6, 10, 1, 1, 1, 0),      # single tap, c and kn not multiples of 4: element paths
    (2, 11, 10, 20, 36, 3, 2, 1, 1),   # stride 2: four stride phases of the input gradient
    (1, 13, 12, 8, 12, (3, 3), (3, 2), 2, 2),   # strides 3 x 2 with dilation 2: six phases, uneven taps
    (2, 10, 10, 32, 64, 1, 2, 1, 0),   # 1x1 stride 2: one phase with the tap, three reached by none
])
def test_operand_alignment_and_layout_paths_keep_the_bits(cglib, oracle_lib, b, h, w, c, kn, k, stride, dil, pad):
    """The FP32 kernels read operands through vector or element paths and through NCHW copies or
    repacked weights, chosen by alignment, channel counts and layout; none of that changes the
    arithmetic.  Every operation gives the same bits with 16-byte aligned tensors and with tensors at
    a 4-byte offset, the forward and weight gradient equal the reference-order port, and the
    input gradient (strided ones grouped by stride phase) accumulates within FP32 tolerance of it."""
    kh, kw = (k, k) if isinstance(k, int) else k
    sv, sh = (stride, stride) if isinstance(stride, int) else stride
    g = C.geom(b, h, w, c, kn, kh, kw, vpad=pad, hpad=pad, vstr=sv, hstr=sh, vdil=dil, hdil=dil)
    ho, wo = C.out_hw(g)
    K = c * kh * kw
    rng = np.random.default_rng(b * 7 + c * 3 + kn)
    x = rng.uniform(-1, 1, b * h * w * c).astype(np.float32)
    wt = rng.standard_normal(K * kn).astype(np.float32)
    dy = rng.uniform(-1, 1, b * ho * wo * kn).astype(np.float32)
    dx0 = rng.uniform(-1, 1, b * h * w * c).astype(np.float32)
    bias = rng.uniform(-.1, .1, kn).astype(np.float32)
    cg = cglib
    for layout in (C.NHWC, C.NCHW):
        nhwc = layout == C.NHWC
        conv = cg.sconvGemmNHWC if nhwc else cg.sconvGemmNCHW
        back = cg.sconvGemmNHWC_back if nhwc else cg.sconvGemmNCHW_back
        dims = (b, h, w, c) if nhwc else (b, c, h, w)
        geo = (kn, kh, kw, pad, pad, sv, sh, dil, dil)
        outs = []
        for off in (0, 1):
            keep = []
            dev = lambda a: keep.append(_offset_copy(a, off)) or keep[-1][1]
            y, dw, dx = dev(np.zeros(b * ho * wo * kn, np.float32)), dev(np.zeros(K * kn, np.float32)), dev(dx0)
            conv("N", *dims, *geo, dev(wt), dev(x), y, dev(bias), relu=True)
            conv("T", *dims, *geo, dev(dy), dev(x), dw)
            back(*dims, kn, kh, kw, sv, sh, pad, pad, dil, dil, dev(wt), dev(dy), dx)
            torch.cuda.synchronize()
            outs.append([t.cpu().numpy() for t in (y, dw, dx)])
        for name, a0, a1 in zip(("fwd", "wgrad", "dgrad"), *outs):
            assert bitexact(a0, a1), (layout, name, "aligned and 4-byte-offset operands differ")
        inp = {"x": x, "w": wt, "dy": dy, "dx0": dx0, "epi": {"bias": bias, "relu": True}}
        assert bitexact(outs[0][0], port(oracle_lib, "fwd", layout, g, inp, b * ho * wo * kn)), layout
        assert bitexact(outs[0][1], port(oracle_lib, "wgrad", layout, g, inp, K * kn)), layout
        want = port(oracle_lib, "dgrad", layout, g, inp, None)
        assert errors(outs[0][2], want)[0] <= FP32_TOL, layout


@pytest.mark.parametrize("layout", ["nhwc", "nchw"])
def test_capture_without_scratch_reads_caller_tensors_with_same_bits(cglib, layout):
    """Under stream capture the library allocates nothing.  A call on a capturing stream whose
    scratch (operand copies, repacked weights, split planes) does not exist yet runs the form that
    reads the caller's tensors in their own layouts, in one kernel; replaying the graph gives the
    bits of the eager call, which used the copies."""
    import convgemm_gb300 as cg
    lay = cg.NHWC if layout == "nhwc" else cg.NCHW
    for (b, h, c, kn, k, st) in [(4, 14, 64, 96, 3, 1), (2, 15, 32, 48, 3, 2), (2, 9, 32, 40, 1, 2)]:
        s = cg.Shape.of(b, h, h, c, kn, k, k, k // 2, k // 2, st, st)
        gen = torch.Generator(device="cuda").manual_seed(b * 100 + c + kn)
        x = torch.randn(b * h * h * c, device="cuda", generator=gen)
        w = torch.randn(c * k * k * kn, device="cuda", generator=gen)
        dy = torch.randn(b * s.ho * s.wo * kn, device="cuda", generator=gen)
        bias = torch.randn(kn, device="cuda", generator=gen) * 0.1
        dx_start = torch.randn(b * h * h * c, device="cuda", generator=gen)
        y0, y1 = (torch.empty(b * s.ho * s.wo * kn, device="cuda") for _ in range(2))
        dx0, dx1 = dx_start.clone(), dx_start.clone()
        cg.fwd_f32(lay, s, w, x, y0, bias=bias, relu=True)
        cg.dgrad_f32(lay, s, w, dy, dx0, accumulate=True)
        torch.cuda.synchronize()
        stream = torch.cuda.Stream()   # no scratch exists for this stream yet
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph, stream=stream, capture_error_mode="relaxed"):
            cg.fwd_f32(lay, s, w, x, y1, bias=bias, relu=True)
            cg.dgrad_f32(lay, s, w, dy, dx1, accumulate=True)
        graph.replay()
        torch.cuda.synchronize()
        cg.check_device()
        assert torch.equal(y0.view(torch.int32), y1.view(torch.int32)), (layout, b, h, c, kn, k, st)
        assert torch.equal(dx0.view(torch.int32), dx1.view(torch.int32)), (layout, b, h, c, kn, k, st)
