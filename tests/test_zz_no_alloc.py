"""The allocation-free weight gradient (convgemm_wgrad_bf16_noalloc).

Some callers of this library cannot hand it a workspace: code that runs while a
stream is being captured into a CUDA graph, where cudaMalloc is not permitted,
and services that fix their GPU memory footprint at start-up so that nothing can
fail or fragment later.  This entry point keeps its split partials in a fixed
16 MiB device array instead.  These tests call it through the C ABI, one shape
after another (each call reuses the array the previous call left behind), and
check every result against the workspace form convgemm_wgrad_bf16 within the
weight-gradient tolerance of the other GPU tests.  The shapes cover each way the
partials are combined: one split written directly, 2-8 splits reduced inside a
thread-block cluster, 9-16 splits summed by one reduction pass, more than 16 in
two passes, and a split count cut down by the size of the array.  The stem shape
(3 channels, 7x7, stride 2), which the workspace form runs through a different
kernel, is checked against the FP64 oracle as well.  This file is collected last
on purpose.
"""
import ctypes
import gc

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

WGRAD_TOL = 1e-4   # the FP32-accumulation tolerance of tests/test_gpu_tc.py for weight gradients
SCRATCH_FLOATS = 4 << 20


def _inputs(tc, s, seed):
    g = torch.Generator(device="cuda").manual_seed(seed)
    x = torch.randn(s.b, s.h, s.w, tc.c8(s.c), device="cuda", generator=g)
    x[..., s.c:] = 0
    x = x.to(torch.bfloat16)
    dy = torch.randn(s.b, s.ho, s.wo, tc.c8(s.kn), device="cuda", generator=g).to(torch.bfloat16)
    return x, dy


def _noalloc(cg, layout, s, dy, x, out):
    st = cg.lib().convgemm_wgrad_bf16_noalloc(layout, ctypes.byref(s), dy.data_ptr(), x.data_ptr(), out.data_ptr(),
                                              torch.cuda.current_stream().cuda_stream)
    assert st == 0, cg.last_error()


def _workspace_form(tc, layout, s, dy, x):
    K = s.c * s.kh * s.kw
    ws = torch.empty(tc.wgrad_bf16_workspace_size(s) // 4 + 1, device="cuda")
    want = torch.empty(K * s.kn, device="cuda")
    tc.wgrad_bf16(layout, s, dy, x, want, ws)
    return want


# (shape, how the no-allocation call combines its splits)
SHAPES = [
    ((8, 28, 28, 128, 128, 3, 3, 1, 1), "9-16 splits, one reduction pass"),
    ((2, 28, 28, 128, 128, 3, 3, 1, 1), "2-8 splits in a cluster"),
    ((4, 14, 14, 64, 64, 3, 3, 1, 1, 2, 2), "one split, dW written directly"),
    ((8, 56, 56, 64, 64, 1, 1), "more than 16 splits, two passes"),
    ((32, 28, 28, 128, 256, 3, 3, 1, 1), "splits capped by the scratch"),
]


def test_noalloc_split_plans_cover_every_reduction(cglib):
    """The shapes above do reach the reduction forms named beside them."""
    from convgemm_gb300 import tc
    cg = cglib
    for dims, what in SHAPES:
        s = cg.Shape.of(*dims)
        Nx = s.kh * s.kw * tc.c8(s.c)
        tile = Nx * s.kn
        if "capped" in what:
            assert tile * 16 > SCRATCH_FLOATS, (dims, "scratch would not cap this shape")
        P = s.b * s.ho * s.wo
        if "more than 16" in what:
            assert (P + 63) // 64 // 8 > 16


@pytest.mark.parametrize("layout", [0, 1], ids=["nhwc", "nchw"])
def test_noalloc_wgrad_matches_workspace_form(cglib, layout):
    from convgemm_gb300 import tc
    cg = cglib
    for i, (dims, what) in enumerate(SHAPES):
        s = cg.Shape.of(*dims)
        x, dy = _inputs(tc, s, 100 + i)
        want = _workspace_form(tc, layout, s, dy, x)
        # two calls in a row: the second reads only what it wrote itself
        for rep in range(2):
            got = torch.full_like(want, float("nan"))
            _noalloc(cg, layout, s, dy, x, got)
            torch.cuda.synchronize()
            cg.check_device()
            assert torch.isfinite(got).all(), (what, rep)
            err = ((got - want).abs().max() / want.abs().max()).item()
            assert err <= WGRAD_TOL, (what, rep, err)


def test_noalloc_stem_against_fp64_oracle(cglib, oracle_lib):
    """The 3-channel 7x7 stride-2 stem, which the workspace form sends to its slab kernel."""
    from convgemm_gb300 import tc
    cg, O = cglib, oracle_lib
    s = cg.Shape.of(2, 112, 112, 3, 64, 7, 7, 3, 3, 2, 2)
    x, dy = _inputs(tc, s, 7)
    got = torch.empty(3 * 49 * 64, device="cuda")
    _noalloc(cg, cg.NHWC, s, dy, x, got)
    torch.cuda.synchronize()
    cg.check_device()
    xf = np.ascontiguousarray(x[..., :3].float().cpu().numpy()).ravel()
    dyf = np.ascontiguousarray(dy.float().cpu().numpy()).ravel()
    want = O.wgrad_f64(O.NHWC, s.as_dict(), dyf, xf)
    g = got.cpu().numpy().astype(np.float64)
    err = np.abs(g - want).max() / np.abs(want).max()
    assert err <= WGRAD_TOL, err
    ws_form = _workspace_form(tc, cg.NHWC, s, dy, x).cpu().numpy().astype(np.float64)
    assert np.abs(ws_form - want).max() / np.abs(want).max() <= WGRAD_TOL


def test_noalloc_allocates_nothing(cglib):
    """A repeated call changes neither torch's allocation count nor the device's free memory."""
    from convgemm_gb300 import tc
    cg = cglib
    s = cg.Shape.of(8, 28, 28, 128, 128, 3, 3, 1, 1)
    x, dy = _inputs(tc, s, 3)
    out = torch.empty(s.c * 9 * s.kn, device="cuda")
    _noalloc(cg, cg.NHWC, s, dy, x, out)   # the first call of this shape loads its kernels
    torch.cuda.synchronize()
    gc.collect()   # tensors of earlier tests freed now, not during the measured call
    torch.cuda.synchronize()
    a0, (f0, _) = torch.cuda.memory_allocated(), torch.cuda.mem_get_info()
    _noalloc(cg, cg.NHWC, s, dy, x, out)
    torch.cuda.synchronize()
    a1, (f1, _) = torch.cuda.memory_allocated(), torch.cuda.mem_get_info()
    assert a1 == a0 and f1 == f0, (a0, a1, f0, f1)


def test_noalloc_rejects_layers_beyond_its_scratch(cglib):
    cg = cglib
    s = cg.Shape.of(1, 8, 8, 1024, 2048, 3, 3, 1, 1)   # 9*1024*2048 partials > 4 Mi
    dummy = ctypes.c_void_p(16)
    st = cg.lib().convgemm_wgrad_bf16_noalloc(cg.NHWC, ctypes.byref(s), dummy, dummy, dummy, None)
    assert st == 2
    assert "16 MiB" in cg.last_error()[1]


def test_noalloc_rejects_filters_without_a_kernel(cglib):
    """Filters above 49 taps are refused here exactly as by the workspace form."""
    cg = cglib
    s = cg.Shape.of(1, 16, 16, 8, 8, 8, 8, 3, 3)   # 64 taps
    dummy = ctypes.c_void_p(16)
    st = cg.lib().convgemm_wgrad_bf16_noalloc(cg.NHWC, ctypes.byref(s), dummy, dummy, dummy, None)
    assert st == 2
    assert "49 taps" in cg.last_error()[1]
