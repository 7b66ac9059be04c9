"""The allocation-free weight gradient (convgemm_wgrad_bf16_noalloc).

Callers such as code running inside a CUDA-graph stream capture (where
cudaMalloc is not allowed) or services with a memory footprint fixed at
start-up cannot hand the library a workspace.  This entry point keeps its
split partials in a fixed 16 MiB device array instead.  The test calls it
through the C ABI twice in a row, on two different shapes (so a stale partial
left by the first call would show in the second), and checks each result
against the workspace form convgemm_wgrad_bf16 within the weight-gradient
tolerance the other GPU tests use.  This file is collected last on purpose.
"""
import ctypes

import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

WGRAD_TOL = 1e-4   # the FP32-accumulation tolerance of tests/test_gpu_tc.py for weight gradients


def _inputs(tc, s, seed):
    g = torch.Generator(device="cuda").manual_seed(seed)
    x = torch.randn(s.b, s.h, s.w, tc.c8(s.c), device="cuda", generator=g).to(torch.bfloat16)
    dy = torch.randn(s.b, s.ho, s.wo, tc.c8(s.kn), device="cuda", generator=g).to(torch.bfloat16)
    return x, dy


def test_noalloc_wgrad_matches_workspace_form(cglib):
    from convgemm_gb300 import tc
    cg = cglib
    L = cg.lib()
    shapes = [cg.Shape.of(8, 28, 28, 128, 128, 3, 3, 1, 1, 1, 1),   # several splits, dY is the A operand
              cg.Shape.of(4, 14, 14, 64, 64, 3, 3, 1, 1, 2, 2)]      # stride 2, X is the A operand
    for i, s in enumerate(shapes):
        x, dy = _inputs(tc, s, 100 + i)
        K = s.c * s.kh * s.kw
        ws = torch.empty(tc.wgrad_bf16_workspace_size(s) // 4 + 1, device="cuda")
        want = torch.empty(K * s.kn, device="cuda")
        tc.wgrad_bf16(cg.NHWC, s, dy, x, want, ws)
        got = torch.full((K * s.kn,), float("nan"), device="cuda")
        st = L.convgemm_wgrad_bf16_noalloc(cg.NHWC, ctypes.byref(s), dy.data_ptr(), x.data_ptr(), got.data_ptr(),
                                          torch.cuda.current_stream().cuda_stream)
        assert st == 0, cg.last_error()
        torch.cuda.synchronize()
        assert torch.isfinite(got).all()
        err = ((got - want).abs().max() / want.abs().max()).item()
        assert err <= WGRAD_TOL, (i, err)


def test_noalloc_rejects_layers_beyond_its_scratch(cglib):
    cg = cglib
    s = cg.Shape.of(1, 8, 8, 1024, 2048, 3, 3, 1, 1)   # 9*1024*2048 partials > 4 Mi
    dummy = ctypes.c_void_p(16)
    st = cg.lib().convgemm_wgrad_bf16_noalloc(cg.NHWC, ctypes.byref(s), dummy, dummy, dummy, None)
    assert st == 2
    assert "16 MiB" in cg.last_error()[1]
