"""The PyTorch operator convgemm::conv2d_nhwc (forward, and its autograd backward
through the BF16 input- and weight-gradient kernels) in a two-layer network,
against the same network in plain PyTorch FP32 (torch.nn.functional.conv2d on
the BF16-rounded tensors)."""
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL_FWD = 1e-2   # BF16 output rounding of two layers
TOL_GRAD = 3e-2  # plus the BF16 rounding of dY before the gradient kernels


def rel(a, b):
    return ((a.float() - b.float()).abs().max() / b.float().abs().max().clamp_min(1e-30)).item()


def test_two_layer_network_fwd_bwd_against_torch_fp32(cglib):
    from convgemm_gb300 import torch_ops  # noqa: F401  (registers the operator)
    op = torch.ops.convgemm.conv2d_nhwc
    g = torch.Generator(device="cuda").manual_seed(3)
    x = torch.randn(2, 12, 12, 16, device="cuda", generator=g).to(torch.bfloat16).requires_grad_()
    w1 = (torch.randn(16, 3, 3, 32, device="cuda", generator=g) * (2 / 144) ** 0.5).requires_grad_()
    w2 = (torch.randn(32, 3, 3, 24, device="cuda", generator=g) * (2 / 288) ** 0.5).requires_grad_()
    scale = torch.rand(24, device="cuda", generator=g) + 0.5
    shift = torch.rand(24, device="cuda", generator=g) * 0.2 - 0.1
    r = torch.randn(2, 6, 6, 24, device="cuda", generator=g)
    y1 = op(x, w1, None, None, 1, 1, 1, True)
    y2 = op(y1, w2, scale, shift, 2, 1, 1, False)
    (y2.float() * r).sum().backward()
    cglib.check_device()

    # the same network in FP32 PyTorch (NCHW), weights [c][kh][kw][kn] -> [kn][c][kh][kw]
    xr = x.detach().float().permute(0, 3, 1, 2).requires_grad_()
    w1r = w1.detach().to(torch.bfloat16).float().permute(3, 0, 1, 2).contiguous().requires_grad_()
    w2r = w2.detach().to(torch.bfloat16).float().permute(3, 0, 1, 2).contiguous().requires_grad_()
    F = torch.nn.functional
    z1 = torch.relu(F.conv2d(xr, w1r, stride=1, padding=1))
    z2 = F.conv2d(z1, w2r, stride=2, padding=1) * scale[None, :, None, None] + shift[None, :, None, None]
    (z2 * r.permute(0, 3, 1, 2)).sum().backward()
    assert rel(y2, z2.permute(0, 2, 3, 1)) <= TOL_FWD
    assert rel(x.grad, xr.grad.permute(0, 2, 3, 1)) <= TOL_GRAD
    assert rel(w1.grad, w1r.grad.permute(1, 2, 3, 0)) <= TOL_GRAD
    assert rel(w2.grad, w2r.grad.permute(1, 2, 3, 0)) <= TOL_GRAD
