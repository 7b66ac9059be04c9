"""PyTorch operator over the BF16 tensor-core convolution (forward, input gradient,
weight gradient) for training steps written in PyTorch.

`convgemm::conv2d_nhwc` takes a BF16 NHWC activation whose channel count is a
multiple of 8 and FP32 weights in the reference's NHWC-API layout
[c][kh][kw][kn] (src/convGemm.c:66).  It returns BF16 NHWC output
y = relu?(conv(x, w) * scale + shift) (scale / shift per output channel, e.g.
a folded batch norm; None = 1 / 0).  Its backward gives dX (BF16, through
convgemm_dgrad_bf16) and dW (FP32, through convgemm_wgrad_bf16, deterministic)
of the convolution itself (ReLU and the scale apply to dY first).  There is no
fallback: the operator runs the library's kernels or raises.
"""
import weakref
from typing import Optional, Tuple

import torch

from . import NHWC, Shape
from . import tc

_LIB = "convgemm"

# Packed-weight caching for repeated calls on unchanged weights (off by default).  When on,
# a contiguous FP32 weight tensor's packed operands come from the library's cache, keyed
# on its address and re-packed when its _version changes (an optimizer step, any in-place
# write); the entries are evicted when the tensor is freed, before its address can be reused.
_CACHE = {"on": False, "tracked": {}}


def cache_weights(on: bool = True) -> bool:
    """Turns packed-weight caching of the operator on or off; returns the previous setting."""
    prev = _CACHE["on"]
    _CACHE["on"] = bool(on)
    if not on:
        for addr in list(_CACHE["tracked"]):
            tc.weights_cache_evict(addr)
        _CACHE["tracked"].clear()
    return prev


def _evict(addr):
    if _CACHE["tracked"].pop(addr, None) is not None:
        tc.weights_cache_evict(addr)


def _packed(s, kind, w):
    """(packed operand address or tensor, keep-alive) for the FP32 weights w."""
    if _CACHE["on"] and w.is_contiguous() and w.dtype == torch.float32:
        addr = w.data_ptr()
        if addr not in _CACHE["tracked"]:
            _CACHE["tracked"][addr] = weakref.finalize(w, _evict, addr)
        return tc.weights_cached(NHWC, s, kind, w, w._version)
    op = tc.OPERAND_FWD if kind == tc.CACHE_BF16_FWD else tc.OPERAND_DGRAD
    wp = torch.empty(max(1, tc.weights_size(s, op) // 2), dtype=torch.bfloat16, device=w.device)
    tc.pack_weights(NHWC, s, op, w.contiguous(), wp)
    return wp


def _shape(x, w, stride, pad, dil):
    b, h, wd, c = x.shape
    cw, kh, kw, kn = w.shape
    if cw != c:
        raise ValueError(f"weights have {cw} input channels, x has {c}")
    return Shape.of(b, h, wd, c, kn, kh, kw, pad, pad, stride, stride, dil, dil)


@torch.library.custom_op(f"{_LIB}::conv2d_nhwc", mutates_args=())
def conv2d_nhwc(x: torch.Tensor, w: torch.Tensor, scale: Optional[torch.Tensor], shift: Optional[torch.Tensor],
                stride: int, pad: int, dil: int, relu: bool) -> torch.Tensor:
    s = _shape(x, w, stride, pad, dil)
    wp = _packed(s, tc.CACHE_BF16_FWD, w)
    y = torch.empty(s.b, s.ho, s.wo, s.kn, dtype=torch.bfloat16, device=x.device)
    tc.fwd_bf16(s, x.contiguous(), wp, y, scale, shift, relu=relu)
    return y


@conv2d_nhwc.register_fake
def _(x, w, scale, shift, stride, pad, dil, relu):
    b, h, wd, _ = x.shape
    _, kh, kw, kn = w.shape
    ho = (h + 2 * pad - dil * (kh - 1) - 1) // stride + 1
    wo = (wd + 2 * pad - dil * (kw - 1) - 1) // stride + 1
    return x.new_empty(b, ho, wo, kn)


@torch.library.custom_op(f"{_LIB}::conv2d_nhwc_backward", mutates_args=())
def conv2d_nhwc_backward(dy: torch.Tensor, x: torch.Tensor, w: torch.Tensor, stride: int, pad: int,
                         dil: int) -> Tuple[torch.Tensor, torch.Tensor]:
    """(dX BF16 NHWC, dW FP32 [c][kh][kw][kn]) of the bare convolution for the BF16 dY."""
    s = _shape(x, w, stride, pad, dil)
    dy = dy.contiguous()
    dx = torch.empty_like(x)
    wpd = _packed(s, tc.CACHE_BF16_DGRAD, w)
    tc.dgrad_bf16(s, dy, wpd, dx)
    ws = torch.empty(tc.wgrad_bf16_workspace_size(s) // 4 + 1, device=x.device)
    dw = torch.empty_like(w, dtype=torch.float32)
    tc.wgrad_bf16(NHWC, s, dy, x.contiguous(), dw, ws)
    return dx, dw


@conv2d_nhwc_backward.register_fake
def _(dy, x, w, stride, pad, dil):
    return torch.empty_like(x), torch.empty_like(w, dtype=torch.float32)


def _setup(ctx, inputs, output):
    x, w, scale, shift, stride, pad, dil, relu = inputs
    ctx.save_for_backward(x, w, scale, output)
    ctx.conf = (stride, pad, dil, relu)


def _backward(ctx, gy):
    x, w, scale, y = ctx.saved_tensors
    stride, pad, dil, relu = ctx.conf
    g = gy.float()
    if relu:
        g = g * (y > 0)
    if scale is not None:
        g = g * scale
    dx, dw = conv2d_nhwc_backward(g.to(torch.bfloat16), x, w, stride, pad, dil)
    return dx, dw.to(w.dtype), None, None, None, None, None, None


conv2d_nhwc.register_autograd(_backward, setup_context=_setup)
