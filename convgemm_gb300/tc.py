"""BF16 tensor-core forms (tcgen05, FP32 accumulation in TMEM) of the convGemm path.

Thin wrappers over the convgemm_*_bf16 entry points of include/convgemm_gpu.h;
tensors are torch CUDA tensors (NHWC, BF16 activations, FP32 weights before
packing).  Nothing here falls back to another implementation.
"""
from __future__ import annotations

import ctypes

from . import Epilogue, Shape, _raise_if, _stream, lib, ptr

OPERAND_FWD, OPERAND_DGRAD = 0, 1


def c8(c: int) -> int:
    return (c + 7) // 8 * 8


def weights_size(shape: Shape, kind: int) -> int:
    return lib().convgemm_bf16_weights_size(ctypes.byref(shape), kind)


def pack_weights(layout, shape: Shape, kind: int, weights, packed, stream=None):
    _raise_if(lib().convgemm_bf16_pack_weights(layout, ctypes.byref(shape), kind, ptr(weights), ptr(packed),
                                               _stream(stream)))


def fold_epilogue(kn, scale, shift, bias=None, mean=None, inv_std=None, gamma=None, beta=None, stream=None):
    e = Epilogue(ptr(bias), ptr(mean), ptr(inv_std), ptr(gamma), ptr(beta), 0)
    _raise_if(lib().convgemm_fold_epilogue(kn, ctypes.byref(e), ptr(scale), ptr(shift), _stream(stream)))


def to_bf16_nhwc(layout, b, c, h, w, x, out, stream=None):
    _raise_if(lib().convgemm_to_bf16_nhwc(layout, b, c, h, w, ptr(x), ptr(out), _stream(stream)))


def fwd_bf16(shape: Shape, x, wpacked, y, scale=None, shift=None, relu=False, stream=None):
    _raise_if(lib().convgemm_fwd_bf16(ctypes.byref(shape), ptr(x), ptr(wpacked), ptr(y), ptr(scale), ptr(shift),
                                      int(bool(relu)), _stream(stream)))


def dgrad_bf16(shape: Shape, dy, wpacked, dx, stream=None):
    _raise_if(lib().convgemm_dgrad_bf16(ctypes.byref(shape), ptr(dy), ptr(wpacked), ptr(dx), _stream(stream)))


def wgrad_bf16_workspace_size(shape: Shape) -> int:
    return lib().convgemm_wgrad_bf16_workspace_size(ctypes.byref(shape))


def wgrad_bf16(layout, shape: Shape, dy, x, dw, workspace, stream=None):
    nbytes = workspace.numel() * workspace.element_size()
    _raise_if(lib().convgemm_wgrad_bf16(layout, ctypes.byref(shape), ptr(dy), ptr(x), ptr(dw), ptr(workspace),
                                        nbytes, _stream(stream)))
