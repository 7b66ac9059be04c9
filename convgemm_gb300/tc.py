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


def dgrad_bf16_relu(shape: Shape, dy, wpacked, dx, x, stream=None):
    """Input gradient times the derivative of the ReLU that produced x (dx = 0 where x <= 0)."""
    _raise_if(lib().convgemm_dgrad_bf16_relu(ctypes.byref(shape), ptr(dy), ptr(wpacked), ptr(dx), ptr(x),
                                             _stream(stream)))


def dgrad_bf16_ex(shape: Shape, dy, wpacked, dx, relu_x=None, accumulate=False, stream=None):
    """Input gradient; accumulate=True adds into dx (the reference's dx += ...), relu_x masks the result."""
    _raise_if(lib().convgemm_dgrad_bf16_ex(ctypes.byref(shape), ptr(dy), ptr(wpacked), ptr(dx), ptr(relu_x),
                                           int(bool(accumulate)), _stream(stream)))


def dgrad_bf16_bias_grad(shape: Shape, dy, wpacked, dx, db, relu_x=None, workspace=None, stream=None):
    """Input gradient (masked by relu_x > 0 when given) with the column sums of dx fused into its
    epilogue: db[ci] = sum over pixels of dx, the bias gradient of the layer that produced relu_x."""
    import torch
    n = lib().convgemm_dgrad_bf16_bias_grad_workspace_size(ctypes.byref(shape))
    if workspace is None:
        workspace = torch.empty(n // 4 + 4, device=dy.device)
    _raise_if(lib().convgemm_dgrad_bf16_bias_grad(ctypes.byref(shape), ptr(dy), ptr(wpacked), ptr(dx), ptr(relu_x),
                                                  ptr(db), ptr(workspace), workspace.numel() * workspace.element_size(),
                                                  _stream(stream)))


def bias_grad_bf16(shape: Shape, dy, db, workspace=None, stream=None):
    """db[co] = sum over output pixels of dy[p][co] (FP32, fixed order)."""
    import torch
    n = lib().convgemm_bias_grad_bf16_workspace_size(ctypes.byref(shape))
    if workspace is None:
        workspace = torch.empty(n // 4 + 1, device=dy.device)
    _raise_if(lib().convgemm_bias_grad_bf16(ctypes.byref(shape), ptr(dy), ptr(db), ptr(workspace),
                                            workspace.numel() * workspace.element_size(), _stream(stream)))


def fwd_bf16_stats_workspace_size(shape: Shape) -> int:
    return lib().convgemm_fwd_bf16_stats_workspace_size(ctypes.byref(shape))


def fwd_bf16_stats(shape: Shape, x, wpacked, y, stats, scale=None, shift=None, relu=False, workspace=None,
                   stream=None):
    """BF16 forward with the batch statistics of z = conv * scale + shift fused into the
    epilogue: stats (FP64 [2][kn], device) = per-channel sums and sums of squares."""
    import torch
    n = fwd_bf16_stats_workspace_size(shape)
    if workspace is None:
        workspace = torch.empty(n // 8 + 2, dtype=torch.float64, device=x.device)
    _raise_if(lib().convgemm_fwd_bf16_stats(ctypes.byref(shape), ptr(x), ptr(wpacked), ptr(y), ptr(scale),
                                            ptr(shift), int(relu), ptr(stats), ptr(workspace),
                                            workspace.numel() * workspace.element_size(), _stream(stream)))


def bn_stats_fold(kn: int, stats, count: int, scale, shift, gamma=None, beta=None, eps: float = 1e-5,
                  batch_mean=None, batch_var=None, stream=None):
    """scale / shift of training-mode batch norm from the forward's batch statistics."""
    _raise_if(lib().convgemm_bn_stats_fold(kn, ptr(stats), count, ptr(gamma), ptr(beta), eps, ptr(scale),
                                           ptr(shift), ptr(batch_mean), ptr(batch_var), _stream(stream)))


def bn_apply_bf16(npix: int, kn: int, z, scale, shift, y, relu=True, stream=None):
    """y = relu?(z * scale + shift) per channel (BF16 NHWC)."""
    _raise_if(lib().convgemm_bn_apply_bf16(npix, kn, ptr(z), ptr(scale), ptr(shift), int(relu), ptr(y),
                                           _stream(stream)))


def wgrad_bf16_workspace_size(shape: Shape) -> int:
    return lib().convgemm_wgrad_bf16_workspace_size(ctypes.byref(shape))


def wgrad_bf16_plan(shape: Shape):
    """(tile width, pixel splits, largest useful split count) of the weight gradient."""
    bn, sp, mx = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    _raise_if(lib().convgemm_wgrad_bf16_plan(ctypes.byref(shape), ctypes.byref(bn), ctypes.byref(sp),
                                             ctypes.byref(mx)))
    return bn.value, sp.value, mx.value


TUNE_FWD, TUNE_DGRAD, TUNE_WGRAD, TUNE_FWD_FP8, TUNE_FWD_BF16X3 = range(5)
WGRAD_X_ON_A = 0x10000      # weight-gradient aux flags: X as the A operand of a wide layer,
WGRAD_IM2COL_X = 0x20000    # X of a 1x1 stride-1 unpadded layer by im2col instead of tiled boxes
WGRAD_SLAB = 0x80000        # stride-1 layers with 128-channel blocks: the slab kernel
WGRAD_STAGES1 = 0x400000    # im2col path: one chunk per ring stage, twice the stages
WGRAD_TWO_ISSUERS = 0x800000  # im2col path, two chunks per stage: a second MMA-issuing warp
WGRAD_WIDE_CHUNKS = 0x1000000  # im2col path: 128-pixel chunks, one per stage (TMA boxes of twice the bytes)
WGRAD_PAIR = 0x2000000      # im2col path: CTA pairs sharing 256 x 256 / 256 x 128 tiles (cta_group::2 MMAs)
CONV_STAGES1 = 16           # forward / input-gradient aux: one K block per ring stage, twice the stages


def WGRAD_GROUPS(csize: int) -> int:
    """Weight-gradient aux flag: more than 8 splits reduced inside the kernel by clusters of csize (2/4/8)."""
    return {2: 0x100000, 4: 0x200000, 8: 0x300000}[csize]


def tune_set(op: int, shape: Shape, bn: int = 0, splits: int = 0):
    """Overrides the tile heuristics for one operation on one shape (0, 0 removes the entry)."""
    _raise_if(lib().convgemm_tune_set(op, ctypes.byref(shape), bn, splits))


def tune_describe(op: int, shape: Shape):
    """(kernel, bn, stages, cluster) that the tuning entry or heuristic selects for op on shape:
    kernel 0 general / 1 slab / 2 small-channel; stages 0 where buffers are sized at run time."""
    v = [ctypes.c_int() for _ in range(4)]
    _raise_if(lib().convgemm_tune_describe(op, ctypes.byref(shape), *[ctypes.byref(x) for x in v]))
    return tuple(x.value for x in v)


def tune_clear():
    lib().convgemm_tune_clear()


def wgrad_bf16(layout, shape: Shape, dy, x, dw, workspace, stream=None):
    nbytes = workspace.numel() * workspace.element_size()
    _raise_if(lib().convgemm_wgrad_bf16(layout, ctypes.byref(shape), ptr(dy), ptr(x), ptr(dw), ptr(workspace),
                                        nbytes, _stream(stream)))


# ------------------------------------------------------------- FP8-E4M3 form
def fp8_quantize(x, out, scale2, stream=None):
    """Per-tensor E4M3 quantisation; scale2 is a 2-float device tensor (scale, scratch)."""
    in_bf16 = 1 if str(x.dtype) == "torch.bfloat16" else 0
    _raise_if(lib().convgemm_fp8_quantize(x.numel(), in_bf16, ptr(x), ptr(out), ptr(scale2), _stream(stream)))


def fp8_weights_size(shape: Shape) -> int:
    return lib().convgemm_fp8_weights_size(ctypes.byref(shape))


def fp8_pack_weights(layout, shape: Shape, weights, packed, wscale, stream=None):
    _raise_if(lib().convgemm_fp8_pack_weights(layout, ctypes.byref(shape), ptr(weights), ptr(packed), ptr(wscale),
                                              _stream(stream)))


def fp8_epilogue_scales(kn, scale, shift, wscale, xscale, out_scale, out_shift, stream=None):
    _raise_if(lib().convgemm_fp8_epilogue_scales(kn, ptr(scale), ptr(shift), ptr(wscale), ptr(xscale),
                                                 ptr(out_scale), ptr(out_shift), _stream(stream)))


def fwd_fp8(shape: Shape, x, wpacked, y, scale, shift=None, relu=False, stream=None):
    _raise_if(lib().convgemm_fwd_fp8(ctypes.byref(shape), ptr(x), ptr(wpacked), ptr(y), ptr(scale), ptr(shift),
                                     int(bool(relu)), _stream(stream)))


# ------------------------------------------------------------- 3xBF16 form
def split_bf16x2(x, hi, lo, stream=None):
    _raise_if(lib().convgemm_split_bf16x2(x.numel(), ptr(x), ptr(hi), ptr(lo), _stream(stream)))


def bf16x3_pack_weights(layout, shape: Shape, weights, hi, lo, stream=None):
    _raise_if(lib().convgemm_bf16x3_pack_weights(layout, ctypes.byref(shape), ptr(weights), ptr(hi), ptr(lo),
                                                 _stream(stream)))


def fwd_bf16x3(shape: Shape, x_hi, x_lo, w_hi, w_lo, y, scale=None, shift=None, relu=False, stream=None):
    _raise_if(lib().convgemm_fwd_bf16x3(ctypes.byref(shape), ptr(x_hi), ptr(x_lo), ptr(w_hi), ptr(w_lo), ptr(y),
                                        ptr(scale), ptr(shift), int(bool(relu)), _stream(stream)))


# ------------------------------------------------ grouped persistent forward launch
class GroupConv(ctypes.Structure):
    """convgemm_group_conv_t (include/convgemm_gpu.h)."""
    _fields_ = [("shape", Shape), ("x", ctypes.c_void_p), ("w", ctypes.c_void_p), ("y", ctypes.c_void_p),
                ("scale", ctypes.c_void_p), ("shift", ctypes.c_void_p), ("relu", ctypes.c_int), ("bn", ctypes.c_int)]


CACHE_BF16_FWD, CACHE_BF16_DGRAD, CACHE_FP8_FWD = 0, 1, 2


def weights_cached(layout, shape: Shape, kind: int, weights, version: int, stream=None):
    """Device address of the cached packed operand of FP32 `weights` (re-packed only when
    `version` changed since it was packed); for CACHE_FP8_FWD, (packed, wscale) addresses."""
    packed, wscale = ctypes.c_void_p(), ctypes.c_void_p()
    _raise_if(lib().convgemm_weights_cached(layout, ctypes.byref(shape), kind, ptr(weights),
                                            ctypes.c_ulonglong(version), ctypes.byref(packed),
                                            ctypes.byref(wscale), _stream(stream)))
    return (packed.value, wscale.value) if kind == CACHE_FP8_FWD else packed.value


def weights_cache_evict(weights=None) -> int:
    """Frees the cached operands of `weights` (all entries when None); returns how many."""
    return lib().convgemm_weights_cache_evict(ptr(weights) if weights is not None else None)


def weights_cache_bytes() -> int:
    return lib().convgemm_weights_cache_bytes()


def group_weights_size(shape: Shape) -> int:
    return lib().convgemm_group_weights_size(ctypes.byref(shape))


def group_pack_weights(layout, shape: Shape, weights, packed, stream=None):
    _raise_if(lib().convgemm_group_pack_weights(layout, ctypes.byref(shape), ptr(weights), ptr(packed),
                                                _stream(stream)))


class Group:
    """Many BF16 NHWC forward convolutions run by one persistent launch.

    convs: sequence of dicts with keys shape, x, w (packed by group_pack_weights),
    y, and optionally scale, shift, relu, bn (64/128/256 output channels per tile;
    0 lets the library choose).  The tensor maps are encoded once here; launch()
    may be captured in a CUDA graph.  The tensors must stay alive and in place.
    """

    def __init__(self, convs, device="cuda"):
        import torch
        n = len(convs)
        arr = (GroupConv * n)()
        for i, c in enumerate(convs):
            arr[i] = GroupConv(c["shape"], ptr(c["x"]), ptr(c["w"]), ptr(c["y"]), ptr(c.get("scale")),
                               ptr(c.get("shift")), int(bool(c.get("relu", False))), int(c.get("bn", 0)))
        nbytes = lib().convgemm_group_table_size(n)
        self.table = torch.empty(nbytes + 64, dtype=torch.uint8, device=device)
        off = (-self.table.data_ptr()) % 64
        self._tptr = self.table.data_ptr() + off
        tiles = ctypes.c_int(0)
        _raise_if(lib().convgemm_group_prepare(n, ctypes.cast(arr, ctypes.c_void_p), self._tptr, nbytes,
                                               ctypes.byref(tiles)))
        self.n, self.tiles = n, tiles.value
        self._keep = convs

    def launch(self, stream=None):
        _raise_if(lib().convgemm_group_launch(self._tptr, self.n, self.tiles, _stream(stream)))


# ------------------------------------------------------ grouped weight preparation
class PrepItem(ctypes.Structure):
    """convgemm_prep_item_t (include/convgemm_gpu.h)."""
    _fields_ = [("layout", ctypes.c_int), ("shape", Shape), ("weights", ctypes.c_void_p),
                ("packed_fwd", ctypes.c_void_p), ("packed_dgrad", ctypes.c_void_p), ("epi", Epilogue),
                ("scale", ctypes.c_void_p), ("shift", ctypes.c_void_p)]


class Prep:
    """Batch-norm folds and weight packings of many layers in one launch.

    items: dicts with layout, shape, weights and any of packed_fwd, packed_dgrad,
    scale + shift (with bias / mean / inv_std / gamma / beta).  The job table is
    built once here; launch() may be captured in a CUDA graph.
    """

    def __init__(self, items, device="cuda"):
        import torch
        n = len(items)
        arr = (PrepItem * n)()
        for i, it in enumerate(items):
            e = Epilogue(ptr(it.get("bias")), ptr(it.get("mean")), ptr(it.get("inv_std")), ptr(it.get("gamma")),
                         ptr(it.get("beta")), 0)
            arr[i] = PrepItem(int(it["layout"]), it["shape"], ptr(it.get("weights")), ptr(it.get("packed_fwd")),
                              ptr(it.get("packed_dgrad")), e, ptr(it.get("scale")), ptr(it.get("shift")))
        nbytes = lib().convgemm_prep_table_size(n)
        self.table = torch.empty(nbytes + 16, dtype=torch.uint8, device=device)
        self._tptr = self.table.data_ptr() + (-self.table.data_ptr()) % 16
        nj, nb = ctypes.c_int(0), ctypes.c_int(0)
        _raise_if(lib().convgemm_prep_prepare(n, ctypes.cast(arr, ctypes.c_void_p), self._tptr, nbytes,
                                              ctypes.byref(nj), ctypes.byref(nb)))
        self.njobs, self.nblocks = nj.value, nb.value
        self._keep = items

    def launch(self, stream=None):
        _raise_if(lib().convgemm_prep_launch(self._tptr, self.njobs, self.nblocks, _stream(stream)))
