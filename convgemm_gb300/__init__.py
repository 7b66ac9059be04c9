"""convgemm_gb300 — GB300 (sm_103a) implicit-GEMM convolution behind convGemm's C entry points.

The compute lives in ``libconvGemm.so`` (hand-written CUDA, built in-tree by
``convgemm_gb300.build``).  This package is the Python side of that C ABI:

* ``alloc_pack_buffs``, ``sconvGemmNHWC``, ``sconvGemmNHWC_back``, ``sconvGemmNCHW``,
  ``sconvGemmNCHW_back`` mirror the reference's five functions (hpca-uji/convGemm
  src/convGemm.h:20-64) argument for argument, the way a ctypes caller such as
  PyDTNN binds them; they accept numpy arrays (host memory, staged by the
  library) or torch tensors (device memory used in place);
* ``fwd_f32``/``wgrad_f32``/``dgrad_f32`` and the tensor-core forms in
  ``convgemm_gb300.tc`` wrap the extended API of ``include/convgemm_gpu.h``
  (explicit stream, status codes, workspaces).

There is no fallback: if the library is missing, importing the ops raises.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libconvGemm.so")

NHWC, NCHW = 0, 1

STATUS = {0: "SUCCESS", 1: "INVALID_VALUE", 2: "NOT_SUPPORTED", 3: "CUDA", 4: "ALLOC", 5: "TIMEOUT", 6: "WORKSPACE"}


class ConvGemmError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"convgemm {STATUS.get(status, status)}: {message}")
        self.status = status


class Shape(ctypes.Structure):
    """convgemm_shape_t (include/convgemm_gpu.h)."""
    _fields_ = [(n, ctypes.c_int) for n in
                ("b", "h", "w", "c", "kn", "kh", "kw", "vpad", "hpad", "vstride", "hstride", "vdil", "hdil")]

    @classmethod
    def of(cls, b, h, w, c, kn, kh, kw, vpad=0, hpad=0, vstride=1, hstride=1, vdil=1, hdil=1):
        return cls(b, h, w, c, kn, kh, kw, vpad, hpad, vstride, hstride, vdil, hdil)

    @property
    def ho(self):
        return (self.h + 2 * self.vpad - self.vdil * (self.kh - 1) - 1) // self.vstride + 1

    @property
    def wo(self):
        return (self.w + 2 * self.hpad - self.hdil * (self.kw - 1) - 1) // self.hstride + 1

    def as_dict(self):
        return {"b": self.b, "h": self.h, "w": self.w, "c": self.c, "kn": self.kn, "kh": self.kh, "kw": self.kw,
                "vpad": self.vpad, "hpad": self.hpad, "vstr": self.vstride, "hstr": self.hstride,
                "vdil": self.vdil, "hdil": self.hdil}


class Epilogue(ctypes.Structure):
    """convgemm_epilogue_t (include/convgemm_gpu.h)."""
    _fields_ = [("bias", ctypes.c_void_p), ("mean", ctypes.c_void_p), ("inv_std", ctypes.c_void_p),
                ("gamma", ctypes.c_void_p), ("beta", ctypes.c_void_p), ("relu", ctypes.c_int)]


_lib = None

_VP = ctypes.c_void_p
_I = ctypes.c_int
_FWD_ARGS = [ctypes.c_char] + [_I] * 13 + [_VP] * 8 + [ctypes.c_bool, _VP, _VP]
_BACK_ARGS = [_I] * 13 + [_VP] * 5


def lib():
    """The loaded libconvGemm.so; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with `python -m convgemm_gb300.build` "
                               "(there is no CPU fallback)")
        L = ctypes.CDLL(LIB_PATH)
        L.alloc_pack_buffs.argtypes = [ctypes.POINTER(_VP), ctypes.POINTER(_VP)]
        L.alloc_pack_buffs.restype = _I
        for n in ("sconvGemmNHWC", "sconvGemmNCHW"):
            getattr(L, n).argtypes = _FWD_ARGS
            getattr(L, n).restype = None
        for n in ("sconvGemmNHWC_back", "sconvGemmNCHW_back"):
            getattr(L, n).argtypes = _BACK_ARGS
            getattr(L, n).restype = None
        L.convgemm_get_last_status.restype = _I
        L.convgemm_get_last_error.restype = ctypes.c_char_p
        L.convgemm_check_device.argtypes = [_VP]
        SP, EP = ctypes.POINTER(Shape), ctypes.POINTER(Epilogue)
        L.convgemm_fwd_f32.argtypes = [_I, SP, _VP, _VP, _VP, EP, _VP]
        L.convgemm_wgrad_f32_workspace_size.argtypes = [SP]
        L.convgemm_wgrad_f32_workspace_size.restype = ctypes.c_size_t
        L.convgemm_wgrad_f32.argtypes = [_I, SP, _VP, _VP, _VP, _VP, ctypes.c_size_t, _VP]
        L.convgemm_dgrad_f32.argtypes = [_I, SP, _VP, _VP, _VP, _I, _VP]
        L.convgemm_bf16_weights_size.argtypes = [SP, _I]
        L.convgemm_bf16_weights_size.restype = ctypes.c_size_t
        L.convgemm_bf16_pack_weights.argtypes = [_I, SP, _I, _VP, _VP, _VP]
        L.convgemm_fold_epilogue.argtypes = [_I, EP, _VP, _VP, _VP]
        L.convgemm_to_bf16_nhwc.argtypes = [_I, _I, _I, _I, _I, _VP, _VP, _VP]
        L.convgemm_fwd_bf16.argtypes = [SP, _VP, _VP, _VP, _VP, _VP, _I, _VP]
        L.convgemm_dgrad_bf16.argtypes = [SP, _VP, _VP, _VP, _VP]
        L.convgemm_wgrad_bf16_workspace_size.argtypes = [SP]
        L.convgemm_wgrad_bf16_workspace_size.restype = ctypes.c_size_t
        L.convgemm_wgrad_bf16.argtypes = [_I, SP, _VP, _VP, _VP, _VP, ctypes.c_size_t, _VP]
        L.convgemm_wgrad_bf16_noalloc.argtypes = [_I, SP, _VP, _VP, _VP, _VP]
        L.convgemm_fp8_quantize.argtypes = [ctypes.c_size_t, _I, _VP, _VP, _VP, _VP]
        L.convgemm_fp8_weights_size.argtypes = [SP]
        L.convgemm_fp8_weights_size.restype = ctypes.c_size_t
        L.convgemm_fp8_pack_weights.argtypes = [_I, SP, _VP, _VP, _VP, _VP]
        L.convgemm_fp8_epilogue_scales.argtypes = [_I, _VP, _VP, _VP, _VP, _VP, _VP, _VP]
        L.convgemm_fwd_fp8.argtypes = [SP, _VP, _VP, _VP, _VP, _VP, _I, _VP]
        L.convgemm_split_bf16x2.argtypes = [ctypes.c_size_t, _VP, _VP, _VP, _VP]
        L.convgemm_bf16x3_pack_weights.argtypes = [_I, SP, _VP, _VP, _VP, _VP]
        L.convgemm_fwd_bf16x3.argtypes = [SP, _VP, _VP, _VP, _VP, _VP, _VP, _VP, _I, _VP]
        L.convgemm_launch_count.restype = ctypes.c_ulonglong
        L.convgemm_set_pdl.argtypes = [_I]
        L.convgemm_set_pdl.restype = _I
        L.convgemm_dgrad_bf16_relu.argtypes = [SP, _VP, _VP, _VP, _VP, _VP]
        L.convgemm_dgrad_bf16_ex.argtypes = [SP, _VP, _VP, _VP, _VP, _I, _VP]
        L.convgemm_selftest_wait_timeout.argtypes = [ctypes.c_uint, _VP]
        L.convgemm_bias_grad_bf16_workspace_size.argtypes = [SP]
        L.convgemm_bias_grad_bf16_workspace_size.restype = ctypes.c_size_t
        L.convgemm_bias_grad_bf16.argtypes = [SP, _VP, _VP, _VP, ctypes.c_size_t, _VP]
        L.convgemm_fwd_bf16_stats_workspace_size.argtypes = [SP]
        L.convgemm_fwd_bf16_stats_workspace_size.restype = ctypes.c_size_t
        L.convgemm_fwd_bf16_stats.argtypes = [SP, _VP, _VP, _VP, _VP, _VP, _I, _VP, _VP, ctypes.c_size_t, _VP]
        L.convgemm_bn_stats_fold.argtypes = [_I, _VP, ctypes.c_longlong, _VP, _VP, ctypes.c_float, _VP, _VP, _VP,
                                             _VP, _VP]
        L.convgemm_bn_apply_bf16.argtypes = [ctypes.c_longlong, _I, _VP, _VP, _VP, _I, _VP, _VP]
        _HG = [_I] * 14
        L.im2row_nhwc.argtypes = [_VP, _I, _VP] + _HG
        L.im2col_nchw.argtypes = [_VP, _I, _VP] + _HG
        L.row2im_nhwc.argtypes = [_I, _I, _VP, _I, _VP] + _HG
        L.col2im_nchw.argtypes = [_I, _I, _VP, _I, _VP] + _HG
        L.transpose_nchw.argtypes = [_I, _I, _VP, _I, ctypes.c_float, _VP, _I, _I, _I, _I, _I]
        L.convgemm_tune_set.argtypes = [_I, SP, _I, _I]
        L.convgemm_wgrad_bf16_plan.argtypes = [SP, ctypes.POINTER(_I), ctypes.POINTER(_I), ctypes.POINTER(_I)]
        L.convgemm_prep_table_size.argtypes = [_I]
        L.convgemm_prep_table_size.restype = ctypes.c_size_t
        L.convgemm_prep_prepare.argtypes = [_I, _VP, _VP, ctypes.c_size_t, ctypes.POINTER(_I), ctypes.POINTER(_I)]
        L.convgemm_prep_launch.argtypes = [_VP, _I, _I, _VP]
        L.convgemm_group_weights_size.argtypes = [SP]
        L.convgemm_group_weights_size.restype = ctypes.c_size_t
        L.convgemm_group_pack_weights.argtypes = [_I, SP, _VP, _VP, _VP]
        L.convgemm_group_table_size.argtypes = [_I]
        L.convgemm_group_table_size.restype = ctypes.c_size_t
        L.convgemm_group_prepare.argtypes = [_I, _VP, _VP, ctypes.c_size_t, ctypes.POINTER(_I)]
        L.convgemm_group_launch.argtypes = [_VP, _I, _I, _VP]
        L.convgemm_weights_cached.argtypes = [_I, SP, _I, _VP, ctypes.c_ulonglong, ctypes.POINTER(_VP),
                                              ctypes.POINTER(_VP), _VP]
        L.convgemm_weights_cache_evict.argtypes = [_VP]
        L.convgemm_weights_cache_evict.restype = _I
        L.convgemm_weights_cache_bytes.restype = ctypes.c_size_t
        L.convgemm_measure_ffma.argtypes = [_I, _VP, ctypes.POINTER(ctypes.c_double), _VP]
        L.convgemm_tune_describe.argtypes = [_I, SP] + [ctypes.POINTER(_I)] * 4
        L.convgemm_dgrad_bf16_bias_grad_workspace_size.argtypes = [SP]
        L.convgemm_dgrad_bf16_bias_grad_workspace_size.restype = ctypes.c_size_t
        L.convgemm_dgrad_bf16_bias_grad.argtypes = [SP, _VP, _VP, _VP, _VP, _VP, _VP, ctypes.c_size_t, _VP]
        _lib = L
    return _lib


# ---------------------------------------------- explicit lowering helpers (drop-in)
def _check_void():
    st, msg = last_error()
    if st:
        lib().convgemm_clear_error()
        raise ConvGemmError(st, msg)


def im2row_nhwc(rows, ld, x, b, h, w, c, ho, wo, kh, kw, vpad, hpad, vstr, hstr, vdil, hdil):
    """rows[(b,x,y)][(c,kx,ky)] = x[b][ix][iy][c] (src/im2row_nhwc.c:147-170)."""
    lib().convgemm_clear_error()
    lib().im2row_nhwc(ptr(rows), ld, ptr(x), b, h, w, c, ho, wo, kh, kw, vpad, hpad, vstr, hstr, vdil, hdil)
    _check_void()


def row2im_nhwc(m, n, rows, ld, out, b, h, w, c, ho, wo, kh, kw, vpad, hpad, vstr, hstr, vdil, hdil):
    """out[b][ix][iy][c] += rows[...] (src/im2row_nhwc.c:210-229)."""
    lib().convgemm_clear_error()
    lib().row2im_nhwc(m, n, ptr(rows), ld, ptr(out), b, h, w, c, ho, wo, kh, kw, vpad, hpad, vstr, hstr, vdil, hdil)
    _check_void()


def im2col_nchw(cols, ld, x, b, c, h, w, ho, wo, kh, kw, vpad, hpad, vstr, hstr, vdil, hdil):
    """cols[(c,kx,ky)][(b,x,y)] = x[b][c][ix][iy] (src/im2col_nchw.c:146-170)."""
    lib().convgemm_clear_error()
    lib().im2col_nchw(ptr(cols), ld, ptr(x), b, c, h, w, ho, wo, kh, kw, vpad, hpad, vstr, hstr, vdil, hdil)
    _check_void()


def col2im_nchw(m, n, cols, ld, out, b, c, h, w, ho, wo, kh, kw, vpad, hpad, vstr, hstr, vdil, hdil):
    """out[b][c][ix][iy] += cols[...] (src/im2col_nchw.c:337-359)."""
    lib().convgemm_clear_error()
    lib().col2im_nchw(m, n, ptr(cols), ld, ptr(out), b, c, h, w, ho, wo, kh, kw, vpad, hpad, vstr, hstr, vdil, hdil)
    _check_void()


def transpose_nchw(rows, cols, x, ld, beta, out, kn, ho, wo, start_row, start_col):
    """out[b][start_col + j][x][y] = x[j*ld + i] (+ beta*out) (src/im2col_nchw.c:208-233)."""
    lib().convgemm_clear_error()
    lib().transpose_nchw(rows, cols, ptr(x), ld, beta, ptr(out), kn, ho, wo, start_row, start_col)
    _check_void()


def launch_count() -> int:
    """Kernels launched (or captured) by the library so far in this process."""
    return int(lib().convgemm_launch_count())


def set_pdl(on: int) -> int:
    """Programmatic dependent launch of the persistent chain kernels for this host
    thread: 1 on, 0 off, -1 default (on unless CONVGEMM_NO_PDL=1).  Returns the
    previous setting.  Turn it off while other streams run work beside the chain."""
    return int(lib().convgemm_set_pdl(int(on)))


def last_error() -> tuple[int, str]:
    L = lib()
    return L.convgemm_get_last_status(), (L.convgemm_get_last_error() or b"").decode()


def _raise_if(status: int):
    if status:
        raise ConvGemmError(status, last_error()[1])


def _check_dropin():
    st, msg = last_error()
    lib().convgemm_clear_error()
    if st:
        raise ConvGemmError(st, msg)


def ptr(t):
    """Address of a numpy array or torch tensor (None -> NULL)."""
    if t is None:
        return None
    if isinstance(t, int):   # a device address returned by the library (e.g. a cached operand)
        return t
    if hasattr(t, "data_ptr"):
        if not t.is_contiguous():
            raise ValueError("tensor must be contiguous")
        return t.data_ptr()
    if not t.flags.c_contiguous:
        raise ValueError("array must be C-contiguous")
    return t.ctypes.data


# ------------------------------------------------- reference-API mirror
def alloc_pack_buffs():
    """int alloc_pack_buffs(float**, float**): returns (0, None, None); the GPU needs no pack buffers."""
    a, b = _VP(), _VP()
    rc = lib().alloc_pack_buffs(ctypes.byref(a), ctypes.byref(b))
    return rc, a.value, b.value


def sconvGemmNHWC(trans, b, h, w, c, kn, kh, kw, vpadding, hpadding, vstride, hstride, vdilation, hdilation,
                  in_, x, out, bias_vector=None, bn_running_mean=None, bn_inv_std=None, bn_gamma=None,
                  bn_beta=None, relu=False, ac_pack=None, bc_pack=None):
    """src/convGemm.c:48-77. trans='N': out = epi(conv(x, in_)); else out = dW from dY=in_."""
    lib().convgemm_clear_error()
    lib().sconvGemmNHWC(trans.encode() if isinstance(trans, str) else trans, b, h, w, c, kn, kh, kw,
                        vpadding, hpadding, vstride, hstride, vdilation, hdilation, ptr(in_), ptr(x), ptr(out),
                        ptr(bias_vector), ptr(bn_running_mean), ptr(bn_inv_std), ptr(bn_gamma), ptr(bn_beta),
                        bool(relu), None, None)
    _check_dropin()


def sconvGemmNHWC_back(b, h, w, c, kn, kh, kw, vstride, hstride, vpadding, hpadding, vdilation, hdilation,
                       weights, dy, dx, ac_pack=None, bc_pack=None):
    """src/convGemm.c:82-97: dx += dgrad (stride before padding, as in the reference)."""
    lib().convgemm_clear_error()
    lib().sconvGemmNHWC_back(b, h, w, c, kn, kh, kw, vstride, hstride, vpadding, hpadding, vdilation, hdilation,
                             ptr(weights), ptr(dy), ptr(dx), None, None)
    _check_dropin()


def sconvGemmNCHW(trans, b, c, h, w, kn, kh, kw, vpadding, hpadding, vstride, hstride, vdilation, hdilation,
                  in_, x, out, bias_vector=None, bn_running_mean=None, bn_inv_std=None, bn_gamma=None,
                  bn_beta=None, relu=False, ac_pack=None, bc_pack=None):
    """src/convGemm.c:99-125 (NCHW, weights [kn][c][kh][kw])."""
    lib().convgemm_clear_error()
    lib().sconvGemmNCHW(trans.encode() if isinstance(trans, str) else trans, b, c, h, w, kn, kh, kw,
                        vpadding, hpadding, vstride, hstride, vdilation, hdilation, ptr(in_), ptr(x), ptr(out),
                        ptr(bias_vector), ptr(bn_running_mean), ptr(bn_inv_std), ptr(bn_gamma), ptr(bn_beta),
                        bool(relu), None, None)
    _check_dropin()


def sconvGemmNCHW_back(b, c, h, w, kn, kh, kw, vstride, hstride, vpadding, hpadding, vdilation, hdilation,
                       weights, dy, dx, ac_pack=None, bc_pack=None):
    """src/convGemm.c:130-146: dx += dgrad, NCHW."""
    lib().convgemm_clear_error()
    lib().sconvGemmNCHW_back(b, c, h, w, kn, kh, kw, vstride, hstride, vpadding, hpadding, vdilation, hdilation,
                             ptr(weights), ptr(dy), ptr(dx), None, None)
    _check_dropin()


# ------------------------------------------------------ extended API (FP32)
def _stream(stream):
    if stream is None:
        try:
            import torch
            return torch.cuda.current_stream().cuda_stream
        except Exception:
            return None
    return stream if isinstance(stream, int) else stream.cuda_stream


def _epi(bias=None, mean=None, inv_std=None, gamma=None, beta=None, relu=False):
    return Epilogue(ptr(bias), ptr(mean), ptr(inv_std), ptr(gamma), ptr(beta), int(bool(relu)))


def fwd_f32(layout, shape: Shape, weights, x, y, bias=None, mean=None, inv_std=None, gamma=None, beta=None,
            relu=False, stream=None):
    e = _epi(bias, mean, inv_std, gamma, beta, relu)
    _raise_if(lib().convgemm_fwd_f32(layout, ctypes.byref(shape), ptr(weights), ptr(x), ptr(y), ctypes.byref(e),
                                     _stream(stream)))


def wgrad_f32_workspace_size(shape: Shape) -> int:
    return lib().convgemm_wgrad_f32_workspace_size(ctypes.byref(shape))


def wgrad_f32(layout, shape: Shape, dy, x, dw, workspace, stream=None):
    nbytes = workspace.numel() * workspace.element_size()
    _raise_if(lib().convgemm_wgrad_f32(layout, ctypes.byref(shape), ptr(dy), ptr(x), ptr(dw), ptr(workspace),
                                       nbytes, _stream(stream)))


def dgrad_f32(layout, shape: Shape, weights, dy, dx, accumulate=True, stream=None):
    _raise_if(lib().convgemm_dgrad_f32(layout, ctypes.byref(shape), ptr(weights), ptr(dy), ptr(dx),
                                       int(bool(accumulate)), _stream(stream)))


def check_device(stream=None):
    _raise_if(lib().convgemm_check_device(_stream(stream)))
