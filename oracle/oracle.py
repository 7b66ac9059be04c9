"""ctypes front-end of the test oracle.

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()`` and
by bench.py's CPU-baseline leg, never by the library.

Three checkers live behind it:

* ``liboracle.so`` (built from ``direct_conv.c`` and ``convgemm_port.c``):
  an FP64 direct convolution, and an FP32 restatement of convGemm that follows
  the reference's KC=384 blocked summation order (forward and weight gradient
  match the reference bit for bit);
* ``_ref/libconvgemm_ref.so``: the reference's own sources compiled against the
  project-written BLIS shim (``make -C oracle ref``; only where the reference
  checkout exists).

Arrays are numpy float32 (inputs) / float64 (FP64 results), C-contiguous.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libconvgemm_ref.so")
REF_SRC = os.path.join(os.environ.get("CONVGEMM_REFERENCE", "/root/reference"), "src")

NHWC, NCHW = 0, 1

_lib = None
_ref = None


def build(with_ref: bool | None = None) -> None:
    """Compile the oracle (and, where the reference checkout exists, the reference)."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    if with_ref is None:
        with_ref = os.path.isdir(REF_SRC)
    if with_ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref"], check=True)


def _f32p(a):
    if a is None:
        return None
    assert a.dtype == np.float32 and a.flags.c_contiguous
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def _f64p(a):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _i64p(a):
    assert a.dtype == np.int64 and a.flags.c_contiguous
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))


_FP = ctypes.POINTER(ctypes.c_float)
_DP = ctypes.POINTER(ctypes.c_double)
_LP = ctypes.POINTER(ctypes.c_int64)
_I = ctypes.c_int
_API_FWD = [ctypes.c_char] + [_I] * 13 + [_FP, _FP, _FP, _FP, _FP, _FP, _FP, _FP, ctypes.c_bool, _FP, _FP]
_API_BACK = [_I] * 13 + [_FP, _FP, _FP, _FP, _FP]


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build(with_ref=False)
        L = ctypes.CDLL(LIB_PATH)
        L.oracle_fwd_f64.argtypes = [_I] * 14 + [_FP, _FP, _DP, _FP, _FP, _FP, _FP, _FP, _I]
        L.oracle_fwd_points_f64.argtypes = [_I] * 14 + [_FP, _FP, _LP, ctypes.c_int64, _DP,
                                                         _FP, _FP, _FP, _FP, _FP, _I]
        L.oracle_wgrad_f64.argtypes = [_I] * 14 + [_FP, _FP, _DP]
        L.oracle_dgrad_f64.argtypes = [_I] * 14 + [_FP, _FP, _DP]
        L.oracle_dgrad_points_f64.argtypes = [_I] * 14 + [_FP, _FP, _LP, ctypes.c_int64, _DP]
        L.oracle_wgrad_points_f64.argtypes = [_I] * 14 + [_FP, _FP, _LP, ctypes.c_int64, _DP]
        L.oracle_bn_fold_f64.argtypes = [_I, _FP, _FP, _FP, _FP, _FP, _DP, _DP]
        L.oracle_im2row_nhwc.argtypes = [_FP, _FP] + [_I] * 12
        L.oracle_im2col_nchw.argtypes = [_FP, _FP] + [_I] * 12
        L.port_fwd_points.argtypes = [_I] * 14 + [_FP, _FP, _LP, ctypes.c_int64, _FP, _FP, _FP, _FP, _FP, _FP, _I]
        L.port_wgrad_points.argtypes = [_I] * 14 + [_FP, _FP, _LP, ctypes.c_int64, _FP]
        for name in ("port_sconvGemmNHWC", "port_sconvGemmNCHW"):
            getattr(L, name).argtypes = _API_FWD
        for name in ("port_sconvGemmNHWC_back", "port_sconvGemmNCHW_back"):
            getattr(L, name).argtypes = _API_BACK
        _lib = L
    return _lib


def ref_available() -> bool:
    return os.path.exists(REF_PATH)


def ref():
    """The reference's own code built against the BLIS shim (x86/aarch64 where it was built)."""
    global _ref
    if _ref is None:
        R = ctypes.CDLL(REF_PATH)
        R.sconvGemmNHWC.argtypes = _API_FWD
        R.sconvGemmNCHW.argtypes = _API_FWD
        R.sconvGemmNHWC_back.argtypes = _API_BACK
        R.sconvGemmNCHW_back.argtypes = _API_BACK
        R.alloc_pack_buffs.argtypes = [ctypes.POINTER(_FP), ctypes.POINTER(_FP)]
        R.alloc_pack_buffs.restype = _I
        _ref = R
    return _ref


def out_hw(h, w, kh, kw, vpad, hpad, vstr, hstr, vdil, hdil):
    """Output size (src/convGemm.c:60-61)."""
    ho = (h + 2 * vpad - vdil * (kh - 1) - 1) // vstr + 1
    wo = (w + 2 * hpad - hdil * (kw - 1) - 1) // hstr + 1
    return ho, wo


# ---------------------------------------------------------------- FP64 oracle
def _geom(g):
    return [g[k] for k in ("b", "h", "w", "c", "kn", "kh", "kw", "vpad", "hpad", "vstr", "hstr", "vdil", "hdil")]


def fwd_f64(layout, g, wts, x, epi=None):
    epi = epi or {}
    ho, wo = out_hw(g["h"], g["w"], g["kh"], g["kw"], g["vpad"], g["hpad"], g["vstr"], g["hstr"], g["vdil"], g["hdil"])
    shape = (g["b"], ho, wo, g["kn"]) if layout == NHWC else (g["b"], g["kn"], ho, wo)
    y = np.empty(shape, np.float64)
    lib().oracle_fwd_f64(layout, *_geom(g), _f32p(wts), _f32p(x), _f64p(y),
                         _f32p(epi.get("bias")), _f32p(epi.get("mean")), _f32p(epi.get("inv_std")),
                         _f32p(epi.get("gamma")), _f32p(epi.get("beta")), int(bool(epi.get("relu", False))))
    return y


def fwd_points_f64(layout, g, wts, x, idx, epi=None):
    epi = epi or {}
    idx = np.ascontiguousarray(idx, dtype=np.int64)
    out = np.empty(idx.shape[0], np.float64)
    lib().oracle_fwd_points_f64(layout, *_geom(g), _f32p(wts), _f32p(x), _i64p(idx), idx.shape[0], _f64p(out),
                                _f32p(epi.get("bias")), _f32p(epi.get("mean")), _f32p(epi.get("inv_std")),
                                _f32p(epi.get("gamma")), _f32p(epi.get("beta")), int(bool(epi.get("relu", False))))
    return out


def wgrad_f64(layout, g, dy, x):
    K = g["c"] * g["kh"] * g["kw"]
    dw = np.empty(K * g["kn"], np.float64)
    lib().oracle_wgrad_f64(layout, *_geom(g), _f32p(dy), _f32p(x), _f64p(dw))
    return dw


def wgrad_points_f64(layout, g, dy, x, idx):
    idx = np.ascontiguousarray(idx, dtype=np.int64)
    out = np.empty(idx.shape[0], np.float64)
    lib().oracle_wgrad_points_f64(layout, *_geom(g), _f32p(dy), _f32p(x), _i64p(idx), idx.shape[0], _f64p(out))
    return out


def dgrad_f64(layout, g, wts, dy):
    dx = np.empty(g["b"] * g["h"] * g["w"] * g["c"], np.float64)
    lib().oracle_dgrad_f64(layout, *_geom(g), _f32p(wts), _f32p(dy), _f64p(dx))
    return dx


def dgrad_points_f64(layout, g, wts, dy, idx):
    idx = np.ascontiguousarray(idx, dtype=np.int64)
    out = np.empty(idx.shape[0], np.float64)
    lib().oracle_dgrad_points_f64(layout, *_geom(g), _f32p(wts), _f32p(dy), _i64p(idx), idx.shape[0], _f64p(out))
    return out


def port_fwd_points(layout, g, wts, x, idx, epi=None):
    """The FP32 port's forward at sampled output indices (bit-identical to the whole-layer port)."""
    epi = epi or {}
    idx = np.ascontiguousarray(idx, dtype=np.int64)
    out = np.empty(idx.shape[0], np.float32)
    lib().port_fwd_points(layout, *_geom(g), _f32p(wts), _f32p(x), _i64p(idx), idx.shape[0], _f32p(out),
                          _f32p(epi.get("bias")), _f32p(epi.get("mean")), _f32p(epi.get("inv_std")),
                          _f32p(epi.get("gamma")), _f32p(epi.get("beta")), int(bool(epi.get("relu", False))))
    return out


def port_wgrad_points(layout, g, dy, x, idx):
    """The FP32 port's weight gradient at sampled dW indices (bit-identical to the whole-layer port)."""
    idx = np.ascontiguousarray(idx, dtype=np.int64)
    out = np.empty(idx.shape[0], np.float32)
    lib().port_wgrad_points(layout, *_geom(g), _f32p(dy), _f32p(x), _i64p(idx), idx.shape[0], _f32p(out))
    return out


def bn_fold_f64(kn, bias=None, mean=None, inv_std=None, gamma=None, beta=None):
    scale = np.empty(kn, np.float64)
    shift = np.empty(kn, np.float64)
    lib().oracle_bn_fold_f64(kn, _f32p(bias), _f32p(mean), _f32p(inv_std), _f32p(gamma), _f32p(beta),
                             _f64p(scale), _f64p(shift))
    return scale, shift


# --------------------------------------------- reference-API calls (port / ref)
def _api(which):
    if which == "port":
        L = lib()
        return {"NHWC": L.port_sconvGemmNHWC, "NCHW": L.port_sconvGemmNCHW,
                "NHWC_back": L.port_sconvGemmNHWC_back, "NCHW_back": L.port_sconvGemmNCHW_back}
    R = ref()
    return {"NHWC": R.sconvGemmNHWC, "NCHW": R.sconvGemmNCHW,
            "NHWC_back": R.sconvGemmNHWC_back, "NCHW_back": R.sconvGemmNCHW_back}


def _pack_buffs(which):
    if which == "port":
        return None, None
    a, b = _FP(), _FP()
    if ref().alloc_pack_buffs(ctypes.byref(a), ctypes.byref(b)) != 0:
        raise MemoryError("alloc_pack_buffs failed")
    return a, b


_libc = ctypes.CDLL(None)


def _free_pack(a, b):
    if a is not None:
        _libc.free(ctypes.cast(a, ctypes.c_void_p))
        _libc.free(ctypes.cast(b, ctypes.c_void_p))


def call_fwd(which, layout, g, wts, x, out, epi=None, trans="N"):
    """Calls sconvGemmNHWC/NCHW of the port or the shim-built reference with its exact argument order."""
    epi = epi or {}
    ac, bc = _pack_buffs(which)
    fn = _api(which)["NHWC" if layout == NHWC else "NCHW"]
    if layout == NHWC:
        dims = [g["b"], g["h"], g["w"], g["c"]]
    else:
        dims = [g["b"], g["c"], g["h"], g["w"]]
    fn(trans.encode(), *dims, g["kn"], g["kh"], g["kw"], g["vpad"], g["hpad"], g["vstr"], g["hstr"],
       g["vdil"], g["hdil"], _f32p(wts), _f32p(x), _f32p(out), _f32p(epi.get("bias")), _f32p(epi.get("mean")),
       _f32p(epi.get("inv_std")), _f32p(epi.get("gamma")), _f32p(epi.get("beta")), bool(epi.get("relu", False)),
       ac, bc)
    _free_pack(ac, bc)
    return out


def call_back(which, layout, g, wts, dy, dx):
    """Calls sconvGemm{NHWC,NCHW}_back (stride before padding, src/convGemm.h:36-38)."""
    ac, bc = _pack_buffs(which)
    fn = _api(which)["NHWC_back" if layout == NHWC else "NCHW_back"]
    if layout == NHWC:
        dims = [g["b"], g["h"], g["w"], g["c"]]
    else:
        dims = [g["b"], g["c"], g["h"], g["w"]]
    fn(*dims, g["kn"], g["kh"], g["kw"], g["vstr"], g["hstr"], g["vpad"], g["hpad"], g["vdil"], g["hdil"],
       _f32p(wts), _f32p(dy), _f32p(dx), ac, bc)
    _free_pack(ac, bc)
    return dx
