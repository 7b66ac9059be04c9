"""Error metrics the parity tests use.

The reference's own check is element-wise |a-b|/|a| <= 1e-5 against its
explicit path (tests/test_base.h:19-29).  With signed data that ratio is
ill-conditioned where the exact value is near zero, so the tests use two
numbers, both held to the same 1e-5 tolerance for FP32:
  * normwise: max|out - ref| / max|ref|;
  * elementwise: max |out - ref| / |ref| over elements with |ref| >= 1e-3 * max|ref|.
"""
import numpy as np

FP32_TOL = 1e-5


def errors(out, ref):
    out = np.asarray(out, dtype=np.float64).ravel()
    ref = np.asarray(ref, dtype=np.float64).ravel()
    d = np.abs(out - ref)
    scale = np.abs(ref).max()
    if scale == 0:
        return float(d.max()), float(d.max())
    mask = np.abs(ref) >= 1e-3 * scale
    ew = float((d[mask] / np.abs(ref[mask])).max()) if mask.any() else 0.0
    return float(d.max() / scale), ew


def bitexact(a, b):
    a = np.ascontiguousarray(a, dtype=np.float32).ravel()
    b = np.ascontiguousarray(b, dtype=np.float32).ravel()
    return a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32))


def rel_max_rms(out, ref):
    """max and RMS relative error against an FP64 reference, normalised by max|ref| and RMS(ref)."""
    out = np.asarray(out, dtype=np.float64).ravel()
    ref = np.asarray(ref, dtype=np.float64).ravel()
    d = out - ref
    return float(np.abs(d).max() / max(np.abs(ref).max(), 1e-300)), \
        float(np.sqrt(np.mean(d * d)) / max(np.sqrt(np.mean(ref * ref)), 1e-300))
