"""Error metrics the parity tests use.

The reference's own check is element-wise |a-b|/|a| <= 1e-5 against its
explicit path (tests/test_base.h:19-29), on all-positive data.  With signed
data that ratio is ill-conditioned where a sum cancels (the reference itself is
off the exact result by up to ~5e-2 in that sense), so the FP32 tolerance of
1e-5 is applied to three well-conditioned numbers:
  * normwise: max|out - ref| / max|ref|  (errors()[0]);
  * componentwise: max |out_i - ref_i| / sum_k |a_ik b_kj|, the magnitude
    FP32 rounding error scales with (magnitude(), componentwise());
  * the reference's own element-wise ratio, on the all-positive cases
    (elementwise_ref_check()).
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


def magnitude(O, op, layout, g, inp):
    """Per-element error scale sum_k |a_k b_k| (+ the epilogue's terms): the
    quantity FP32 rounding error is proportional to, from the FP64 oracle run
    on absolute values.  A per-element check |out - ref| <= tol * magnitude is
    well conditioned even where signed sums cancel."""
    ab = lambda a: None if a is None else np.abs(a)  # noqa: E731
    if op == "fwd":
        e = inp["epi"]
        acc = O.fwd_f64(layout, g, ab(inp["w"]), ab(inp["x"])).ravel()
        kn = g["kn"]
        ch = (np.arange(acc.size) % kn) if layout == 0 else \
            ((np.arange(acc.size) // (acc.size // (g["b"] * kn))) % kn)
        m = acc.copy()
        if e.get("bias") is not None:
            m += np.abs(e["bias"][ch])
        if e.get("mean") is not None:
            m = (m + np.abs(e["mean"][ch])) * np.abs(e["inv_std"][ch] * e["gamma"][ch]) + np.abs(e["beta"][ch])
        return m
    if op == "wgrad":
        return O.wgrad_f64(layout, g, ab(inp["dy"]), ab(inp["x"]))
    return O.dgrad_f64(layout, g, ab(inp["w"]), ab(inp["dy"])) + np.abs(inp["dx0"])


def componentwise(out, ref, mag):
    out = np.asarray(out, dtype=np.float64).ravel()
    ref = np.asarray(ref, dtype=np.float64).ravel()
    mag = np.maximum(np.asarray(mag, dtype=np.float64).ravel(), 1e-30)
    return float((np.abs(out - ref) / mag).max())


def elementwise_ref_check(out, ref):
    """The reference's own check (tests/test_base.h:19-29): max |a-b|/|a| over all elements
    (meaningful on its all-positive data)."""
    out = np.asarray(out, dtype=np.float64).ravel()
    ref = np.asarray(ref, dtype=np.float64).ravel()
    nz = ref != 0
    return float((np.abs(out[nz] - ref[nz]) / np.abs(ref[nz])).max()) if nz.any() else 0.0
