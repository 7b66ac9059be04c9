"""Per-shape autotuner of the grouped BF16 forward launch.

The grouped kernel has one runtime tile choice per convolution: the number of
output channels per tile (64, 128 or 256; tiles are always 128 output pixels).
Wider tiles re-read the activation tile fewer times; narrower ones waste less
work on ragged output channels and make more tiles for small problems.

A shape is tuned in throughput mode, the way it runs inside a big group: the
convolution is repeated in a table enough times to give every SM several
tiles, so the measured cost per convolution is the steady-state cost of its
tiles and not the latency of one underfilled wave.  The fastest width is kept
in a JSON cache keyed by the device name and the shape.  Widths measured on
a GB300 for the shapes of the 256-convolution grouped workload ship with the
package (autotune_gb300.json) and are used when the user cache has no entry.

Other choices of the design are fixed and not tuned: one CTA per cluster (no
operand is shared between the CTAs of a group, whose tiles belong to unrelated
convolutions), four pipeline stages (the largest ring that holds a 256-wide
stage of 48 KB beside the output staging buffer), and no split-K in the
forward (the grouped table spreads small-M / long-K convolutions across SMs
instead; split-K is used by the weight gradient, whose K is the pixel count).
"""
from __future__ import annotations

import json
import os

from . import tc

WIDTHS = (64, 128, 256)
CACHE_VERSION = "group-bn-v1"


def cache_path() -> str:
    return os.environ.get("CONVGEMM_AUTOTUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "convgemm_gb300", "autotune.json"))


SHIPPED = os.path.join(os.path.dirname(os.path.abspath(__file__)), "autotune_gb300.json")


def shape_key(s) -> str:
    return "x".join(str(v) for v in (s.b, s.h, s.w, s.c, s.kn, s.kh, s.kw, s.vpad, s.hpad, s.vstride, s.hstride,
                                     s.vdil, s.hdil))


def candidate_widths(kn: int):
    """Widths worth trying: none wider than the next one that already covers kn."""
    out = []
    for w in WIDTHS:
        out.append(w)
        if w >= kn:
            break
    return out


def default_width(kn: int) -> int:
    return 256 if kn >= 256 else (128 if kn > 64 else 64)


def tiles_of(s, bn: int) -> int:
    return -(-(s.b * s.ho * s.wo) // 128) * -(-s.kn // bn)


def _load(path):
    try:
        with open(path) as f:
            d = json.load(f)
        return d if d.get("version") == CACHE_VERSION else {"version": CACHE_VERSION}
    except (OSError, ValueError):
        return {"version": CACHE_VERSION}


def _save(path, d):
    os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(d, f, indent=0, sort_keys=True)
    os.replace(tmp, path)


def measure(conv: dict, bn: int, sms: int, reps: int = 3) -> float:
    """Milliseconds per convolution of `conv` at tile width bn, in throughput mode."""
    import torch
    s = conv["shape"]
    r = max(1, min(64, -(-4 * sms // tiles_of(s, bn))))
    # the copies write identical values to the same output
    grp = tc.Group([dict(conv, bn=bn)] * r)
    grp.launch()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    start.record()
    for _ in range(reps):
        grp.launch()
    end.record()
    end.synchronize()
    return start.elapsed_time(end) / reps / r


def tune(convs, path: str | None = None, force: bool = False):
    """Chooses the tile width of every convolution (dicts as for tc.Group).

    Returns the list of widths; sets conv["bn"].  Measured shapes are cached.
    """
    import torch
    path = path or cache_path()
    dev = torch.cuda.get_device_properties(torch.cuda.current_device())
    db = _load(path)
    table = db.setdefault(dev.name, {})
    shipped = {} if force else _load(SHIPPED).get(dev.name, {})
    dirty = False
    out = []
    for conv in convs:
        s = conv["shape"]
        k = shape_key(s)
        if k not in table and k in shipped:
            conv["bn"] = int(shipped[k]["bn"])
            out.append(conv["bn"])
            continue
        if force or k not in table:
            cands = candidate_widths(s.kn)
            if len(cands) == 1:
                table[k] = {"bn": cands[0], "ms": None}
            else:
                ms = {bn: measure(conv, bn, dev.multi_processor_count) for bn in cands}
                best = min(ms, key=ms.get)
                table[k] = {"bn": best, "ms": {str(b): v for b, v in ms.items()}}
            dirty = True
        conv["bn"] = int(table[k]["bn"])
        out.append(conv["bn"])
    if dirty:
        _save(path, db)
    return out
