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
OP_CACHE_TAG = "v6"   # op entries: fwd / dgrad with the M-tile, epilogue-warp and ring-stage choices
WGRAD_CACHE_TAG = "v12"   # wgrad: ring stages, two issuers, 128-pixel chunks, TMA-written single-split and one-cluster dW, grouped clusters, CTA pairs, slab kernel


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


# ------------------------------------------------ single-convolution operations
# The forward, input-gradient and weight-gradient entry points take their tile
# configuration from the library's tuning table (convgemm_tune_set) when it has
# an entry for the shape.  tune_ops measures the candidates of each (operation,
# shape) -- tile widths, and for the weight gradient also pixel-split counts --
# with `reps` calls replayed from one CUDA graph (device time, no host launch
# cost), installs the fastest and caches it beside the grouped-launch widths.

OP_NAMES = {tc.TUNE_FWD: "fwd", tc.TUNE_DGRAD: "dgrad", tc.TUNE_WGRAD: "wgrad", tc.TUNE_FWD_FP8: "fwd_fp8",
            tc.TUNE_FWD_BF16X3: "fwd_bf16x3"}


def op_key(op: int, s) -> str:
    tag = WGRAD_CACHE_TAG if op == tc.TUNE_WGRAD else OP_CACHE_TAG
    return f"{OP_NAMES[op]}.{tag}|{shape_key(s)}"


def graph_time_us(run, reps: int = 10) -> float:
    import torch
    run()
    torch.cuda.synchronize()
    st = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.stream(st):
        run()
        st.synchronize()
        with torch.cuda.graph(g, stream=st):
            for _ in range(reps):
                run()
    torch.cuda.synchronize()
    g.replay()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    g.replay()
    b.record()
    b.synchronize()
    return a.elapsed_time(b) * 1000 / reps


def _mt_ew(widths):
    """(bn, aux) of the BF16 forward / input gradient: aux = M tiles sharing a weight tile (1 / 2),
    + 4 for eight epilogue warps (bn >= 128 or two M tiles, not bn 256 with two), and for one M
    tile with four epilogue warps at widths 64 / 128 also the ring of one K block per stage with
    twice the stages (+ CONV_STAGES1)."""
    out = []
    for w in widths:
        for m in (1, 2):
            out.append((w, m))
            if (w >= 128 or m == 2) and not (w == 256 and m == 2):
                out.append((w, m + 4))
        if w != 256:
            out.append((w, 1 | tc.CONV_STAGES1))
    return out


def op_candidates(op: int, s):
    """(bn, aux) candidates: aux = weight-gradient pixel splits, or for the BF16 forward / input
    gradient the M tiles (1 / 2) sharing each weight tile, + 4 for eight epilogue warps."""
    if op == tc.TUNE_DGRAD:
        return _mt_ew(candidate_widths(s.c))
    if op == tc.TUNE_FWD:
        return _mt_ew(candidate_widths(s.kn))
    if op != tc.TUNE_WGRAD:
        return [(w, 0) for w in candidate_widths(s.kn)]
    tc.tune_set(op, s, 0, 0)
    bn0, s0, mx = tc.wgrad_bf16_plan(s)
    widths = [64, 128] if s.kn < 128 else candidate_widths(s.kh * s.kw * tc.c8(s.c))
    # around the heuristic, plus the cluster-reduced split counts (2..8) that fit
    splits = sorted({max(1, s0 // 4), max(1, s0 // 2), s0, min(mx, 2 * s0)} | {x for x in (2, 4, 8) if x <= mx})
    out = [(w, sp) for w in widths for sp in splits]
    if tc.c8(s.c) % 64 == 0:
        one = s.kh == 1 and s.kw == 1 and s.vstride == 1 and s.hstride == 1 and s.vpad == 0 and s.hpad == 0
        if one:   # the same tiling with X by im2col boxes instead of tiled boxes
            out += [(w, s0 | tc.WGRAD_IM2COL_X) for w in widths]
        if s.kn >= 128:   # X as the A operand of a wide layer, around its own split heuristic
            for w in (128, 256) if s.kn >= 256 else (128,):
                tc.tune_set(op, s, w, tc.WGRAD_X_ON_A)
                _, s2, _ = tc.wgrad_bf16_plan(s)
                for sp in sorted({max(1, s2 // 2), s2, min(mx, 2 * s2)} | {x for x in (2, 4, 8) if x <= mx}):
                    out.append((w, sp | tc.WGRAD_X_ON_A))
            tc.tune_set(op, s, 0, 0)
    # the ring of one chunk per stage with twice the stages, and two MMA-issuing warps on the two-chunk
    # ring (im2col path), for every tile and split
    if tc.c8(s.c) % 64 == 0:
        base = list(out)
        out += [(w, sp | tc.WGRAD_STAGES1) for w, sp in base] + [(w, sp | tc.WGRAD_TWO_ISSUERS) for w, sp in base] + \
            [(w, sp | tc.WGRAD_WIDE_CHUNKS) for w, sp in base]
    # more than 8 splits: also the in-kernel reduction by clusters of 2 / 4 / 8 splits
    out += [(w, sp | tc.WGRAD_GROUPS(cs)) for w, sp in list(out)
            if (sp & 0xffff) > 8 and not sp & (tc.WGRAD_STAGES1 | tc.WGRAD_TWO_ISSUERS | tc.WGRAD_WIDE_CHUNKS)
            for cs in (2, 4, 8)]
    # CTA pairs (256 x 256 tiles), both operand sides, around their own split heuristic
    if tc.c8(s.c) % 64 == 0:
        for xa in (0, tc.WGRAD_X_ON_A) if s.kn >= 128 else (0,):
            for w in (128, 256):
                tc.tune_set(op, s, w, tc.WGRAD_PAIR | xa)
                _, s4, _ = tc.wgrad_bf16_plan(s)
                out += [(w, sp | tc.WGRAD_PAIR | xa) for sp in sorted({max(1, s4 // 2), s4, min(mx, 2 * s4)})]
        tc.tune_set(op, s, 0, 0)
    # stride-1 layers with 128-channel blocks: the slab kernel around its own split heuristic
    tc.tune_set(op, s, 0, tc.WGRAD_SLAB)
    bn_s, s3, _ = tc.wgrad_bf16_plan(s)
    tc.tune_set(op, s, 0, 0)
    if s.vstride == 1 and s.hstride == 1 and tc.c8(s.c) % 128 == 0 and s.kw >= 2 and s.kn >= 64:
        out += [(0, tc.WGRAD_SLAB | sp) for sp in sorted({max(1, s3 // 2), s3, min(mx, 2 * s3)})]
    return out


def tune_ops(items, path: str | None = None, force: bool = False, measure_missing: bool = True,
             ws_limit_bytes: int = 1 << 30):
    """items: dicts {"op": tc.TUNE_*, "shape": Shape, "run": callable(workspace)}; run(ws) launches
    the operation once (the workspace argument matters to the weight gradient only).

    Installs the chosen configuration of every item in the library and returns
    {"measured": n, "cached": n, "shipped": n}.
    """
    import torch
    path = path or cache_path()
    dev = torch.cuda.get_device_properties(torch.cuda.current_device())
    db = _load(path)
    table = db.setdefault(dev.name, {})
    shipped = {} if force else _load(SHIPPED).get(dev.name, {})
    stats = {"measured": 0, "cached": 0, "shipped": 0, "heuristic": 0}
    dirty = False
    for it in items:
        op, s = it["op"], it["shape"]
        k = op_key(op, s)
        entry = None
        if not force and k in table:
            entry, src = table[k], "cached"
        elif not force and k in shipped:
            entry, src = shipped[k], "shipped"
        elif measure_missing:
            best, times = None, {}
            for bn, sp in op_candidates(op, s):
                tc.tune_set(op, s, bn, sp)
                ws = None
                if op == tc.TUNE_WGRAD:
                    nbytes = tc.wgrad_bf16_workspace_size(s)
                    if nbytes > ws_limit_bytes:
                        continue
                    ws = torch.empty(nbytes // 4 + 1, device="cuda")
                us = graph_time_us(lambda: it["run"](ws))
                times[f"{bn}/{sp}"] = us
                if best is None or us < best[0]:
                    best = (us, bn, sp)
            tc.tune_set(op, s, 0, 0)
            if best is None:
                stats["heuristic"] += 1
                continue
            tc.tune_set(op, s, best[1], best[2])
            kern, bnd, stages, cluster = tc.tune_describe(op, s) if op in (tc.TUNE_FWD, tc.TUNE_DGRAD, tc.TUNE_WGRAD) \
                else (0, best[1], 0, 1)
            entry, src = {"bn": best[1], "splits": best[2], "kernel": kern, "stages": stages, "cluster": cluster,
                          "us": times}, "measured"
            table[k] = entry
            dirty = True
        else:
            stats["heuristic"] += 1
            continue
        tc.tune_set(op, s, int(entry["bn"]), int(entry.get("splits", 0)))
        stats[src] += 1
    if dirty:
        _save(path, db)
    return stats
