#!/usr/bin/env python3
"""ResNet-50 conv fwd+bwd throughput on one GB300: BF16 tensor-core form vs FP32 plain.

One step = for each of the 53 convolutions of ResNet-50 v1.5 at batch 64
(224x224, NHWC): BN fold (FP64), weight packing, forward with the fused
BN/ReLU epilogue, input gradient (not for the stem, whose input needs none)
and weight gradient.  Inputs are synthetic, seeded, resident in HBM; the
working set of a step (several GB) is far larger than L2.

  value  : BF16 img/s, the step captured once in a CUDA graph and replayed;
  e2e    : the same step through the public API call by call, with the
           image batch and the top gradient copied host->device and all
           weight gradients copied device->host inside every timed step;
  fp32_plain : the same step with the FP32 plain kernels (the drop-in form);
  roofline   : the dominant kernel family, CUDA-event timed, against
           MEASURED_PEAKS.json;
  cpu_baseline: the FP32 CPU restatement of the reference (oracle port) on
           this host's cores, one image through all 53 layers.

`--impl reference` times the reference's CPU path (the oracle port: the
reference's sources are not on the GPU host) on the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from convgemm_gb300.workloads import conv_flops, out_hw, resnet50_layers  # noqa: E402

METRIC = "ResNet-50 conv fwd+bwd img/s, BF16-TC vs FP32 plain on GB300 at stated rel err"
BATCH = 64


def c8(c):
    return (c + 7) // 8 * 8


def step_flops(layers, batch):
    return sum(conv_flops(l, batch) * (2 if i == 0 else 3) for i, l in enumerate(layers))


def max_over_ranks(torch, values, device="cuda"):
    """Element-wise maximum of this rank's timings over all ranks (torch.distributed); the
    whole-job time of a step is the slowest rank's."""
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return [float(v) for v in t.tolist()]


def profile_traffic(prefixes, path=os.path.join(ROOT, "profiles", "launches_resnet50_bf16_b64.md")):
    """DRAM bytes (read + write) per step of the kernels whose names start with one of
    `prefixes`, from the committed ncu launch-list summary of one step (cold-cache capture)."""
    try:
        tot = 0.0
        for line in open(path):
            cells = [c.strip() for c in line.strip().strip("|").split("|")]
            if len(cells) == 5 and cells[0].startswith("`") and cells[0].strip("`").startswith(tuple(prefixes)):
                tot += float(cells[4]) * 1e6
        return tot or None
    except (OSError, ValueError):
        return None


def read_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


def measure_ffma_peak(torch, cg, reps=5):
    """FP32 FMA (SIMT) peak in TFLOP/s: the library's FMA-chain kernel on every SM, timed with CUDA
    events (best of `reps` launches of about 2 ms); the denominator of the FP32 plain form's fraction."""
    import ctypes
    out = torch.zeros(1, device="cuda")
    fl = ctypes.c_double()
    st = torch.cuda.current_stream()
    best = None
    for i in range(reps + 2):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(st)
        cg._raise_if(cg.lib().convgemm_measure_ffma(2000, cg.ptr(out), ctypes.byref(fl), st.cuda_stream))
        b.record(st)
        b.synchronize()
        if i >= 2:
            t = fl.value / (a.elapsed_time(b) / 1000) / 1e12
            best = t if best is None else max(best, t)
    return best


def measure_fp8_peak(torch, reps=10):
    """Dense FP8-E4M3 tensor peak in TFLOP/s: an 8192^3 E4M3 x E4M3 -> BF16 GEMM through cuBLASLt
    (torch._scaled_mm), best of `reps`, CUDA events; None where the call is unavailable."""
    try:
        n = 8192
        a = torch.randn(n, n, device="cuda").to(torch.float8_e4m3fn)
        bt = torch.randn(n, n, device="cuda").to(torch.float8_e4m3fn)
        one = torch.ones((), device="cuda")
        f = lambda: torch._scaled_mm(a, bt.t(), scale_a=one, scale_b=one, out_dtype=torch.bfloat16)
        for _ in range(3):
            f()
        best = None
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            f()
            e1.record()
            e1.synchronize()
            t = 2.0 * n ** 3 / (e0.elapsed_time(e1) / 1000) / 1e12
            best = t if best is None else max(best, t)
        return best
    except Exception:
        return None


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(gpu_index), "--query-gpu=" + self.Q,
                                       "--format=csv,noheader,nounits", "-lms", "100"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None
        # start timing only once the sampler is producing samples
        t0 = time.time()
        while self.p is not None and time.time() - t0 < 3.0:
            try:
                if os.path.getsize(self.f.name) > 0:
                    break
            except OSError:
                pass
            time.sleep(0.02)

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.flush()
        self.f.seek(0)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.f:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        os.unlink(self.f.name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


# ---------------------------------------------------------------- CPU side
def cpu_baseline_run(layers, images, threads=None):
    """The oracle port (FP32, the reference's summation order) on `images` images through all layers.
    Returns (seconds, images)."""
    import numpy as np
    if threads:
        os.environ["OMP_NUM_THREADS"] = str(threads)
    from oracle import oracle as O
    O.build(with_ref=False)
    rng = np.random.default_rng(0)
    t_total = 0.0
    for i, l in enumerate(layers):
        g = dict(b=images, h=l["h"], w=l["w"], c=l["c"], kn=l["kn"], kh=l["k"], kw=l["k"], vpad=l["pad"],
                 hpad=l["pad"], vstr=l["stride"], hstr=l["stride"], vdil=1, hdil=1)
        ho, wo = out_hw(l)
        K = l["c"] * l["k"] * l["k"]
        x = rng.standard_normal(images * l["h"] * l["w"] * l["c"]).astype(np.float32)
        w = (rng.standard_normal(K * l["kn"]) * np.sqrt(2.0 / K)).astype(np.float32)
        dy = rng.standard_normal(images * ho * wo * l["kn"]).astype(np.float32)
        kn = l["kn"]
        epi = {"mean": rng.normal(0, .1, kn).astype(np.float32), "inv_std": np.ones(kn, np.float32),
               "gamma": np.ones(kn, np.float32), "beta": np.zeros(kn, np.float32), "bias": np.zeros(kn, np.float32),
               "relu": True}
        y = np.empty(images * ho * wo * kn, np.float32)
        dw = np.empty(K * kn, np.float32)
        dx = np.zeros_like(x)
        t0 = time.perf_counter()
        O.call_fwd("port", O.NHWC, g, w, x, y, epi)
        if i > 0:
            O.call_back("port", O.NHWC, g, w, dy, dx)
        O.call_fwd("port", O.NHWC, g, dy, x, dw, None, trans="T")
        t_total += time.perf_counter() - t0
    return t_total, images


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    layers = resnet50_layers()
    threads = os.cpu_count()
    images = args.ref_images
    for _ in range(args.warmup):
        cpu_baseline_run(layers, images, threads)
    times = []
    for _ in range(args.steps):
        t, n = cpu_baseline_run(layers, images, threads)
        times.append(t)
    tot = sum(times)
    v = args.steps * images / tot
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "img/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * tot / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "resnet50 v1.5 53 convs fwd+dgrad+wgrad, NHWC, FP32, CPU",
                       "global_batch": images, "seq_len": None, "parallelism": "replicas"},
            "cpu_baseline": {"value": v, "unit": "img/s", "cores": threads, "kind": "port",
                             "sample": f"{images} image(s) x 53 layers fwd+wgrad+dgrad per step "
                                       "(reference's KC=384 order, FP32)"},
            "e2e": {"value": v, "unit": "img/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- GPU side
class Net:
    """Per-layer device buffers for both precision forms (synthetic, seeded)."""

    def __init__(self, torch, cg, tc, layers, batch, with_fp32=True):
        self.torch, self.cg, self.tc, self.layers, self.batch = torch, cg, tc, layers, batch
        dev = "cuda"
        g = torch.Generator(device=dev).manual_seed(20261203)
        self.L = []
        ws_bf16 = ws_f32 = 16
        for i, l in enumerate(layers):
            ho, wo = out_hw(l)
            s = cg.Shape.of(batch, l["h"], l["w"], l["c"], l["kn"], l["k"], l["k"], l["pad"], l["pad"], l["stride"],
                            l["stride"], 1, 1)
            K = l["c"] * l["k"] * l["k"]
            kn = l["kn"]
            d = {"i": i, "s": s, "relu": not (l["name"].endswith("conv3") or l["name"].endswith("down")), "first": i == 0}
            d["w32"] = torch.randn(K * kn, device=dev, generator=g) * (2.0 / K) ** 0.5
            d["mean"] = torch.randn(kn, device=dev, generator=g) * 0.1
            var = torch.rand(kn, device=dev, generator=g) * 1.5 + 0.5
            d["inv_std"] = 1.0 / torch.sqrt(var + 1e-5)
            d["gamma"] = torch.rand(kn, device=dev, generator=g) + 0.5
            d["beta"] = torch.rand(kn, device=dev, generator=g) * 0.2 - 0.1
            d["scale"] = torch.empty(kn, device=dev)
            d["shift"] = torch.empty(kn, device=dev)
            d["x"] = torch.randn(batch, l["h"], l["w"], c8(l["c"]), device=dev, generator=g).to(torch.bfloat16)
            d["dy"] = (torch.randn(batch, ho, wo, c8(kn), device=dev, generator=g) * 0.1).to(torch.bfloat16)
            d["y"] = torch.empty(batch, ho, wo, kn, device=dev, dtype=torch.bfloat16)
            d["dx"] = None if i == 0 else torch.empty(batch, l["h"], l["w"], l["c"], device=dev, dtype=torch.bfloat16)
            d["dw"] = torch.empty(K * kn, device=dev)
            d["wp"] = torch.empty(tc.weights_size(s, tc.OPERAND_FWD) // 2, device=dev, dtype=torch.bfloat16)
            d["wpd"] = None if i == 0 else torch.empty(tc.weights_size(s, tc.OPERAND_DGRAD) // 2, device=dev,
                                                       dtype=torch.bfloat16)
            ws_bf16 = max(ws_bf16, tc.wgrad_bf16_workspace_size(s))
            if with_fp32:
                ws_f32 = max(ws_f32, cg.wgrad_f32_workspace_size(s))
            self.L.append(d)
        self.ws = torch.empty(ws_bf16 // 4 + 1, device=dev)
        self.ws2 = self.ws
        self.side = torch.cuda.Stream()
        # every layer's BN fold and weight packings in one grouped launch
        self.prep = tc.Prep([dict(layout=cg.NHWC, shape=d["s"], weights=d["w32"], packed_fwd=d["wp"],
                                  packed_dgrad=d["wpd"], mean=d["mean"], inv_std=d["inv_std"], gamma=d["gamma"],
                                  beta=d["beta"], scale=d["scale"], shift=d["shift"]) for d in self.L])
        self.ws32 = torch.empty(ws_f32 // 4 + 1, device=dev) if with_fp32 else None
        self.with_fp32 = with_fp32
        if with_fp32:
            for d in self.L:
                s = d["s"]
                ho, wo = s.ho, s.wo
                d["x32"] = torch.randn(batch, s.h, s.w, s.c, device=dev, generator=g)
                d["dy32"] = torch.randn(batch, ho, wo, s.kn, device=dev, generator=g) * 0.1
                d["y32"] = torch.empty(batch, ho, wo, s.kn, device=dev)
                d["dx32"] = None if d["first"] else torch.empty(batch, s.h, s.w, s.c, device=dev)
                d["dw32"] = torch.empty(s.c * s.kh * s.kw * s.kn, device=dev)

    def launches_f32(self):
        return sum(3 if d["first"] else 4 for d in self.L)

    def tune_items(self):
        """(operation, shape, launcher) of every BF16 convolution of the step, for the autotuner."""
        tc, cg = self.tc, self.cg
        items = []
        for d in self.L:
            s = d["s"]
            items.append({"op": tc.TUNE_FWD, "shape": s, "run": lambda ws, d=d, s=s: tc.fwd_bf16(
                s, d["x"], d["wp"], d["y"], d["scale"], d["shift"], relu=d["relu"])})
            if not d["first"]:
                items.append({"op": tc.TUNE_DGRAD, "shape": s,
                              "run": lambda ws, d=d, s=s: tc.dgrad_bf16(s, d["dy"], d["wpd"], d["dx"])})
            items.append({"op": tc.TUNE_WGRAD, "shape": s, "run": lambda ws, d=d, s=s: tc.wgrad_bf16(
                cg.NHWC, s, d["dy"], d["x"], d["dw"], ws)})
        return items

    def resize_workspace(self):
        need = max(self.tc.wgrad_bf16_workspace_size(d["s"]) for d in self.L)
        if need > self.ws.numel() * 4:
            self.ws = self.torch.empty(need // 4 + 1, device="cuda")
        self.ws2 = self.ws   # the step's weight gradients run one at a time on the side stream

    def step_bf16(self):
        """One BF16 step: weight preparation, forward, input gradient, weight gradient of every layer,
        scheduled as a training step's dependencies allow on two streams:
          forward  -- the layer chain; a first block's downsample convolution (same input as its
                      conv1) runs beside conv1..conv3 and joins before the next block;
          backward -- the input-gradient chain in reverse layer order on the main stream; the weight
                      gradient of layer i on the second stream as soon as dY_i exists (after the input
                      gradient of layer i+1; the last layer's at once)."""
        torch, tc, cg = self.torch, self.tc, self.cg
        main, side = torch.cuda.current_stream(), self.side
        self.prep.launch(main)
        blk = None
        for d in self.L:
            s, name = d["s"], self.layers[d["i"]]["name"]
            if name.endswith("_conv1"):
                blk = torch.cuda.Event()
                blk.record(main)
            st = main
            if name.endswith("_down"):
                side.wait_event(blk)
                st = side
            tc.fwd_bf16(s, d["x"], d["wp"], d["y"], d["scale"], d["shift"], relu=d["relu"], stream=st)
            if st is side:
                main.wait_stream(side)
        ready = torch.cuda.Event()
        ready.record(main)
        # the weight gradients fill the SMs the input-gradient chain leaves idle: no early
        # (programmatic) launches on the chain while they run
        pdl = cg.set_pdl(0)
        for d in reversed(self.L):
            s = d["s"]
            side.wait_event(ready)
            tc.wgrad_bf16(cg.NHWC, s, d["dy"], d["x"], d["dw"], self.ws2, stream=side)
            if not d["first"]:
                tc.dgrad_bf16(s, d["dy"], d["wpd"], d["dx"], stream=main)
                ready = torch.cuda.Event()
                ready.record(main)
        cg.set_pdl(pdl)
        main.wait_stream(side)

    def step_family(self, fam):
        """Launches one kernel family of the BF16 step; returns how many kernels it launched."""
        tc, cg = self.tc, self.cg
        n = 0
        if fam == "prep":
            self.prep.launch()
            return 1
        for d in self.L:
            s = d["s"]
            if fam == "fwd":
                tc.fwd_bf16(s, d["x"], d["wp"], d["y"], d["scale"], d["shift"], relu=d["relu"])
                n += 1
            elif fam == "dgrad" and not d["first"]:
                tc.dgrad_bf16(s, d["dy"], d["wpd"], d["dx"])
                n += 1
            elif fam == "wgrad":
                tc.wgrad_bf16(cg.NHWC, s, d["dy"], d["x"], d["dw"], self.ws)
                n += 2
        return n

    def family_flops(self, fam):
        if fam == "prep":
            return 0
        return sum(conv_flops(self.layers[d["i"]], self.batch) for d in self.L
                   if not (fam == "dgrad" and d["first"]))

    def step_f32(self):
        cg = self.cg
        for d in self.L:
            s = d["s"]
            cg.fwd_f32(cg.NHWC, s, d["w32"], d["x32"], d["y32"], mean=d["mean"], inv_std=d["inv_std"],
                       gamma=d["gamma"], beta=d["beta"], relu=d["relu"])
            if not d["first"]:
                cg.dgrad_f32(cg.NHWC, s, d["w32"], d["dy32"], d["dx32"], accumulate=False)
            cg.wgrad_f32(cg.NHWC, s, d["dy32"], d["x32"], d["dw32"], self.ws32)


def layer_bytes(l, batch, op="fwd", elem=2):
    """Algorithmic HBM bytes of one BF16 operation of a layer: each operand once.

    X counts only the pixels the layer reads: a 1x1 convolution with stride s and no padding
    reads every s-th pixel of every s-th row, so (ho * wo) pixels, not (h * w).  The input
    gradient writes all of dX (pixels that no tap reaches are written as zeros), and the
    weight gradient writes dW in FP32."""
    ho, wo = out_hw(l)
    cx = c8(l["c"])
    x_all = batch * l["h"] * l["w"] * cx
    x_read = batch * ho * wo * cx if (l["k"] == 1 and l["pad"] == 0) else x_all
    y = batch * ho * wo * l["kn"]
    w = l["c"] * l["k"] * l["k"] * l["kn"]
    if op == "fwd":
        return elem * (x_read + y + w)
    if op == "dgrad":
        return elem * (y + w + x_all)
    return elem * (x_read + y) + 4 * w


def per_layer_table(torch, net, layers, batch, peaks, path, reps=20):
    """Device time of each BF16 op of each layer (reps calls replayed from one CUDA graph),
    with its roofline bound."""
    tc, cg = net.tc, net.cg
    rows = []
    pk_t = peaks["bf16_tflops_sustained"] * 1e12
    pk_b = peaks["hbm_gbs"] * 1e9
    for d, l in zip(net.L, layers):
        s = d["s"]
        ops = {"fwd": lambda: tc.fwd_bf16(s, d["x"], d["wp"], d["y"], d["scale"], d["shift"], relu=d["relu"]),
               "wgrad": lambda: tc.wgrad_bf16(cg.NHWC, s, d["dy"], d["x"], d["dw"], net.ws)}
        if not d["first"]:
            ops["dgrad"] = lambda: tc.dgrad_bf16(s, d["dy"], d["wpd"], d["dx"])
        fl = conv_flops(l, batch)
        row = {"layer": l["name"], "shape": [l["h"], l["c"], l["kn"], l["k"], l["stride"]], "gflop": fl / 1e9}
        for name, fn in ops.items():
            # `reps` calls captured in one CUDA graph: device time, not host launch cost
            st = torch.cuda.Stream()
            g = torch.cuda.CUDAGraph()
            with torch.cuda.stream(st):
                fn()
                st.synchronize()
                with torch.cuda.graph(g, stream=st):
                    for _ in range(reps):
                        fn()
            torch.cuda.synchronize()
            g.replay()
            torch.cuda.synchronize()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            g.replay()
            b.record()
            torch.cuda.synchronize()
            us = a.elapsed_time(b) * 1000 / reps
            del g
            by = layer_bytes(l, batch, name)
            roof = max(fl / pk_t, by / pk_b) * 1e6
            row[name + "_mb"] = by / 1e6
            row[name + "_roofline_us"] = roof
            row[name + "_us"] = us
            row[name + "_frac"] = roof / us
        rows.append(row)
    with open(path, "w") as f:
        json.dump(rows, f, indent=1)


def run_only(torch, cg, tc, layers, batch, args):
    name, op = args.only.split(":")
    idx = next(i for i, l in enumerate(layers) if l["name"] == name)
    f32 = op.endswith("32")
    net = Net(torch, cg, tc, [layers[idx]], batch, with_fp32=f32)
    d = net.L[0]
    d["first"] = False
    s = d["s"]
    if f32 and d["dx32"] is None:
        d["dx32"] = torch.empty(batch, s.h, s.w, s.c, device="cuda")
    if d["wpd"] is None:
        d["wpd"] = torch.empty(tc.weights_size(s, tc.OPERAND_DGRAD) // 2, device="cuda", dtype=torch.bfloat16)
        d["dx"] = torch.empty(batch, s.h, s.w, s.c, device="cuda", dtype=torch.bfloat16)
    tc.fold_epilogue(s.kn, d["scale"], d["shift"], mean=d["mean"], inv_std=d["inv_std"], gamma=d["gamma"],
                     beta=d["beta"])
    tc.pack_weights(cg.NHWC, s, tc.OPERAND_FWD, d["w32"], d["wp"])
    tc.pack_weights(cg.NHWC, s, tc.OPERAND_DGRAD, d["w32"], d["wpd"])
    if not args.no_autotune:
        from convgemm_gb300 import autotune
        autotune.tune_ops(net.tune_items(), measure_missing=False)   # the step's tile configuration
        net.resize_workspace()
    fn = {"fwd": lambda: tc.fwd_bf16(s, d["x"], d["wp"], d["y"], d["scale"], d["shift"], relu=d["relu"]),
          "dgrad": lambda: tc.dgrad_bf16(s, d["dy"], d["wpd"], d["dx"]),
          "wgrad": lambda: tc.wgrad_bf16(cg.NHWC, s, d["dy"], d["x"], d["dw"], net.ws),
          "fwd32": lambda: cg.fwd_f32(cg.NHWC, s, d["w32"], d["x32"], d["y32"], mean=d["mean"],
                                      inv_std=d["inv_std"], gamma=d["gamma"], beta=d["beta"], relu=d["relu"]),
          "dgrad32": lambda: cg.dgrad_f32(cg.NHWC, s, d["w32"], d["dy32"], d["dx32"], accumulate=False),
          "wgrad32": lambda: cg.wgrad_f32(cg.NHWC, s, d["dy32"], d["x32"], d["dw32"], net.ws32)}[op]
    ms = timed(torch, fn, args.steps, args.warmup, torch.cuda.current_stream())
    cg.check_device()
    fl = conv_flops(layers[idx], batch)
    print(json.dumps({"only": args.only, "batch": batch, "us": ms * 1000, "tflops": fl / (ms / 1000) / 1e12}))


def timed(torch, fn, steps, warmup, stream):
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    start.record(stream)
    for _ in range(steps):
        fn()
    end.record(stream)
    torch.cuda.synchronize()
    return start.elapsed_time(end) / steps


def grouped_cpu_baseline(specs, every=8, threads=None):
    """The oracle port (FP32 sconvGemmNHWC in the reference's order) on every `every`-th
    convolution of the grouped workload.  Returns (seconds, flops)."""
    import numpy as np
    if threads:
        os.environ["OMP_NUM_THREADS"] = str(threads)
    from oracle import oracle as O
    O.build(with_ref=False)
    rng = np.random.default_rng(1)
    t_total, fl = 0.0, 0
    for d in specs[::every]:
        g = dict(b=d["b"], h=d["h"], w=d["w"], c=d["c"], kn=d["kn"], kh=d["k"], kw=d["k"], vpad=d["pad"],
                 hpad=d["pad"], vstr=d["stride"], hstr=d["stride"], vdil=1, hdil=1)
        ho = (d["h"] + 2 * d["pad"] - d["k"]) // d["stride"] + 1
        K = d["c"] * d["k"] * d["k"]
        x = rng.uniform(-1, 1, d["b"] * d["h"] * d["w"] * d["c"]).astype(np.float32)
        w = (rng.standard_normal(K * d["kn"]) * np.sqrt(2.0 / K)).astype(np.float32)
        epi = {"bias": rng.uniform(-.1, .1, d["kn"]).astype(np.float32), "relu": True}
        y = np.empty(d["b"] * ho * ho * d["kn"], np.float32)
        t0 = time.perf_counter()
        O.call_fwd("port", O.NHWC, g, w, x, y, epi)
        t_total += time.perf_counter() - t0
        fl += 2 * d["b"] * ho * ho * d["kn"] * K
    return t_total, fl


class VggNet:
    """VGG-16 NCHW training step buffers (synthetic, seeded): the FP32 plain form on the
    reference's NCHW layouts, and the BF16 form fed from the same FP32 NCHW tensors."""

    def __init__(self, torch, cg, tc, layers, batch):
        self.torch, self.cg, self.tc, self.layers, self.batch = torch, cg, tc, layers, batch
        g = torch.Generator(device="cuda").manual_seed(20261204)
        self.L = []
        ws32 = ws16 = 16
        for i, l in enumerate(layers):
            s = cg.Shape.of(batch, l["h"], l["w"], l["c"], l["kn"], 3, 3, 1, 1, 1, 1, 1, 1)
            K, kn = l["c"] * 9, l["kn"]
            d = {"s": s, "first": i == 0}
            d["x32"] = torch.randn(batch, l["c"], l["h"], l["w"], device="cuda", generator=g)
            d["w32"] = torch.randn(kn, l["c"], 3, 3, device="cuda", generator=g) * (2.0 / K) ** 0.5   # OIHW
            d["bias"] = torch.rand(kn, device="cuda", generator=g) * 0.2 - 0.1
            d["dy32"] = torch.randn(batch, kn, l["h"], l["w"], device="cuda", generator=g) * 1e-2 ** 0.5
            d["y32"] = torch.empty(batch, kn, l["h"], l["w"], device="cuda")
            d["dx32"] = None if i == 0 else torch.empty(batch, l["c"], l["h"], l["w"], device="cuda")
            d["dw32"] = torch.empty(kn, l["c"], 3, 3, device="cuda")
            # BF16 form: NHWC BF16 activations, packed weights, FP32 dW in the NCHW API's OIHW layout
            d["xb"] = torch.empty(batch, l["h"], l["w"], c8(l["c"]), device="cuda", dtype=torch.bfloat16)
            d["dyb"] = torch.empty(batch, l["h"], l["w"], kn, device="cuda", dtype=torch.bfloat16)
            d["yb"] = torch.empty(batch, l["h"], l["w"], kn, device="cuda", dtype=torch.bfloat16)
            d["dxb"] = None if i == 0 else torch.empty(batch, l["h"], l["w"], l["c"], device="cuda",
                                                       dtype=torch.bfloat16)
            d["dwb"] = torch.empty(kn, l["c"], 3, 3, device="cuda")
            d["wp"] = torch.empty(tc.weights_size(s, tc.OPERAND_FWD) // 2, device="cuda", dtype=torch.bfloat16)
            d["wpd"] = None if i == 0 else torch.empty(tc.weights_size(s, tc.OPERAND_DGRAD) // 2, device="cuda",
                                                       dtype=torch.bfloat16)
            d["scale"] = torch.ones(kn, device="cuda")
            d["shift"] = torch.empty(kn, device="cuda")
            ws32 = max(ws32, cg.wgrad_f32_workspace_size(s))
            ws16 = max(ws16, tc.wgrad_bf16_workspace_size(s))
            self.L.append(d)
        self.ws32 = torch.empty(ws32 // 4 + 1, device="cuda")
        self.ws16 = torch.empty(ws16 // 4 + 1, device="cuda")
        self.side = torch.cuda.Stream()
        self.prep = tc.Prep([dict(layout=cg.NCHW, shape=d["s"], weights=d["w32"], packed_fwd=d["wp"],
                                  packed_dgrad=d["wpd"], bias=d["bias"], scale=d["scale"], shift=d["shift"])
                             for d in self.L])

    def tune_items(self):
        tc, cg = self.tc, self.cg
        items = []
        for d in self.L:
            s = d["s"]
            items.append({"op": tc.TUNE_FWD, "shape": s, "run": lambda ws, d=d, s=s: tc.fwd_bf16(
                s, d["xb"], d["wp"], d["yb"], d["scale"], d["shift"], relu=True)})
            if not d["first"]:
                items.append({"op": tc.TUNE_DGRAD, "shape": s,
                              "run": lambda ws, d=d, s=s: tc.dgrad_bf16(s, d["dyb"], d["wpd"], d["dxb"])})
            items.append({"op": tc.TUNE_WGRAD, "shape": s, "run": lambda ws, d=d, s=s: tc.wgrad_bf16(
                cg.NCHW, s, d["dyb"], d["xb"], d["dwb"], ws)})
        return items

    def resize_workspace(self):
        need = max(self.tc.wgrad_bf16_workspace_size(d["s"]) for d in self.L)
        if need > self.ws16.numel() * 4:
            self.ws16 = self.torch.empty(need // 4 + 1, device="cuda")

    def step_f32(self):
        cg = self.cg
        for d in self.L:
            s = d["s"]
            cg.fwd_f32(cg.NCHW, s, d["w32"], d["x32"], d["y32"], bias=d["bias"], relu=True)
            if not d["first"]:
                cg.dgrad_f32(cg.NCHW, s, d["w32"], d["dy32"], d["dx32"], accumulate=False)
            cg.wgrad_f32(cg.NCHW, s, d["dy32"], d["x32"], d["dw32"], self.ws32)

    def wgrad_f32(self):
        for d in self.L:
            self.cg.wgrad_f32(self.cg.NCHW, d["s"], d["dy32"], d["x32"], d["dw32"], self.ws32)

    def step_bf16(self):
        """The BF16 form of the step: one grouped preparation (bias folds, OIHW weight packings),
        then per layer the NCHW FP32 -> NHWC BF16 conversions and the convolutions, scheduled on
        two streams: the forward chain, then the input-gradient chain on the main stream with each
        layer's weight gradient on the second stream as soon as its dY has been converted."""
        torch, cg, tc = self.torch, self.cg, self.tc
        main, side = torch.cuda.current_stream(), self.side
        self.prep.launch(main)
        for d in self.L:
            s = d["s"]
            tc.to_bf16_nhwc(cg.NCHW, s.b, s.c, s.h, s.w, d["x32"], d["xb"], stream=main)
            tc.fwd_bf16(s, d["xb"], d["wp"], d["yb"], d["scale"], d["shift"], relu=True, stream=main)
        pdl = cg.set_pdl(0)   # no early launches on the chain while the weight gradients run beside it
        for d in reversed(self.L):
            s = d["s"]
            tc.to_bf16_nhwc(cg.NCHW, s.b, s.kn, s.h, s.w, d["dy32"], d["dyb"], stream=main)
            ev = torch.cuda.Event()
            ev.record(main)
            side.wait_event(ev)
            tc.wgrad_bf16(cg.NCHW, s, d["dyb"], d["xb"], d["dwb"], self.ws16, stream=side)
            if not d["first"]:
                tc.dgrad_bf16(s, d["dyb"], d["wpd"], d["dxb"], stream=main)
        cg.set_pdl(pdl)
        main.wait_stream(side)

    def wgrad_bf16(self):
        for d in self.L:
            self.tc.wgrad_bf16(self.cg.NCHW, d["s"], d["dyb"], d["xb"], d["dwb"], self.ws16)


def vgg_points_check(torch, O, net, idx_layers, npts=512):
    """Max normwise relative error of y, dx, dW (FP32 and BF16 forms) against FP64 at sampled points."""
    import numpy as np
    rng = np.random.default_rng(5)
    out = {}
    for i in idx_layers:
        d, l = net.L[i], net.layers[i]
        s = d["s"]
        g = dict(b=s.b, h=s.h, w=s.w, c=s.c, kn=s.kn, kh=3, kw=3, vpad=1, hpad=1, vstr=1, hstr=1, vdil=1, hdil=1)
        x = d["x32"].cpu().numpy().ravel()
        w = d["w32"].cpu().numpy().ravel()
        dy = d["dy32"].cpu().numpy().ravel()
        epi = {"bias": d["bias"].cpu().numpy(), "relu": True}
        r = {}
        # forward: NCHW points (b, k, y, x)
        pb, pk, py, px = (rng.integers(0, n, npts) for n in (s.b, s.kn, s.h, s.w))
        idx = ((pb * s.kn + pk) * s.h + py) * s.w + px
        ref = O.fwd_points_f64(O.NCHW, g, w, x, idx, epi)
        got32 = d["y32"].cpu().numpy().ravel()[idx]
        gotb = d["yb"].float().cpu().numpy()[pb, py, px, pk]
        scale = np.abs(ref).max() or 1.0
        r["fwd"] = {"f32": float(np.abs(got32 - ref).max() / scale), "bf16": float(np.abs(gotb - ref).max() / scale)}
        if not d["first"]:
            pc = rng.integers(0, s.c, npts)
            idx = ((pb * s.c + pc) * s.h + py) * s.w + px
            ref = O.dgrad_points_f64(O.NCHW, g, w, dy, idx)
            got32 = d["dx32"].cpu().numpy().ravel()[idx]
            gotb = d["dxb"].float().cpu().numpy()[pb, py, px, pc]
            scale = np.abs(ref).max() or 1.0
            r["dgrad"] = {"f32": float(np.abs(got32 - ref).max() / scale),
                          "bf16": float(np.abs(gotb - ref).max() / scale)}
        idx = rng.integers(0, s.kn * s.c * 9, npts)
        ref = O.wgrad_points_f64(O.NCHW, g, dy, x, idx)
        scale = np.abs(ref).max() or 1.0
        r["wgrad"] = {"f32": float(np.abs(d["dw32"].cpu().numpy().ravel()[idx] - ref).max() / scale),
                      "bf16": float(np.abs(d["dwb"].cpu().numpy().ravel()[idx] - ref).max() / scale)}
        out[l["name"]] = r
    return out


def vgg_cpu_baseline(layers, images, threads=None):
    """The oracle port (FP32 NCHW, the reference's order) on `images` images through the 13 layers:
    forward with bias + ReLU, input gradient (not layer 1), weight gradient.  Returns seconds."""
    import numpy as np
    if threads:
        os.environ["OMP_NUM_THREADS"] = str(threads)
    from oracle import oracle as O
    O.build(with_ref=False)
    rng = np.random.default_rng(3)
    t = 0.0
    for i, l in enumerate(layers):
        g = dict(b=images, h=l["h"], w=l["w"], c=l["c"], kn=l["kn"], kh=3, kw=3, vpad=1, hpad=1, vstr=1, hstr=1,
                 vdil=1, hdil=1)
        K = l["c"] * 9
        x = rng.standard_normal(images * l["c"] * l["h"] * l["w"]).astype(np.float32)
        w = (rng.standard_normal(K * l["kn"]) * np.sqrt(2.0 / K)).astype(np.float32)
        dy = (rng.standard_normal(images * l["kn"] * l["h"] * l["w"]) * 0.1).astype(np.float32)
        y = np.empty(images * l["kn"] * l["h"] * l["w"], np.float32)
        dw = np.empty(K * l["kn"], np.float32)
        dx = np.zeros_like(x)
        epi = {"bias": rng.uniform(-.1, .1, l["kn"]).astype(np.float32), "relu": True}
        t0 = time.perf_counter()
        O.call_fwd("port", O.NCHW, g, w, x, y, epi)
        if i > 0:
            O.call_back("port", O.NCHW, g, w, dy, dx)
        O.call_fwd("port", O.NCHW, g, dy, x, dw, None, trans="T")
        t += time.perf_counter() - t0
    return t


def run_vgg(args):
    """VGG-16 NCHW training step (13 3x3 convs, batch 32): forward (bias + ReLU), input gradient,
    split-K weight gradient, in the FP32 plain form and the BF16 tensor-core form."""
    import torch
    import convgemm_gb300 as cg
    from convgemm_gb300 import tc
    from convgemm_gb300.workloads import vgg16_layers
    local = int(os.environ.get("LOCAL_RANK", "0"))
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    cg.lib()
    layers = vgg16_layers()
    batch = 32 if args.batch == BATCH else args.batch
    net = VggNet(torch, cg, tc, layers, batch)
    flops = sum(conv_flops(l, batch) * (2 if i == 0 else 3) for i, l in enumerate(layers))
    net.step_bf16()
    torch.cuda.synchronize()
    from convgemm_gb300 import autotune
    t0 = time.perf_counter()
    tune_stats = None if args.no_autotune else autotune.tune_ops(net.tune_items())
    tune_s = time.perf_counter() - t0
    net.resize_workspace()
    net.step_f32()
    torch.cuda.synchronize()
    cg.check_device()

    stream = torch.cuda.Stream()
    graphs = {}
    per_step = {}
    for name, fn in (("bf16", net.step_bf16), ("f32", net.step_f32)):
        g = torch.cuda.CUDAGraph()
        with torch.cuda.stream(stream):
            fn()
            stream.synchronize()
            n0 = cg.launch_count()
            with torch.cuda.graph(g, stream=stream):
                fn()
            per_step[name] = cg.launch_count() - n0
        graphs[name] = g
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    ms = timed(torch, graphs["bf16"].replay, args.steps, args.warmup, torch.cuda.current_stream())
    clk = clocks.stop()
    ms32 = timed(torch, graphs["f32"].replay, max(2, args.fp32_steps), 1, torch.cuda.current_stream())
    if world > 1:
        ms, ms32 = max_over_ranks(torch, [ms, ms32])
    cg.check_device()

    # dW bit-reproducibility run to run (both forms), then FP64 point checks
    dw1 = [(d["dw32"].clone(), d["dwb"].clone()) for d in net.L]
    net.wgrad_f32()
    net.wgrad_bf16()
    torch.cuda.synchronize()
    repro = {"f32": all(torch.equal(a, d["dw32"]) for (a, _), d in zip(dw1, net.L)),
             "bf16": all(torch.equal(b, d["dwb"]) for (_, b), d in zip(dw1, net.L))}
    checks = None
    if rank == 0:
        from oracle import oracle as O
        O.build(with_ref=False)
        checks = vgg_points_check(torch, O, net, [0, 6, 12])

    # e2e: the BF16 step through the API with the image batch and the top gradient from pinned
    # host memory and every dW back to pinned host memory
    img_h = torch.randn(batch, 3, 224, 224).pin_memory()
    top_h = (torch.randn(batch, 512, 14, 14) * 0.1).pin_memory()
    dw_h = [torch.empty(d["dwb"].shape).pin_memory() for d in net.L]
    h2d = (img_h.numel() + top_h.numel()) * 4
    d2h = sum(t.numel() * 4 for t in dw_h)

    def e2e_step():
        net.L[0]["x32"].copy_(img_h, non_blocking=True)
        net.L[-1]["dy32"].copy_(top_h, non_blocking=True)
        net.step_bf16()
        for d, h in zip(net.L, dw_h):
            h.copy_(d["dwb"], non_blocking=True)

    for _ in range(2):
        e2e_step()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    n_e2e = max(3, args.steps // 2)
    for _ in range(n_e2e):
        e2e_step()
    torch.cuda.synchronize()
    e2e_ms = (time.perf_counter() - t0) * 1000 / n_e2e

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        t = vgg_cpu_baseline(layers, 1, os.cpu_count())
        cpu = {"value": 1.0 / t, "unit": "img/s", "cores": os.cpu_count(), "kind": "port",
               "sample": "1 image x 13 layers fwd + dX + dW, NCHW FP32, sconvGemmNCHW/_back of the oracle port"}
    peaks, peak_kind = read_peaks()
    tf = flops / (ms / 1000) / 1e12
    ffma_pk = measure_ffma_peak(torch, cg)
    if rank == 0:
        line = {"metric": "VGG-16 NCHW conv training step img/s (fwd + dX + dW), BF16-TC and FP32 plain",
                "value": world * batch / (ms / 1000), "unit": "img/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "bf16", "data": "synthetic",
                "config": {"workload": "vgg16: 13 3x3/s1/p1 convs at 224x224, fwd (bias + ReLU) + dX (not layer 1) "
                                       "+ dW, NCHW FP32 tensors; the BF16 form converts x and dY to NHWC BF16 and "
                                       "packs OIHW weights inside the step (one grouped launch), dW in OIHW FP32",
                           "schedule": "two streams: forward chain; dgrad chain with each wgrad beside it",
                           "global_batch": batch * world, "per_gpu_batch": batch, "seq_len": None,
                           "parallelism": f"replicas{world}", "l2": "inputs larger than L2",
                           "gflop_per_img": flops / batch / 1e9, "autotune": tune_stats, "autotune_s": tune_s},
                "tflops": tf,
                "fp32_plain": {"value": world * batch / (ms32 / 1000), "unit": "img/s", "ms_per_step": ms32,
                               "tflops": flops / (ms32 / 1000) / 1e12, "ffma_peak_tflops": ffma_pk,
                               "frac": flops / (ms32 / 1000) / 1e12 / ffma_pk if ffma_pk else None,
                               "peak_source": "measured FP32 FMA peak (convgemm_measure_ffma, this run)"},
                "bf16_vs_fp32": ms32 / ms,
                "dw_bitwise_reproducible": repro, "fp64_point_errors": checks,
                "roofline": {"bound": "tensor", "kernel": "whole BF16 step", "achieved": tf,
                             "peak": peaks["bf16_tflops_sustained"], "unit": "TFLOP/s",
                             "frac": tf / peaks["bf16_tflops_sustained"], "traffic": None,
                             "peak_source": f"{peak_kind} bf16_tflops_sustained"},
                "cpu_baseline": cpu,
                "e2e": {"value": world * batch / (e2e_ms / 1000), "unit": "img/s", "h2d_bytes_per_step": h2d,
                        "d2h_bytes_per_step": d2h, "ms_per_step": e2e_ms},
                "clocks": clk, "gpu_launches": per_step["bf16"] * args.steps}
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def run_forms(args):
    """Forward pass of the 53 ResNet-50 convolutions at batch 128 in the three tensor-core
    forms: BF16, FP8-E4M3 (per-tensor activation scale, per-channel weight scales, FP32
    accumulation) and 3xBF16 (split products, FP32 output).  Each form's forward over all
    layers is one CUDA graph; errors are max / RMS relative (normwise) against FP64 at
    sampled output points of image 0 of every layer."""
    import numpy as np
    import torch
    import convgemm_gb300 as cg
    from convgemm_gb300 import tc
    from oracle import oracle as O
    local = int(os.environ.get("LOCAL_RANK", "0"))
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    cg.lib()
    if rank == 0:
        O.build(with_ref=False)
    layers = resnet50_layers()
    batch = 128 if args.batch == BATCH else args.batch
    gen = torch.Generator(device="cuda").manual_seed(20261205)
    L = []
    for i, l in enumerate(layers):
        s = cg.Shape.of(batch, l["h"], l["w"], l["c"], l["kn"], l["k"], l["k"], l["pad"], l["pad"], l["stride"],
                        l["stride"], 1, 1)
        K, kn = l["c"] * l["k"] * l["k"], l["kn"]
        d = {"s": s, "l": l, "relu": not (l["name"].endswith("conv3") or l["name"].endswith("down"))}
        d["x"] = torch.randn(batch, l["h"], l["w"], l["c"], device="cuda", generator=gen)
        d["w"] = torch.randn(K * kn, device="cuda", generator=gen) * (2.0 / K) ** 0.5
        var = torch.rand(kn, device="cuda", generator=gen) * 1.5 + 0.5
        d["epi"] = {"mean": torch.randn(kn, device="cuda", generator=gen) * 0.1,
                    "inv_std": 1.0 / torch.sqrt(var + 1e-5),
                    "gamma": torch.rand(kn, device="cuda", generator=gen) + 0.5,
                    "beta": torch.rand(kn, device="cuda", generator=gen) * 0.2 - 0.1}
        d["scale"], d["shift"] = torch.empty(kn, device="cuda"), torch.empty(kn, device="cuda")
        tc.fold_epilogue(kn, d["scale"], d["shift"], **d["epi"])
        # BF16
        d["xb"] = torch.empty(batch, l["h"], l["w"], c8(l["c"]), device="cuda", dtype=torch.bfloat16)
        tc.to_bf16_nhwc(cg.NHWC, batch, l["c"], l["h"], l["w"], d["x"], d["xb"])
        d["wp"] = torch.empty(tc.weights_size(s, tc.OPERAND_FWD) // 2, device="cuda", dtype=torch.bfloat16)
        tc.pack_weights(cg.NHWC, s, tc.OPERAND_FWD, d["w"], d["wp"])
        d["yb"] = torch.empty(batch, s.ho, s.wo, kn, device="cuda", dtype=torch.bfloat16)
        d["fp8"] = l["c"] % 64 == 0   # FP8 / 3xBF16 forms need channels a multiple of 64 (not the stem)
        if d["fp8"]:
            d["xq"] = torch.empty(d["x"].numel(), dtype=torch.uint8, device="cuda")
            d["xs"] = torch.zeros(2, device="cuda")
            tc.fp8_quantize(d["x"], d["xq"], d["xs"])
            d["wq"] = torch.empty(tc.fp8_weights_size(s), dtype=torch.uint8, device="cuda")
            d["wsc"] = torch.empty(kn, device="cuda")
            tc.fp8_pack_weights(cg.NHWC, s, d["w"], d["wq"], d["wsc"])
            d["sc8"], d["sh8"] = torch.empty(kn, device="cuda"), torch.empty(kn, device="cuda")
            tc.fp8_epilogue_scales(kn, d["scale"], d["shift"], d["wsc"], d["xs"], d["sc8"], d["sh8"])
            d["y8"] = torch.empty(batch, s.ho, s.wo, kn, device="cuda", dtype=torch.bfloat16)
            d["xh"] = torch.empty(d["x"].numel(), dtype=torch.bfloat16, device="cuda")
            d["xl"] = torch.empty_like(d["xh"])
            tc.split_bf16x2(d["x"], d["xh"], d["xl"])
            d["wh"] = torch.empty(d["wp"].numel(), dtype=torch.bfloat16, device="cuda")
            d["wl"] = torch.empty_like(d["wh"])
            tc.bf16x3_pack_weights(cg.NHWC, s, d["w"], d["wh"], d["wl"])
            d["y3"] = torch.empty(batch, s.ho, s.wo, kn, device="cuda")
        L.append(d)
    torch.cuda.synchronize()
    cg.check_device()
    from convgemm_gb300 import autotune
    items = []
    for d in L:
        s = d["s"]
        items.append({"op": tc.TUNE_FWD, "shape": s, "run": lambda ws, d=d, s=s: tc.fwd_bf16(
            s, d["xb"], d["wp"], d["yb"], d["scale"], d["shift"], relu=d["relu"])})
        if d["fp8"]:
            items.append({"op": tc.TUNE_FWD_FP8, "shape": s, "run": lambda ws, d=d, s=s: tc.fwd_fp8(
                s, d["xq"], d["wq"], d["y8"], d["sc8"], d["sh8"], relu=d["relu"])})
            items.append({"op": tc.TUNE_FWD_BF16X3, "shape": s, "run": lambda ws, d=d, s=s: tc.fwd_bf16x3(
                s, d["xh"], d["xl"], d["wh"], d["wl"], d["y3"], d["scale"], d["shift"], relu=d["relu"])})
    t0 = time.perf_counter()
    tune_stats = None if args.no_autotune else autotune.tune_ops(items)
    tune_s = time.perf_counter() - t0

    def fwd(form):
        def run():
            for d in L:
                s = d["s"]
                if form == "bf16" or not d["fp8"]:
                    if form == "bf16":
                        tc.fwd_bf16(s, d["xb"], d["wp"], d["yb"], d["scale"], d["shift"], relu=d["relu"])
                elif form == "fp8":
                    tc.fwd_fp8(s, d["xq"], d["wq"], d["y8"], d["sc8"], d["sh8"], relu=d["relu"])
                else:
                    tc.fwd_bf16x3(s, d["xh"], d["xl"], d["wh"], d["wl"], d["y3"], d["scale"], d["shift"],
                                  relu=d["relu"])
        return run

    peaks, peak_kind = read_peaks()
    fp8_pk = measure_fp8_peak(torch)
    stream = torch.cuda.Stream()
    res = {}
    clk = None
    for form in ("bf16", "fp8", "bf16x3"):
        fn = fwd(form)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.stream(stream):
            fn()
            stream.synchronize()
            n0 = cg.launch_count()
            with torch.cuda.graph(g, stream=stream):
                fn()
            nl = cg.launch_count() - n0
        torch.cuda.synchronize()
        clocks = ClockSampler(local) if form == "fp8" else None
        ms = timed(torch, g.replay, args.steps, args.warmup, torch.cuda.current_stream())
        if clocks:
            clk = clocks.stop()
        if world > 1:
            ms = max_over_ranks(torch, [ms])[0]
        cg.check_device()
        fl = sum(conv_flops(d["l"], batch) for d in L if form == "bf16" or d["fp8"])
        issued = fl * (3 if form == "bf16x3" else 1)
        peak = (fp8_pk or peaks["bf16_tflops"] * 2) if form == "fp8" else peaks["bf16_tflops"]
        res[form] = {"ms": ms, "gflop": fl / 1e9, "tflops": fl / (ms / 1000) / 1e12,
                     "issued_tflops": issued / (ms / 1000) / 1e12, "launches": nl,
                     "tensor_frac": issued / (ms / 1000) / 1e12 / peak,
                     "layers": sum(1 for d in L if form == "bf16" or d["fp8"])}
        del g

    # errors against FP64 at sampled points of image 0
    if rank == 0:
        rng = np.random.default_rng(9)
        errs = {"bf16": [], "fp8": [], "bf16x3": []}
        for d in L:
            s, l = d["s"], d["l"]
            g1 = dict(b=1, h=s.h, w=s.w, c=s.c, kn=s.kn, kh=s.kh, kw=s.kw, vpad=s.vpad, hpad=s.hpad,
                      vstr=s.vstride, hstr=s.hstride, vdil=1, hdil=1)
            x0 = d["x"][0].contiguous().cpu().numpy().ravel()
            w = d["w"].cpu().numpy()
            epi = {k: v.cpu().numpy() for k, v in d["epi"].items()}
            epi["relu"] = d["relu"]
            npts = 1024
            py, px, pk = rng.integers(0, s.ho, npts), rng.integers(0, s.wo, npts), rng.integers(0, s.kn, npts)
            idx = (py * s.wo + px) * s.kn + pk
            ref = O.fwd_points_f64(O.NHWC, g1, w, x0, idx, epi)
            outs = {"bf16": d["yb"][0].float().cpu().numpy().ravel()[idx]}
            if d["fp8"]:
                outs["fp8"] = d["y8"][0].float().cpu().numpy().ravel()[idx]
                outs["bf16x3"] = d["y3"][0].cpu().numpy().ravel()[idx]
            for f, o in outs.items():
                dd = o - ref
                errs[f].append((float(np.abs(dd).max() / max(np.abs(ref).max(), 1e-300)),
                                float(np.sqrt(np.mean(dd * dd)) / max(np.sqrt(np.mean(ref * ref)), 1e-300)),
                                l["name"]))
        for f, e in errs.items():
            worst = max(e)
            res[f].update({"max_rel_err": worst[0], "max_rel_err_layer": worst[2],
                           "rms_rel_err": max(v[1] for v in e)})
        line = {"metric": "ResNet-50 layer set forward at batch 128: TFLOP/s and error of the FP8-E4M3 and "
                          "3xBF16 forms beside BF16",
                "value": res["fp8"]["tflops"], "unit": "TFLOP/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": res["fp8"]["ms"], "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "e4m3", "data": "synthetic",
                "config": {"workload": "resnet50 v1.5 53 convs forward (folded BN + ReLU), batch 128, NHWC; FP8 and "
                                       "3xBF16 on the 52 layers with channels a multiple of 64 (the stem stays BF16 "
                                       "and is not counted in their lines)",
                           "global_batch": batch * world, "parallelism": f"replicas{world}",
                           "l2": "inputs larger than L2", "autotune": tune_stats, "autotune_s": tune_s},
                "forms": res,
                "roofline": {"bound": "tensor", "kernel": "tc_conv_kernel (FP8 forward)",
                             "achieved": res["fp8"]["tflops"], "peak": fp8_pk or peaks["bf16_tflops"] * 2,
                             "unit": "TFLOP/s", "frac": res["fp8"]["tensor_frac"], "traffic": None,
                             "peak_source": "measured FP8-E4M3 dense GEMM (cuBLASLt 8192^3 via torch._scaled_mm, "
                                            "this run)" if fp8_pk else
                                            f"2 x {peak_kind} bf16_tflops (the nominal FP8:BF16 dense ratio)"},
                "errors_how": "normwise max|d|/max|ref| and RMS(d)/RMS(ref) against the FP64 direct convolution of "
                              "the FP32 inputs at 1024 sampled outputs of image 0 of every layer; worst layer",
                "cpu_baseline": None, "e2e": None, "clocks": clk,
                "gpu_launches": res["fp8"]["launches"] * args.steps}
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def run_grouped(args):
    """256 independent uneven BF16 convolutions (bias + ReLU): one persistent grouped launch
    in a CUDA graph, against one launch per convolution (also in a CUDA graph)."""
    import torch
    import convgemm_gb300 as cg
    from convgemm_gb300 import autotune, tc
    from convgemm_gb300.workloads import uneven_convs
    local = int(os.environ.get("LOCAL_RANK", "0"))
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    cg.lib()
    specs = uneven_convs(args.group_n, 2024)
    gen = torch.Generator(device="cuda").manual_seed(7)
    convs, singles, flops = [], [], 0
    in_bytes = out_bytes = 0
    for d in specs:
        s = cg.Shape.of(d["b"], d["h"], d["w"], d["c"], d["kn"], d["k"], d["k"], d["pad"], d["pad"],
                        d["stride"], d["stride"], 1, 1)
        K = d["c"] * d["k"] * d["k"]
        x = (torch.rand(d["b"], d["h"], d["w"], d["c"], device="cuda", generator=gen) * 2 - 1).to(torch.bfloat16)
        w32 = torch.randn(K * d["kn"], device="cuda", generator=gen) * (2.0 / K) ** 0.5
        bias = torch.rand(d["kn"], device="cuda", generator=gen) * 0.2 - 0.1
        wp = torch.empty(tc.group_weights_size(s) // 2, dtype=torch.bfloat16, device="cuda")
        tc.group_pack_weights(cg.NHWC, s, w32, wp)
        ws = torch.empty(tc.weights_size(s, tc.OPERAND_FWD) // 2, dtype=torch.bfloat16, device="cuda")
        tc.pack_weights(cg.NHWC, s, tc.OPERAND_FWD, w32, ws)
        y = torch.empty(d["b"], s.ho, s.wo, d["kn"], dtype=torch.bfloat16, device="cuda")
        y1 = torch.empty_like(y)
        convs.append(dict(shape=s, x=x, w=wp, y=y, shift=bias, relu=True))
        singles.append((s, x, ws, y1, bias))
        flops += 2 * d["b"] * s.ho * s.wo * d["kn"] * K
        in_bytes += x.numel() * 2
        out_bytes += y.numel() * 2
    torch.cuda.synchronize()

    t0 = time.perf_counter()
    widths = autotune.tune(convs)
    tune_s = time.perf_counter() - t0
    grp = tc.Group(convs)
    default_grp = tc.Group([dict(c, bn=autotune.default_width(c["shape"].kn)) for c in convs])

    def per_conv():
        for (s, x, ws, y1, bias) in singles:
            tc.fwd_bf16(s, x, ws, y1, None, bias, relu=True)

    stream = torch.cuda.Stream()
    graphs = {}
    per_step = {}
    for name, fn in (("grouped", grp.launch), ("grouped_default_widths", default_grp.launch),
                     ("per_conv", per_conv)):
        with torch.cuda.stream(stream):
            fn()
            stream.synchronize()
            g = torch.cuda.CUDAGraph()
            n0 = cg.launch_count()
            with torch.cuda.graph(g, stream=stream):
                fn()
            per_step[name] = cg.launch_count() - n0
        graphs[name] = g
    torch.cuda.synchronize()
    cg.check_device()
    diff = max(((a["y"].float() - b[3].float()).abs().max() / b[3].float().abs().max().clamp_min(1e-30)).item()
               for a, b in zip(convs, singles))

    clocks = ClockSampler(local)
    ms = timed(torch, graphs["grouped"].replay, args.steps, args.warmup, torch.cuda.current_stream())
    clk = clocks.stop()
    times = {"grouped": ms}
    for name in ("grouped_default_widths", "per_conv"):
        times[name] = timed(torch, graphs[name].replay, args.steps, args.warmup, torch.cuda.current_stream())
    times["per_conv_eager"] = timed(torch, per_conv, max(3, args.steps // 2), 1, torch.cuda.current_stream())
    if world > 1:
        ms = max_over_ranks(torch, [ms])[0]
    cg.check_device()
    value = world * flops / (ms / 1000) / 1e12

    # e2e: inputs from pinned host memory, one grouped launch, outputs back to pinned host memory
    xh = [torch.empty(c["x"].shape, dtype=torch.bfloat16).pin_memory() for c in convs]
    yh = [torch.empty(c["y"].shape, dtype=torch.bfloat16).pin_memory() for c in convs]
    for a, c in zip(xh, convs):
        a.copy_(c["x"])

    def e2e_step():
        for a, c in zip(xh, convs):
            c["x"].copy_(a, non_blocking=True)
        grp.launch()
        for a, c in zip(yh, convs):
            a.copy_(c["y"], non_blocking=True)

    e2e_ms = timed(torch, e2e_step, max(3, args.steps // 2), 1, torch.cuda.current_stream())
    peaks, peak_kind = read_peaks()
    roof = {"bound": "tensor", "kernel": "tc_group_kernel", "achieved": value / world, "peak": peaks["bf16_tflops"],
            "unit": "TFLOP/s", "frac": value / world / peaks["bf16_tflops"], "traffic": None,
            "peak_source": f"{peak_kind} bf16_tflops (burst: one launch timed alone)",
            "how": "algorithmic FLOPs (2*b*ho*wo*kn*c*k*k summed over the convolutions) / CUDA-event time of one "
                   "graph replay of the single grouped launch"}
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        t, fl = grouped_cpu_baseline(specs, 8, os.cpu_count())
        cpu = {"value": fl / t / 1e12, "unit": "TFLOP/s", "cores": os.cpu_count(), "kind": "port",
               "sample": f"every 8th convolution ({len(specs[::8])} of {len(specs)}) in FP32, "
                         "sconvGemmNHWC of the oracle port"}
    if rank == 0:
        hist = {str(w): widths.count(w) for w in sorted(set(widths))}
        line = {"metric": "grouped uneven convolutions: TFLOP/s of one persistent launch", "value": value,
                "unit": "TFLOP/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "bf16", "data": "synthetic",
                "config": {"workload": f"{len(specs)} seeded uneven NHWC BF16 forward convs (batch 1-32, "
                                       "H=W in 7..112, Ci/Co 16..512 step 16, k 1/3/5, stride 1/2, pad k/2), "
                                       "bias + ReLU",
                           "gflop_per_step": flops / 1e9, "input_gb": in_bytes / 1e9, "output_gb": out_bytes / 1e9,
                           "l2": "inputs larger than L2", "parallelism": f"replicas{world}",
                           "tile_widths": hist, "autotune_s": tune_s},
                "times_ms": times, "speedup_vs_per_conv_graph": times["per_conv"] / ms,
                "max_rel_diff_vs_per_conv": diff, "roofline": roof, "cpu_baseline": cpu,
                "e2e": {"value": world * flops / (e2e_ms / 1000) / 1e12, "unit": "TFLOP/s",
                        "h2d_bytes_per_step": in_bytes, "d2h_bytes_per_step": out_bytes, "ms_per_step": e2e_ms},
                "clocks": clk, "gpu_launches": per_step["grouped"] * args.steps,
                "per_conv_launches_per_step": per_step["per_conv"]}
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--batch", type=int, default=BATCH)
    ap.add_argument("--fp32-steps", type=int, default=3)
    ap.add_argument("--no-fp32", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--ref-images", type=int, default=1)
    ap.add_argument("--per-layer", default=None,
                    help="write a per-layer table (forward / input grad / weight grad times) to this JSON file")
    ap.add_argument("--only", default=None,
                    help="LAYER:OP (e.g. s3b2_conv2:fwd; fwd32 / dgrad32 / wgrad32 for the FP32 drop-in): run "
                         "just that op, eagerly, warmup+steps times (for profiler captures)")
    ap.add_argument("--workload", default="resnet50", choices=["resnet50", "grouped", "vgg16", "forms"],
                    help="resnet50: the headline fwd+bwd step; grouped: uneven convolutions in one launch")
    ap.add_argument("--group-n", type=int, default=256)
    ap.add_argument("--no-autotune", action="store_true",
                    help="built-in tile heuristics only (no tuning table)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "grouped":
        return run_grouped(args)
    if args.workload == "vgg16":
        return run_vgg(args)
    if args.workload == "forms":
        return run_forms(args)

    import torch
    import convgemm_gb300 as cg
    from convgemm_gb300 import autotune, tc

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    cg.lib()
    layers = resnet50_layers()
    batch = args.batch
    if args.only:
        return run_only(torch, cg, tc, layers, batch, args)
    net = Net(torch, cg, tc, layers, batch, with_fp32=not args.no_fp32)
    flops = step_flops(layers, batch)

    # per-shape tile configuration: tuning table (cached / shipped / measured now)
    net.step_family("prep")
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    tune_stats = None if args.no_autotune else autotune.tune_ops(net.tune_items())
    tune_s = time.perf_counter() - t0
    net.resize_workspace()

    # warm every launch path once outside any capture (attribute setup, error word)
    net.step_bf16()
    torch.cuda.synchronize()
    cg.check_device()

    # ---- value: the step as one CUDA graph
    stream = torch.cuda.Stream()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.stream(stream):
        net.step_bf16()
        torch.cuda.synchronize()
        n0 = cg.launch_count()
        with torch.cuda.graph(graph, stream=stream):
            net.step_bf16()
        launches_per_step = cg.launch_count() - n0
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clocks = ClockSampler(local)
    ms = timed(torch, graph.replay, args.steps, args.warmup, torch.cuda.current_stream())
    clk = clocks.stop()
    if world > 1:
        ms = max_over_ranks(torch, [ms])[0]
    cg.check_device()
    value = world * batch / (ms / 1000.0)

    # ---- per-kernel-family device times: each family captured as its own graph and replayed
    peaks, peak_kind = read_peaks()
    fam_summary = {}
    for fam in ("prep", "fwd", "dgrad", "wgrad"):
        g_f = torch.cuda.CUDAGraph()
        with torch.cuda.stream(stream):
            n0 = cg.launch_count()
            with torch.cuda.graph(g_f, stream=stream):
                net.step_family(fam)
            n_launch = cg.launch_count() - n0
        torch.cuda.synchronize()
        ms_f = timed(torch, g_f.replay, max(5, args.steps), 2, torch.cuda.current_stream())
        fl = net.family_flops(fam)
        fam_summary[fam] = {"ms": ms_f, "launches": n_launch, "tflops": fl / (ms_f / 1000) / 1e12 if fl else 0.0,
                            "gflop": fl / 1e9}
        del g_f
    kern_of = {"fwd": "tc_conv_kernel (forward)", "dgrad": "tc_conv_kernel (input gradient)",
               "wgrad": "tc_wgrad_kernel + tc_stem_wgrad_kernel + wgrad_reduce_kernel"}
    dominant = max(("fwd", "dgrad", "wgrad"), key=lambda k: fam_summary[k]["ms"])
    dom = fam_summary[dominant]
    # algorithmic bytes of the family per step: each operand of each layer once
    alg_bytes = sum(layer_bytes(l, batch, dominant) for d, l in zip(net.L, layers)
                    if not (dominant == "dgrad" and d["first"]))
    traffic = profile_traffic(("tc_wgrad_kernel", "tc_stem_wgrad_kernel", "wgrad_reduce_kernel",
                               "wgrad_group_sum_kernel")) \
        if dominant == "wgrad" else None
    roofline = {"bound": "tensor", "kernel": kern_of[dominant], "achieved": dom["tflops"],
                "peak": peaks["bf16_tflops_sustained"], "unit": "TFLOP/s",
                "frac": dom["tflops"] / peaks["bf16_tflops_sustained"], "traffic": traffic,
                "traffic_unit": "bytes per step of the family",
                "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one step's launches, "
                                  "profiles/launches_resnet50_bf16_b64.md (cold cache between launches)",
                "algorithmic_bytes": alg_bytes,
                "peak_source": f"{peak_kind} bf16_tflops_sustained (kernel timed inside a long step)",
                "how": "each kernel family of the step captured as its own CUDA graph, replayed, CUDA events; "
                       "achieved = algorithmic FLOPs (2*b*ho*wo*kn*c*kh*kw per conv) / device time",
                "families": fam_summary}

    if args.per_layer and rank == 0:
        per_layer_table(torch, net, layers, batch, peaks, args.per_layer)

    # ---- e2e: public API call by call, host buffers in and out every step
    img_host = torch.randn(batch, 224, 224, 3).pin_memory()
    top_host = torch.randn(batch, 7, 7, 2048).pin_memory()
    img_dev = torch.empty(batch, 224, 224, 3, device="cuda")
    top_dev = torch.empty(batch, 7, 7, 2048, device="cuda")
    dw_host = [torch.empty(d["dw"].numel()).pin_memory() for d in net.L]
    h2d = img_host.numel() * 4 + top_host.numel() * 4
    d2h = sum(t.numel() * 4 for t in dw_host)

    def e2e_step():
        img_dev.copy_(img_host, non_blocking=True)
        top_dev.copy_(top_host, non_blocking=True)
        tc.to_bf16_nhwc(cg.NHWC, batch, 3, 224, 224, img_dev, net.L[0]["x"])
        tc.to_bf16_nhwc(cg.NHWC, batch, 2048, 7, 7, top_dev, net.L[-1]["dy"])
        net.step_bf16()
        for d, hbuf in zip(net.L, dw_host):
            hbuf.copy_(d["dw"], non_blocking=True)

    e2e_steps = max(3, args.steps // 2)
    for _ in range(args.warmup):
        e2e_step()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_step()
    torch.cuda.synchronize()
    e2e_ms = (time.perf_counter() - t0) * 1000 / e2e_steps
    e2e = {"value": world * batch / (e2e_ms / 1000), "unit": "img/s", "h2d_bytes_per_step": h2d,
           "d2h_bytes_per_step": d2h, "ms_per_step": e2e_ms,
           "how": "python ctypes calls per layer on the current stream, no graph; pinned host buffers; "
                  "wall clock around the steps with a device sync after the last"}

    # ---- FP32 plain form
    fp32 = None
    if not args.no_fp32:
        net.step_f32()
        torch.cuda.synchronize()
        cg.check_device()
        ms32 = timed(torch, net.step_f32, args.fp32_steps, 1, torch.cuda.current_stream())
        ffma_pk = measure_ffma_peak(torch, cg)
        tf32 = flops / (ms32 / 1000) / 1e12
        fp32 = {"value": world * batch / (ms32 / 1000), "unit": "img/s", "ms_per_step": ms32,
                "tflops": tf32, "ffma_peak_tflops": ffma_pk, "frac": tf32 / ffma_pk if ffma_pk else None,
                "peak_source": "measured FP32 FMA peak (convgemm_measure_ffma, this run)"}

    # ---- CPU baseline (oracle port) on this host's cores, rank 0 only
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        t, n = cpu_baseline_run(layers, 1, os.cpu_count())
        cpu = {"value": n / t, "unit": "img/s", "cores": os.cpu_count(), "kind": "port",
               "sample": "1 image x 53 layers fwd+wgrad+dgrad, FP32 in the reference's KC=384 order"}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "img/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "bf16", "data": "synthetic",
                "config": {"workload": "resnet50 v1.5: 53 convs, fwd (folded BN + ReLU) + input grad (not stem) "
                                       "+ weight grad, NHWC, BF16 tcgen05, FP32 accumulate",
                           "global_batch": batch * world, "per_gpu_batch": batch, "seq_len": None,
                           "parallelism": f"replicas{world}", "step": "one CUDA graph replay",
                           "schedule": "two streams: forward chain with each downsample conv beside its block; "
                                       "backward dgrad chain on one stream, wgrad of layer i on the other once "
                                       "dY_i exists",
                           "l2": "inputs larger than L2 (per-step working set of several GB)",
                           "gflop_per_img": flops / batch / 1e9,
                           "autotune": tune_stats, "autotune_s": tune_s},
                "tflops": flops / (ms / 1000) / 1e12,
                "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "fp32_plain": fp32,
                "bf16_vs_fp32": (value / fp32["value"]) if fp32 else None,
                "clocks": clk, "gpu_launches": launches_per_step * args.steps,
                "gpu_launches_how": "library launch counter (convgemm_launch_count) across the capture of one step, x steps"}
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
