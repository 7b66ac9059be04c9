"""Per-layer precision report of the tensor-core forms against the FP64 oracle.

For every convolution of ResNet-50 v1.5 (synthetic inputs: activations N(0,1),
Kaiming-normal weights, batch-norm folded from gamma U[0.5,1.5], beta
U[-0.1,0.1], mean N(0,0.1), var U[0.5,2], ReLU) it runs on the GPU
  * BF16 forward, input gradient (dY ~ N(0, 1e-2)) and weight gradient,
  * FP8-E4M3 forward (per-tensor activation scale, per-channel weight scales),
  * 3xBF16 forward (split products, FP32 output),
and prints a markdown table of max and RMS relative error (normwise: max|d| /
max|ref| and RMS(d) / RMS(ref)) against the FP64 direct convolution of the
FP32 inputs.  Usage (GPU host):  python tests/precision_report.py [--batch 2] [--out FILE]
"""
from __future__ import annotations

import argparse
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, HERE)

from parity import rel_max_rms  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--batch", type=int, default=2)
    ap.add_argument("--out", default=None)
    args = ap.parse_args()
    import torch
    import convgemm_gb300 as cg
    from convgemm_gb300 import tc
    from convgemm_gb300.workloads import resnet50_layers
    from oracle import oracle as O
    O.build(with_ref=False)
    b = args.batch
    rng = np.random.default_rng(20261203)
    rows = []
    for i, l in enumerate(resnet50_layers()):
        g = dict(b=b, h=l["h"], w=l["w"], c=l["c"], kn=l["kn"], kh=l["k"], kw=l["k"], vpad=l["pad"], hpad=l["pad"],
                 vstr=l["stride"], hstr=l["stride"], vdil=1, hdil=1)
        s = cg.Shape.of(b, l["h"], l["w"], l["c"], l["kn"], l["k"], l["k"], l["pad"], l["pad"], l["stride"],
                        l["stride"], 1, 1)
        kn, c, K = l["kn"], l["c"], l["c"] * l["k"] * l["k"]
        relu = not (l["name"].endswith("conv3") or l["name"].endswith("down"))
        x = rng.standard_normal(b * l["h"] * l["w"] * c).astype(np.float32)
        w = (rng.standard_normal(K * kn) * np.sqrt(2.0 / K)).astype(np.float32)
        dy = (rng.standard_normal(b * s.ho * s.wo * kn) * 0.1).astype(np.float32)
        var = rng.uniform(0.5, 2.0, kn)
        epi = {"mean": rng.normal(0, 0.1, kn).astype(np.float32),
               "inv_std": (1.0 / np.sqrt(var + 1e-5)).astype(np.float32),
               "gamma": rng.uniform(0.5, 1.5, kn).astype(np.float32),
               "beta": rng.uniform(-0.1, 0.1, kn).astype(np.float32)}
        e = dict(epi, relu=relu)
        ref_f = O.fwd_f64(O.NHWC, g, w, x, e).ravel()
        ref_d = O.dgrad_f64(O.NHWC, g, w, dy)
        ref_w = O.wgrad_f64(O.NHWC, g, dy, x)
        dev = {k: torch.from_numpy(v).cuda() for k, v in epi.items()}
        scale, shift = torch.empty(kn, device="cuda"), torch.empty(kn, device="cuda")
        tc.fold_epilogue(kn, scale, shift, **dev)
        xt, wt, dyt = torch.from_numpy(x).cuda(), torch.from_numpy(w).cuda(), torch.from_numpy(dy).cuda()
        row = {"layer": l["name"], "shape": f"{l['h']}x{l['w']} {c}->{kn} {l['k']}x{l['k']}/s{l['stride']}"}
        # BF16
        xb = torch.empty(b, l["h"], l["w"], tc.c8(c), dtype=torch.bfloat16, device="cuda")
        tc.to_bf16_nhwc(cg.NHWC, b, c, l["h"], l["w"], xt, xb)
        dyb = torch.empty(b, s.ho, s.wo, tc.c8(kn), dtype=torch.bfloat16, device="cuda")
        tc.to_bf16_nhwc(cg.NHWC, b, kn, s.ho, s.wo, dyt, dyb)
        wp = torch.empty(tc.weights_size(s, tc.OPERAND_FWD) // 2, dtype=torch.bfloat16, device="cuda")
        tc.pack_weights(cg.NHWC, s, tc.OPERAND_FWD, wt, wp)
        y = torch.empty(b, s.ho, s.wo, kn, dtype=torch.bfloat16, device="cuda")
        tc.fwd_bf16(s, xb, wp, y, scale, shift, relu=relu)
        row["bf16_fwd"] = rel_max_rms(y.float().cpu().numpy(), ref_f)
        if c % 8 == 0:
            wpd = torch.empty(tc.weights_size(s, tc.OPERAND_DGRAD) // 2, dtype=torch.bfloat16, device="cuda")
            tc.pack_weights(cg.NHWC, s, tc.OPERAND_DGRAD, wt, wpd)
            dx = torch.empty(b, l["h"], l["w"], c, dtype=torch.bfloat16, device="cuda")
            tc.dgrad_bf16(s, dyb, wpd, dx)
            row["bf16_dgrad"] = rel_max_rms(dx.float().cpu().numpy(), ref_d)
        ws = torch.empty(tc.wgrad_bf16_workspace_size(s) // 4 + 1, device="cuda")
        dw = torch.empty(K * kn, device="cuda")
        tc.wgrad_bf16(cg.NHWC, s, dyb, xb, dw, ws)
        row["bf16_wgrad"] = rel_max_rms(dw.cpu().numpy(), ref_w)
        if c % 64 == 0:
            xq = torch.empty(x.size, dtype=torch.uint8, device="cuda")
            xs = torch.zeros(2, device="cuda")
            tc.fp8_quantize(xt, xq, xs)
            wq = torch.empty(tc.fp8_weights_size(s), dtype=torch.uint8, device="cuda")
            wsc = torch.empty(kn, device="cuda")
            tc.fp8_pack_weights(cg.NHWC, s, wt, wq, wsc)
            sc8, sh8 = torch.empty(kn, device="cuda"), torch.empty(kn, device="cuda")
            tc.fp8_epilogue_scales(kn, scale, shift, wsc, xs, sc8, sh8)
            y8 = torch.empty(b, s.ho, s.wo, kn, dtype=torch.bfloat16, device="cuda")
            tc.fwd_fp8(s, xq, wq, y8, sc8, sh8, relu=relu)
            row["fp8_fwd"] = rel_max_rms(y8.float().cpu().numpy(), ref_f)
            xh = torch.empty(x.size, dtype=torch.bfloat16, device="cuda")
            xl = torch.empty_like(xh)
            tc.split_bf16x2(xt, xh, xl)
            wh = torch.empty(wp.numel(), dtype=torch.bfloat16, device="cuda")
            wl = torch.empty_like(wh)
            tc.bf16x3_pack_weights(cg.NHWC, s, wt, wh, wl)
            y3 = torch.empty(b, s.ho, s.wo, kn, device="cuda")
            tc.fwd_bf16x3(s, xh, xl, wh, wl, y3, scale, shift, relu=relu)
            row["bf16x3_fwd"] = rel_max_rms(y3.cpu().numpy(), ref_f)
        torch.cuda.synchronize()
        cg.check_device()
        rows.append(row)
    cols = ["bf16_fwd", "bf16_dgrad", "bf16_wgrad", "fp8_fwd", "bf16x3_fwd"]
    lines = [f"Per-layer max / RMS relative error vs the FP64 direct convolution (batch {b}).", "",
             "| layer | shape | " + " | ".join(cols) + " |", "|---|---|" + "---|" * len(cols)]
    worst = {c: [0.0, 0.0] for c in cols}
    for r in rows:
        cells = []
        for c_ in cols:
            if c_ in r:
                mx, rms = r[c_]
                worst[c_][0] = max(worst[c_][0], mx)
                worst[c_][1] = max(worst[c_][1], rms)
                cells.append(f"{mx:.1e} / {rms:.1e}")
            else:
                cells.append("n/a")
        lines.append(f"| {r['layer']} | {r['shape']} | " + " | ".join(cells) + " |")
    lines.append("| **worst** | | " + " | ".join(f"**{w[0]:.1e} / {w[1]:.1e}**" for w in worst.values()) + " |")
    text = "\n".join(lines) + "\n"
    if args.out:
        with open(args.out, "w") as f:
            f.write(text)
    print(text)


if __name__ == "__main__":
    main()
