"""Generates tests/golden/*.npz from the reference's own code.

Run in the container that holds the reference checkout:
    make -C oracle ref && python tests/golden/make_golden.py

For every case in cases.py it calls the shim-built reference
(oracle/_ref/libconvgemm_ref.so: the reference's convGemm.c, loop nests,
packers and epilogues, compiled unmodified) through its public entry points
sconvGemmNHWC / sconvGemmNCHW / sconvGemm*_back, and stores the output, a
SHA-256 of its bytes and of the inputs.  The dgrad cases run the reference
with one OpenMP thread so its atomic scatter has a fixed order.
"""
from __future__ import annotations

import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, HERE)

from oracle import oracle as O  # noqa: E402
import cases as C  # noqa: E402


def run_case(name, op, layout, g, epi_kind, data):
    inp = C.make_inputs(name, op, layout, g, epi_kind, data)
    ho, wo = C.out_hw(g)
    K = g["c"] * g["kh"] * g["kw"]
    if op == "fwd":
        out = np.zeros(g["b"] * ho * wo * g["kn"], np.float32)
        O.call_fwd("ref", layout, g, inp["w"], inp["x"], out, inp["epi"], trans="N")
    elif op == "wgrad":
        out = np.zeros(K * g["kn"], np.float32)
        O.call_fwd("ref", layout, g, inp["dy"], inp["x"], out, None, trans="T")
    else:
        out = inp["dx0"].copy()
        O.call_back("ref", layout, g, inp["w"], inp["dy"], out)
    return inp, out


def main():
    os.environ.setdefault("OMP_NUM_THREADS", "1")
    if not O.ref_available():
        O.build(with_ref=True)
    for case in C.CASES:
        name = case[0]
        inp, out = run_case(*case)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), out=out,
                            out_sha256=hashlib.sha256(out.tobytes()).hexdigest(), in_sha256=inp["hash"])
        print(f"{name}: {out.size} outputs, sha256 {hashlib.sha256(out.tobytes()).hexdigest()[:16]}")


if __name__ == "__main__":
    main()
