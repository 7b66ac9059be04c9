"""Convolution layer sets of the benchmark workloads, derived from the architectures.

ResNet-50 v1.5 (53 convolutions) and VGG-16 (13 convolutions).  Each layer is
a dict with the convGemm geometry: h, w (input size), c (input channels),
kn (output channels), k (square filter), stride, pad.
"""
from __future__ import annotations


def resnet50_layers():
    """53 conv layers of ResNet-50 v1.5 at 224x224 input (stride 2 on the 3x3 of each first block)."""
    L = [dict(name="conv1", h=224, w=224, c=3, kn=64, k=7, stride=2, pad=3)]
    cin, hw = 64, 56
    for stage, (width, blocks) in enumerate(zip((64, 128, 256, 512), (3, 4, 6, 3))):
        out = width * 4
        for blk in range(blocks):
            s = 2 if (blk == 0 and stage > 0) else 1
            pre = f"s{stage + 1}b{blk + 1}"
            L.append(dict(name=pre + "_conv1", h=hw, w=hw, c=cin, kn=width, k=1, stride=1, pad=0))
            L.append(dict(name=pre + "_conv2", h=hw, w=hw, c=width, kn=width, k=3, stride=s, pad=1))
            hw2 = hw // s
            L.append(dict(name=pre + "_conv3", h=hw2, w=hw2, c=width, kn=out, k=1, stride=1, pad=0))
            if blk == 0:
                L.append(dict(name=pre + "_down", h=hw, w=hw, c=cin, kn=out, k=1, stride=s, pad=0))
            cin, hw = out, hw2
    assert len(L) == 53
    return L


def vgg16_layers():
    """13 3x3/s1/p1 conv layers of VGG-16 at 224x224 input."""
    cfg = [(224, 3, 64), (224, 64, 64), (112, 64, 128), (112, 128, 128), (56, 128, 256), (56, 256, 256),
           (56, 256, 256), (28, 256, 512), (28, 512, 512), (28, 512, 512), (14, 512, 512), (14, 512, 512),
           (14, 512, 512)]
    return [dict(name=f"conv{i + 1}", h=hw, w=hw, c=c, kn=kn, k=3, stride=1, pad=1) for i, (hw, c, kn) in enumerate(cfg)]


def out_hw(layer):
    ho = (layer["h"] + 2 * layer["pad"] - layer["k"]) // layer["stride"] + 1
    wo = (layer["w"] + 2 * layer["pad"] - layer["k"]) // layer["stride"] + 1
    return ho, wo


def conv_flops(layer, batch):
    """2*b*ho*wo*kn*c*k*k: the reference's 2*M*N*K (plots/convgemm.plt:56); the same for fwd, dgrad, wgrad."""
    ho, wo = out_hw(layer)
    return 2 * batch * ho * wo * layer["kn"] * layer["c"] * layer["k"] * layer["k"]


def uneven_convs(n=256, seed=2024):
    """Seeded independent convolutions of uneven shapes for the grouped launch:
    batch 1-32, H = W in {7, 14, 28, 56, 112}, input/output channels in
    {16, 32, ..., 512}, kernel 1/3/5, stride 1/2, pad = k // 2 (NHWC, BF16,
    fused bias + ReLU).  Returns dicts with b, h, w, c, kn, k, stride, pad."""
    import numpy as np
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        k = int(rng.choice([1, 3, 5]))
        h = int(rng.choice([7, 14, 28, 56, 112]))
        out.append(dict(b=int(rng.integers(1, 33)), h=h, w=h, c=16 * int(rng.integers(1, 33)),
                        kn=16 * int(rng.integers(1, 33)), k=k, stride=int(rng.choice([1, 2])), pad=k // 2))
    return out
