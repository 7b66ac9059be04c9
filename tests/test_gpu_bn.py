"""GPU tests of training-mode batch normalisation around the BF16 forward: batch
statistics fused into the convolution's epilogue (general and small-channel kernels),
their fold into scale / shift, and the normalising apply.

The statistics are compared with the FP64 oracle's z = conv + bias on the same
BF16-rounded inputs (the only difference left is the FP32 accumulation of the tensor
cores and of the 32-pixel partial sums), the fold with an FP64 NumPy restatement, and
the apply with a PyTorch FP32 computation on the same BF16 z.
"""
import numpy as np
import pytest

import cases as C

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

STATS_TOL = 1e-4   # |sum_got - sum_ref| <= STATS_TOL * sum |z| (and the same for the squares)

SHAPES = [
    # b, h, w, c, kn, k, pad, stride
    (2, 14, 14, 64, 128, 3, 1, 1),     # general kernel, M = 392 (not a multiple of 128)
    (1, 13, 11, 64, 72, 3, 1, 1),      # ragged N tile, M = 143
    (2, 15, 15, 64, 64, 3, 1, 2),      # stride 2
    (3, 8, 8, 256, 512, 1, 0, 1),      # 1x1, several N tiles
    (2, 20, 20, 3, 64, 7, 3, 2),       # small-channel kernel (stem)
    (1, 9, 150, 3, 64, 3, 1, 1),       # small-channel kernel, two 128-pixel chunks per row
]


def bf16r(a):
    return torch.from_numpy(np.ascontiguousarray(a)).to(torch.bfloat16).float().numpy()


@pytest.mark.parametrize("shape", SHAPES, ids=[str(s) for s in SHAPES])
def test_forward_batch_statistics(cglib, oracle_lib, shape):
    from convgemm_gb300 import tc
    cg, O = cglib, oracle_lib
    b, h, w, c, kn, k, pad, stride = shape
    s = cg.Shape.of(b, h, w, c, kn, k, k, pad, pad, stride, stride)
    g = C.geom(b, h, w, c, kn, k, k, pad=pad, stride=stride)
    rng = np.random.default_rng(sum(shape) + 11)
    K = c * k * k
    x = rng.standard_normal(b * h * w * c).astype(np.float32)
    wt = (rng.standard_normal(K * kn) * np.sqrt(2.0 / K)).astype(np.float32)
    bias = rng.uniform(-.5, .5, kn).astype(np.float32)
    xd = torch.empty(b, h, w, tc.c8(c), dtype=torch.bfloat16, device="cuda")
    tc.to_bf16_nhwc(cg.NHWC, b, c, h, w, torch.from_numpy(x).cuda(), xd)
    wp = torch.empty(tc.weights_size(s, tc.OPERAND_FWD) // 2, dtype=torch.bfloat16, device="cuda")
    tc.pack_weights(cg.NHWC, s, tc.OPERAND_FWD, torch.from_numpy(wt).cuda(), wp)
    shift = torch.from_numpy(bias).cuda()
    y = torch.empty(b, s.ho, s.wo, kn, dtype=torch.bfloat16, device="cuda")
    y_plain = torch.empty_like(y)
    stats = torch.empty(2, kn, dtype=torch.float64, device="cuda")
    stats2 = torch.empty_like(stats)
    tc.fwd_bf16_stats(s, xd, wp, y, stats, shift=shift)
    tc.fwd_bf16_stats(s, xd, wp, y, stats2, shift=shift)
    tc.fwd_bf16(s, xd, wp, y_plain, None, shift, relu=False)
    torch.cuda.synchronize()
    cg.check_device()
    # the statistics do not change the output, and are bit-reproducible
    assert torch.equal(y.view(torch.int16), y_plain.view(torch.int16))
    assert torch.equal(stats, stats2)
    z = O.fwd_f64(C.NHWC, g, bf16r(wt), bf16r(x), {"bias": bias, "relu": False}).reshape(-1, kn)
    got = stats.cpu().numpy()
    for q, ref, scale in ((0, z.sum(0), np.abs(z).sum(0)), (1, (z * z).sum(0), (z * z).sum(0))):
        err = np.abs(got[q] - ref) / np.maximum(scale, 1e-30)
        assert err.max() <= STATS_TOL, (q, err.max())


def test_batch_norm_fold_and_apply(cglib):
    from convgemm_gb300 import tc
    rng = np.random.default_rng(3)
    npix, kn, count = 1000, 72, 1000
    z = torch.from_numpy(rng.standard_normal((npix, kn)).astype(np.float32) * 2 + 0.5).to(torch.bfloat16).cuda()
    zf = z.float().cpu().numpy().astype(np.float64)
    stats = torch.from_numpy(np.stack([zf.sum(0), (zf * zf).sum(0)])).cuda()
    gamma = torch.from_numpy(rng.uniform(.5, 1.5, kn).astype(np.float32)).cuda()
    beta = torch.from_numpy(rng.uniform(-.2, .2, kn).astype(np.float32)).cuda()
    scale, shift = torch.empty(kn, device="cuda"), torch.empty(kn, device="cuda")
    mean, var = torch.empty(kn, device="cuda"), torch.empty(kn, device="cuda")
    tc.bn_stats_fold(kn, stats, count, scale, shift, gamma=gamma, beta=beta, eps=1e-5, batch_mean=mean, batch_var=var)
    y = torch.empty_like(z)
    tc.bn_apply_bf16(npix, kn, z, scale, shift, y, relu=True)
    torch.cuda.synchronize()
    cglib.check_device()
    m_ref = zf.mean(0)
    v_ref = zf.var(0)
    sc_ref = gamma.cpu().numpy().astype(np.float64) / np.sqrt(v_ref + 1e-5)
    sh_ref = beta.cpu().numpy().astype(np.float64) - m_ref * sc_ref
    np.testing.assert_allclose(mean.cpu().numpy(), m_ref, rtol=1e-6, atol=1e-6)
    np.testing.assert_allclose(var.cpu().numpy(), v_ref, rtol=1e-5)
    np.testing.assert_allclose(scale.cpu().numpy(), sc_ref, rtol=1e-6)
    np.testing.assert_allclose(shift.cpu().numpy(), sh_ref, rtol=1e-5, atol=1e-6)
    ref = torch.relu(z.float() * scale + shift)
    diff = (y.float() - ref).abs()
    assert float((diff - ref.abs() * 2.0 ** -8).max()) <= 1e-6   # one BF16 rounding of the FP32 result
    # in place
    tc.bn_apply_bf16(npix, kn, z, scale, shift, z, relu=True)
    torch.cuda.synchronize()
    assert torch.equal(z.view(torch.int16), y.view(torch.int16))
