"""Packed-weight cache (convgemm_weights_cached): a hit returns the same operand
without a launch, a new version re-packs in place, evicting frees, a miss during
stream capture is refused, and the cached operands are byte-identical to the
ones the per-call packing entry points write.  The reference re-packs weights on
every call (pack_RB, src/gemm_blis.c:40-88)."""
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


class _DeviceBytes:
    """A view of n bytes of device memory at addr, for torch.as_tensor."""

    def __init__(self, addr, n):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": "|u1", "data": (addr, False), "version": 2}


def _bytes_at(addr, nbytes):
    torch.cuda.synchronize()
    return torch.as_tensor(_DeviceBytes(addr, nbytes), device="cuda").clone()


def test_cache_hit_repack_evict(cglib):
    from convgemm_gb300 import tc
    cg = cglib
    s = cg.Shape.of(4, 14, 14, 64, 128, 3, 3, 1, 1)
    K = 64 * 9
    w = torch.randn(K * 128, device="cuda")
    for kind, op in ((tc.CACHE_BF16_FWD, tc.OPERAND_FWD), (tc.CACHE_BF16_DGRAD, tc.OPERAND_DGRAD)):
        nb = tc.weights_size(s, op)
        want = torch.empty(nb // 2, dtype=torch.bfloat16, device="cuda")
        tc.pack_weights(cg.NHWC, s, op, w, want)
        b0 = tc.weights_cache_bytes()
        a = tc.weights_cached(cg.NHWC, s, kind, w, 7)
        assert tc.weights_cache_bytes() >= b0 + nb
        got = _bytes_at(a, nb)
        assert torch.equal(got, want.view(torch.uint8)), kind
        # a hit: same operand, nothing launched
        n0 = cg.lib().convgemm_launch_count()
        assert tc.weights_cached(cg.NHWC, s, kind, w, 7) == a
        assert cg.lib().convgemm_launch_count() == n0
        # new weights under a new version: re-packed in place
        w.mul_(-0.5)
        assert tc.weights_cached(cg.NHWC, s, kind, w, 8) == a
        assert cg.lib().convgemm_launch_count() > n0
        tc.pack_weights(cg.NHWC, s, op, w, want)
        assert torch.equal(_bytes_at(a, nb), want.view(torch.uint8)), kind
    # another layout of the same pointer is another entry
    b = tc.weights_cached(cg.NCHW, s, tc.CACHE_BF16_FWD, w, 8)
    assert b != tc.weights_cached(cg.NHWC, s, tc.CACHE_BF16_FWD, w, 8)
    assert tc.weights_cache_evict(w) == 3
    assert tc.weights_cache_evict(w) == 0


def test_cache_fp8_operand_and_scales(cglib):
    from convgemm_gb300 import tc
    cg = cglib
    s = cg.Shape.of(2, 8, 8, 64, 64, 3, 3, 1, 1)
    w = torch.randn(64 * 9 * 64, device="cuda")
    nb = tc.fp8_weights_size(s)
    want = torch.empty(nb, dtype=torch.uint8, device="cuda")
    ws_want = torch.empty(64, device="cuda")
    tc.fp8_pack_weights(cg.NHWC, s, w, want, ws_want)
    a, sc = tc.weights_cached(cg.NHWC, s, tc.CACHE_FP8_FWD, w, 1)
    assert torch.equal(_bytes_at(a, nb), want)
    assert torch.equal(_bytes_at(sc, 256), ws_want.view(torch.uint8))
    assert tc.weights_cache_evict(w) == 1


def test_cache_miss_refused_during_capture_hit_allowed(cglib):
    from convgemm_gb300 import tc
    cg = cglib
    s = cg.Shape.of(2, 10, 10, 64, 64, 3, 3, 1, 1)
    w = torch.randn(64 * 9 * 64, device="cuda")
    w2 = torch.randn(64 * 9 * 64, device="cuda")
    x = torch.randn(2, 10, 10, 64, device="cuda").to(torch.bfloat16)
    y = torch.empty(2, 10, 10, 64, dtype=torch.bfloat16, device="cuda")
    a = tc.weights_cached(cg.NHWC, s, tc.CACHE_BF16_FWD, w, 0)
    st = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    refused = None
    with torch.cuda.stream(st):
        torch.cuda.synchronize()
        with torch.cuda.graph(g, stream=st):
            assert tc.weights_cached(cg.NHWC, s, tc.CACHE_BF16_FWD, w, 0) == a   # hit: fine
            tc.fwd_bf16(s, x, a, y)
            try:
                tc.weights_cached(cg.NHWC, s, tc.CACHE_BF16_FWD, w2, 0)        # miss: refused
            except cg.ConvGemmError as e:
                refused = e
    assert refused is not None and refused.status == 2 and "captured" in str(refused)
    g.replay()
    torch.cuda.synchronize()
    want = torch.empty_like(y)
    tc.fwd_bf16(s, x, a, want)
    torch.cuda.synchronize()
    assert torch.equal(y, want)
    tc.weights_cache_evict(w)
    assert tc.weights_cache_evict(w2) == 0


def test_torch_op_with_cache_matches_uncached(cglib):
    from convgemm_gb300 import torch_ops
    torch.manual_seed(3)
    x = torch.randn(2, 12, 12, 64, device="cuda").to(torch.bfloat16)
    w = torch.randn(64, 3, 3, 32, device="cuda") * 0.05
    prev = torch_ops.cache_weights(False)
    try:
        want = torch_ops.conv2d_nhwc(x, w, None, None, 1, 1, 1, True)
        torch_ops.cache_weights(True)
        got = torch_ops.conv2d_nhwc(x, w, None, None, 1, 1, 1, True)
        assert torch.equal(got, want)
        # an in-place update bumps the version: the next call re-packs
        with torch.no_grad():
            w.mul_(2.0)
        got2 = torch_ops.conv2d_nhwc(x, w, None, None, 1, 1, 1, True)
        torch_ops.cache_weights(False)
        want2 = torch_ops.conv2d_nhwc(x, w, None, None, 1, 1, 1, True)
        assert torch.equal(got2, want2)
        assert not torch.equal(got2, got)
    finally:
        torch_ops.cache_weights(prev)
