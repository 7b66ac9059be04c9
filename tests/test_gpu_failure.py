"""Failure detection of the device-side waits, exercised without a GPU fault: a
kernel waits on a barrier that nothing completes, with a 20 ms budget; the wait
runs out, records its code and the kernel returns; the host reads
CONVGEMM_ERROR_TIMEOUT from convgemm_check_device, the error word is cleared,
and the context keeps working (a tensor-core convolution runs afterwards)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def test_bounded_wait_timeout_is_reported_and_context_survives(cglib):
    from convgemm_gb300 import tc
    cg = cglib
    L = cg.lib()
    cg.check_device()                      # nothing pending
    assert L.convgemm_selftest_wait_timeout(20, None) == 0
    with pytest.raises(cg.ConvGemmError) as ei:
        cg.check_device()
    assert ei.value.status == 5 and "code 99" in str(ei.value)
    cg.check_device()                      # the word was cleared
    # the context is still usable
    s = cg.Shape.of(1, 8, 8, 64, 64, 3, 3, 1, 1)
    x = torch.randn(1, 8, 8, 64, device="cuda").to(torch.bfloat16)
    wt = torch.randn(64 * 9 * 64, device="cuda") * 0.05
    wp = torch.empty(tc.weights_size(s, tc.OPERAND_FWD) // 2, dtype=torch.bfloat16, device="cuda")
    tc.pack_weights(cg.NHWC, s, tc.OPERAND_FWD, wt, wp)
    y = torch.empty(1, 8, 8, 64, dtype=torch.bfloat16, device="cuda")
    tc.fwd_bf16(s, x, wp, y)
    torch.cuda.synchronize()
    cg.check_device()
    assert torch.isfinite(y.float()).all()


def test_selftest_rejects_bad_budget(cglib):
    assert cglib.lib().convgemm_selftest_wait_timeout(0, None) == 1
    assert cglib.lib().convgemm_selftest_wait_timeout(5000, None) == 1
    assert np.isscalar(cglib.launch_count())
