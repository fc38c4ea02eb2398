"""The bounded-wait abort path of the pipelined kernels, exercised on the GPU
without a fault: a CTA holding TMEM waits on an mbarrier nobody arrives on,
gives up after a short poll budget, frees TMEM and returns; the host reports
SID_ETIMEOUT and the context keeps working."""
import numpy as np
import pytest

from tests.conftest import rel_l2


def test_selftest_rejects_bad_budget(sidlib):
    from sid_gb300 import _lib
    assert sidlib.sid_selftest_wait_timeout(0, 0) == _lib.SID_EINVAL
    assert sidlib.sid_selftest_wait_timeout(1 << 21, 0) == _lib.SID_EINVAL


@pytest.mark.gpu
def test_wait_runs_out_and_context_survives(gpu):
    from sid_gb300 import Context, _lib, to_device
    lib = _lib.load()
    rc = lib.sid_selftest_wait_timeout(2000, 0)
    assert rc == _lib.SID_ETIMEOUT, lib.sid_last_error()
    assert b"exceeded its budget" in lib.sid_last_error()
    # a barrier that completes: same kernel, no timeout
    assert lib.sid_selftest_wait_timeout(2000, 1) == _lib.SID_OK
    # twice more, so TMEM was released by the aborted CTA
    assert lib.sid_selftest_wait_timeout(50, 0) == _lib.SID_ETIMEOUT
    assert lib.sid_selftest_wait_timeout(50, 1) == _lib.SID_OK
    # the tensor-core pipeline still runs afterwards
    A = np.asfortranarray(np.random.default_rng(3).random((5000, 64)).astype(np.float32))
    G = Context().gram(to_device(A), "split").cpu().numpy()
    A64 = A.astype(np.float64)
    assert rel_l2(G, A64.T @ A64) < 1e-5
