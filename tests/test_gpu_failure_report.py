"""Failure reports reach the host without any GPU fault.

* A decoupled look-back whose predecessor never publishes (the self-test
  entry point: tile 1 of a fresh scan, tile 0 never written) gives up after
  a short spin limit; the kernel returns, and backend().synchronize() raises
  awkward's ValueError with the library's "bounded wait gave up" message.
  The GPU stays usable: a reduction launched afterwards is correct.
* AWKWARD_GB300_FAULT forces an error code on the host path: the kernel
  runs normally, the stream's error word records the code for that
  invocation, and synchronize() raises that code's message, naming the first
  failing invocation like awkward's synchronize_cuda
  (src/awkward/_connect/cuda/__init__.py:257-294).
"""

import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _sum_case(be):
    import torch

    x = torch.arange(10, dtype=torch.float64, device="cuda")
    off = torch.tensor([0, 3, 3, 10], dtype=torch.int64, device="cuda")
    out = torch.empty(3, dtype=torch.float64, device="cuda")
    k = be["awkward_reduce_sum", np.float64, np.float64, np.int64]
    return k, out, x, off


def test_lookback_that_never_completes_reports_timeout():
    import awkward_gb300
    from awkward_gb300._messages import TIMEOUT_MESSAGE

    be = awkward_gb300.backend()
    be.synchronize()
    t0 = time.perf_counter()
    be.selftest_lookback_timeout(spin_limit=2000)
    with pytest.raises(ValueError, match="bounded wait exceeded"):
        be.synchronize()
    assert time.perf_counter() - t0 < 30
    assert TIMEOUT_MESSAGE.startswith("GPU kernel gave up")
    # the context is intact and the error word was reset
    k, out, x, off = _sum_case(be)
    k(out, x, off, 3)
    be.synchronize()
    np.testing.assert_array_equal(out.cpu().numpy(), [3.0, 0.0, 42.0])


def test_injected_fault_raises_that_code(monkeypatch):
    import torch

    import awkward_gb300
    from awkward_gb300.kernel_table import FAULT_ENV

    be = awkward_gb300.backend()
    be.synchronize()
    k, out, x, off = _sum_case(be)
    monkeypatch.setenv(FAULT_ENV, "awkward_reduce_argmax:32")
    k(out, x, off, 3)  # not targeted: no error
    arg = torch.empty(3, dtype=torch.int64, device="cuda")
    be["awkward_reduce_argmax", np.int64, np.float64, np.int64, np.int64](
        arg, x, off, off[:-1].contiguous(), 3)
    with pytest.raises(ValueError, match=r"bounded wait exceeded.*awkward_reduce_argmax"):
        be.synchronize()
    # the kernel itself ran normally
    np.testing.assert_array_equal(arg.cpu().numpy(), [2, -1, 9])
    monkeypatch.setenv(FAULT_ENV, "awkward_ListArray_getitem_jagged_apply:4")
    be["awkward_ListArray_getitem_jagged_apply", np.int64, np.int64, np.int64, np.int64,
       np.int64, np.int64, np.int64](
        torch.empty(4, dtype=torch.int64, device="cuda"), torch.empty(1, dtype=torch.int64, device="cuda"),
        off[:-1].contiguous(), off[:-1].contiguous(), 3, torch.zeros(1, dtype=torch.int64, device="cuda"),
        1, off[:-1].contiguous(), off[1:].contiguous(), 10)
    with pytest.raises(ValueError, match="index out of range"):
        be.synchronize()
    monkeypatch.delenv(FAULT_ENV)
    k(out, x, off, 3)
    be.synchronize()
