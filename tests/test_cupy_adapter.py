"""CPU test of the cupy adapter with fake cupy arrays and a recording C function.

Checks what awkward's CupyKernel relies on (src/awkward/_kernels.py:185-232):
one entry per (family, *dtypes) key, the ``.dir`` / ``.is_ptr`` attributes,
the ``f(grid, block, args)`` call shape with (invocation_index, err_code)
appended, device addresses read from ``.data.ptr``, scalars passed through,
the current stream forwarded, and error messages registered per family in
code order.
"""

import numpy as np
import pytest

from awkward_gb300 import cupy_adapter
from awkward_gb300._signatures import SIGNATURES
from awkward_gb300.kernel_table import kernel_key


class FakeMem:
    def __init__(self, ptr):
        self.ptr = ptr


class FakeArray:
    def __init__(self, ptr):
        self.data = FakeMem(ptr)


def _install():
    calls = []

    def cfunc(name):
        def f(*args):
            calls.append((name, args))
            return 0
        return f

    table, errors = {}, {}
    keys = cupy_adapter.install(table, errors, cfunc=cfunc, current_stream_ptr=lambda: 0xABC)
    return table, errors, keys, calls


def test_every_specialization_is_installed_under_awkwards_key():
    table, errors, keys, _ = _install()
    assert len(table) == len(SIGNATURES) == len(keys)
    k = ("awkward_reduce_argmax", np.int64, np.float64, np.int64, np.int64)
    assert table[k].name == "awkward_reduce_argmax_float64_64"
    assert table[k].is_ptr == [True, True, True, True, False]
    assert table[k].dir == ["out", "in", "in", "in", "in"]
    assert errors["awkward_ListArray_getitem_jagged_apply"][4] == "index out of range"
    assert "bounded wait" in errors["awkward_reduce_sum"][32]


def test_call_marshals_pointers_scalars_and_stream():
    table, _, _, calls = _install()
    f = table[kernel_key("awkward_reduce_max_float64_float64_64")]
    err = FakeArray(0x5000)
    f((1, 1, 1), (1, 1, 1), (FakeArray(0x1000), FakeArray(0x2000), FakeArray(0x3000),
                             np.int64(7), np.float64(-np.inf), 3, err))
    name, args = calls[-1]
    assert name == "awkward_reduce_max_float64_float64_64"
    assert args == (0x1000, 0x2000, 0x3000, 7, -np.inf, 3, 0x5000, 0xABC)


def test_list_of_lists_argument_is_the_device_pointer_array():
    table, _, _, calls = _install()
    f = table[kernel_key("awkward_ListArray64_combinations_64")]
    tocarryraw = FakeArray(0x9000)  # awkward's device array of row pointers
    f(None, None, (tocarryraw, FakeArray(1), FakeArray(2), 2, False, FakeArray(3),
                   FakeArray(4), 10, 0, FakeArray(5)))
    assert calls[-1][1][0] == 0x9000


def test_launch_failure_raises():
    table = cupy_adapter.adapted_kernels(cfunc=lambda n: (lambda *a: 2),
                                         current_stream_ptr=lambda: 0)
    f = table[kernel_key("awkward_reduce_count_64")]
    with pytest.raises(cupy_adapter.CudaLaunchError):
        f(None, None, (FakeArray(1), FakeArray(2), 5, 0, FakeArray(3)))
