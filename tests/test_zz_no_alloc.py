"""GPU test of the no-alloc jagged getitem entry point.

``awkward_ListArray64_getitem_jagged_apply_64_noalloc`` is for callers that
may not allocate device memory while they run, such as awkward code embedded
in a process whose GPU memory belongs to another framework's pooling
allocator: there cudaMalloc fails or goes around the pool.  It keeps its
look-back tile states in a fixed device array inside the library instead of
taking them from the library's memory pool.

The test calls it through the C ABI (ctypes, raw device pointers) and checks
that its outputs equal those of the pool-based entry point
``awkward_ListArray64_getitem_jagged_apply_64`` on the same inputs, bit for bit
(integer offsets and carries), on two calls in a row: the second call is
smaller than the first, so tile states left in the shared array by the first
call would corrupt its offsets if the entry point did not clear them.  A call
above the stated maximum must be refused without launching anything.

The file name puts it last in collection order; it needs no state from other
tests and also passes alone in a fresh process.
"""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NAME = "awkward_ListArray64_getitem_jagged_apply_64_noalloc"
POOLED = "awkward_ListArray64_getitem_jagged_apply_64"
MAX_LISTS = 1 << 26  # AWKWARD_GB300_NOALLOC_MAX_LISTS in include/awkward_gb300.h
CUDA_ERROR_INVALID_VALUE = 1
NO_ERROR = 0xFFFFFFFFFFFFFFFF


def _noalloc_fn():
    from awkward_gb300 import _abi

    f = getattr(_abi.load_library(), NAME)
    f.argtypes = [ctypes.c_void_p] * 4 + [ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64,
                                          ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
                                          ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p]
    f.restype = ctypes.c_int
    return f


def _case(n, seed):
    rng = np.random.default_rng(seed)
    L = rng.poisson(8, n)
    L[rng.random(n) < 0.05] = 0
    off = np.concatenate([[0], np.cumsum(L)]).astype(np.int64)
    K = np.where(L > 0, rng.poisson(3, n), 0)
    soff = np.concatenate([[0], np.cumsum(K)]).astype(np.int64)
    idx = np.concatenate([rng.integers(-l, l, k) for l, k in zip(L, K) if k] or
                         [np.zeros(0, np.int64)]).astype(np.int64)
    return off, soff, idx


def _run(fn, off, soff, idx):
    """One call with fresh outputs; returns (return code, error word, offsets, carry)."""
    import torch

    n = len(off) - 1
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    d_off, d_soff, d_idx = dev(off), dev(soff), dev(idx)
    starts, stops = d_off[:-1].contiguous(), d_off[1:].contiguous()
    sstarts, sstops = d_soff[:-1].contiguous(), d_soff[1:].contiguous()
    to_off = torch.full((n + 1,), -7, dtype=torch.int64, device="cuda")
    to_carry = torch.full((max(len(idx), 1),), -7, dtype=torch.int64, device="cuda")
    err = torch.full((1,), -1, dtype=torch.int64, device="cuda")  # all bits set: no error
    stream = torch.cuda.current_stream().cuda_stream
    rc = fn(to_off.data_ptr(), to_carry.data_ptr(), sstarts.data_ptr(), sstops.data_ptr(), n,
            d_idx.data_ptr(), len(idx), starts.data_ptr(), stops.data_ptr(), int(off[-1]),
            0, err.data_ptr(), stream)
    torch.cuda.synchronize()
    return (rc, int(err.cpu().numpy().view(np.uint64)[0]), to_off.cpu().numpy(),
            to_carry.cpu().numpy()[: len(idx)])


def test_noalloc_matches_pooled_entry_point_on_two_calls_in_a_row():
    import torch

    from awkward_gb300 import _abi

    assert torch.cuda.is_available()
    noalloc, pooled = _noalloc_fn(), _abi.cfunc(POOLED)
    # 40,000 lists span 40 tiles of 1024 lists; the second call spans only 3,
    # so the first call's tile states must have been cleared
    for n, seed in ((40_000, 11), (2_500, 12)):
        off, soff, idx = _case(n, seed)
        rc_a, err_a, off_a, carry_a = _run(noalloc, off, soff, idx)
        rc_b, err_b, off_b, carry_b = _run(pooled, off, soff, idx)
        assert rc_a == 0 and rc_b == 0, (rc_a, rc_b)
        assert err_a == NO_ERROR and err_b == NO_ERROR, (hex(err_a), hex(err_b))
        np.testing.assert_array_equal(off_a, off_b)
        np.testing.assert_array_equal(carry_a, carry_b)
        assert off_a[-1] == len(idx)


def test_noalloc_refuses_sizes_above_its_maximum():
    fn = _noalloc_fn()
    # refused on the host before any pointer is touched or anything launched
    rc = fn(None, None, None, None, MAX_LISTS + 1, None, 0, None, None, 0, 0, None, None)
    assert rc == CUDA_ERROR_INVALID_VALUE
