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
call would corrupt its offsets if the entry point did not clear them.  The
same outputs are checked against the CPU oracle (the C restatement of
awkward-cpp's kernel), an index out of range must raise awkward's error
through the same error word as the pooled entry point, and a call above the
stated maximum must be refused without launching anything.

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


def _oracle(off, soff, idx):
    import oracle

    n = len(off) - 1
    to_off = np.zeros(n + 1, np.int64)
    to_carry = np.zeros(max(len(idx), 1), np.int64)
    msg, _ident, _att = oracle.call(
        oracle.load(), POOLED, tooffsets=to_off, tocarry=to_carry,
        slicestarts=np.ascontiguousarray(soff[:-1]), slicestops=np.ascontiguousarray(soff[1:]),
        sliceouterlen=n, sliceindex=np.ascontiguousarray(idx), sliceinnerlen=len(idx),
        fromstarts=np.ascontiguousarray(off[:-1]), fromstops=np.ascontiguousarray(off[1:]),
        contentlen=int(off[-1]))
    return msg, to_off, to_carry[: len(idx)]


def test_noalloc_matches_the_oracle():
    fn = _noalloc_fn()
    off, soff, idx = _case(30_000, 13)
    rc, err, got_off, got_carry = _run(fn, off, soff, idx)
    msg, exp_off, exp_carry = _oracle(off, soff, idx)
    assert rc == 0 and err == NO_ERROR and msg is None
    np.testing.assert_array_equal(got_off, exp_off)
    np.testing.assert_array_equal(got_carry, exp_carry)


def test_noalloc_reports_an_index_out_of_range_like_the_pooled_entry_point():
    from awkward_gb300 import _abi

    off, soff, idx = _case(5_000, 14)
    idx = idx.copy()
    # one index past its list's length (the list owning slice position 7)
    owner = np.searchsorted(soff, 7, side="right") - 1
    idx[7] = off[owner + 1] - off[owner]
    rc_a, err_a, _, _ = _run(_noalloc_fn(), off, soff, idx)
    rc_b, err_b, _, _ = _run(_abi.cfunc(POOLED), off, soff, idx)
    msg, _, _ = _oracle(off, soff, idx)
    assert rc_a == 0 and rc_b == 0
    assert msg is not None and "index out of range" in msg
    # invocation index 0, message 4 of awkward's jagged_apply kernel
    assert err_a == err_b == 4, (hex(err_a), hex(err_b))
