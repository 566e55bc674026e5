"""GPU parity of compact_offsets and the RegularArray carries beyond the golden fixtures.

Bit-exact against the C oracle at sizes spanning many list tiles (scan
look-back across tiles) and many thread chunks (carry rows wrapping inside a
thread's outputs), for every offset type, and the error of a list with
stops < starts.
"""

import numpy as np
import pytest

import oracle
from test_gpu_nonlocal_large import S, _check, _gpu

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("tag,C", [("32", np.int32), ("U32", np.uint32), ("64", np.int64)])
def test_compact_offsets(tag, C):
    rng = np.random.default_rng(12)
    n = 3_000_000
    L = rng.poisson(7, n)
    starts = rng.integers(0, 1 << 20, n)
    kw = {"tooffsets": np.full(n + 1, S, np.int64), "fromstarts": starts.astype(C),
          "fromstops": (starts + L).astype(C), "length": n}
    _check(f"awkward_ListArray{tag}_compact_offsets_64", kw, ["tooffsets"])


def test_compact_offsets_error():
    rng = np.random.default_rng(13)
    n = 500_000
    starts = rng.integers(10, 1000, n)
    stops = starts + rng.poisson(3, n)
    stops[400_123] = starts[400_123] - 1
    kw = {"tooffsets": np.full(n + 1, S, np.int64), "fromstarts": starts, "fromstops": stops,
          "length": n}
    exp = oracle.call(oracle.load(), "awkward_ListArray64_compact_offsets_64",
                      **{k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in kw.items()})
    assert exp[0] == "stops[i] < starts[i]"
    with pytest.raises(ValueError, match=r"stops\[i\] < starts\[i\]"):
        _gpu("awkward_ListArray64_compact_offsets_64", kw)


@pytest.mark.parametrize("size", [1, 3, 8, 17])
def test_regular_carry_and_localindex(size):
    rng = np.random.default_rng(size)
    lencarry = 2_000_003
    kw = {"tocarry": np.full(lencarry * size, S, np.int64),
          "fromcarry": rng.integers(0, 1 << 30, lencarry).astype(np.int64),
          "lencarry": lencarry, "size": size}
    _check("awkward_RegularArray_getitem_carry_64", kw, ["tocarry"])
    _check("awkward_RegularArray_localindex_64",
           {"toindex": np.full(lencarry * size, S, np.int64), "size": size, "length": lencarry},
           ["toindex"])


@pytest.mark.parametrize("tag,C", [("32", np.int32), ("U32", np.uint32), ("64", np.int64)])
def test_range_counts_and_spread(tag, C):
    rng = np.random.default_rng(14)
    n = 2_000_000
    L = rng.poisson(4, n)
    L[777] = 50_000
    off = np.concatenate([[0], np.cumsum(L)]).astype(C)
    _check(f"awkward_ListArray{tag}_getitem_next_range_counts_64",
           {"total": np.full(1, S, np.int64), "fromoffsets": off, "lenstarts": n}, ["total"])
    _check(f"awkward_ListArray{tag}_getitem_next_range_spreadadvanced_64",
           {"toadvanced": np.full(int(off[-1]), S, np.int64),
            "fromadvanced": rng.integers(0, 1 << 40, n).astype(np.int64), "fromoffsets": off,
            "lenstarts": n}, ["toadvanced"])


def test_missing_jagged_helpers_and_shifts():
    rng = np.random.default_rng(15)
    n = 3_000_000
    idx = np.where(rng.random(n) < 0.3, -1, np.arange(n)).astype(np.int64)
    valid = int((idx >= 0).sum())
    offs = np.concatenate([[0], np.cumsum(rng.poisson(3, valid))]).astype(np.int64)
    _check("awkward_Content_getitem_next_missing_jagged_getmaskstartstop",
           {"index_in": idx, "offsets_in": offs, "mask_out": np.full(n, S, np.int64),
            "starts_out": np.full(n, S, np.int64), "stops_out": np.full(n, S, np.int64),
            "length": n}, ["mask_out", "starts_out", "stops_out"])
    for tag, T in (("32", np.int32), ("U32", np.uint32), ("64", np.int64)):
        ix = rng.integers(0, 1000, n)
        if T != np.uint32:
            ix[rng.random(n) < 0.4] = -1
        st = rng.integers(0, 1 << 40, n).astype(np.int64)
        _check(f"awkward_MaskedArray{tag}_getitem_next_jagged_project",
               {"index": ix.astype(T), "starts_in": st, "stops_in": st + 3,
                "starts_out": np.full(n, S, np.int64), "stops_out": np.full(n, S, np.int64),
                "length": n}, ["starts_out", "stops_out"])
    starts = np.sort(rng.integers(0, 1 << 30, n)).astype(np.int64)
    toptr = np.where(rng.random(n) < 0.2, -1, rng.integers(0, n, n)).astype(np.int64)
    _check("awkward_NumpyArray_reduce_adjust_starts_shifts_64",
           {"toptr": toptr, "outlength": n, "offsets": np.zeros(n + 1, np.int64),
            "starts": starts, "shifts": rng.integers(0, 9, n).astype(np.int64)}, ["toptr"])
    _check("awkward_localindex_64", {"toindex": np.full(n, S, np.int64), "length": n}, ["toindex"])
    _check("awkward_RegularArray_getitem_next_range_spreadadvanced_64",
           {"toadvanced": np.full(n * 3, S, np.int64),
            "fromadvanced": rng.integers(0, 1 << 40, n).astype(np.int64), "length": n,
            "nextsize": 3}, ["toadvanced"])
