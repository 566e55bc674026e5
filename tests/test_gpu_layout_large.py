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
