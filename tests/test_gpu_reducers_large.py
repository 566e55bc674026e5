"""GPU parity of the segmented reducers on adversarial length distributions.

The golden fixtures only hold lists of up to ~1000 elements; these cases
exercise every path of the reduction kernel against the C oracle: lists
reduced by one lane (<= 32 elements), by a warp (33..4096), lists longer than
4096 that cross warp ranges (partial records + fix-up), empty lists, a single
giant list, and offsets that do not start at 0.  Values include NaN at list
starts and inside lists, signed zeros and infinities.

Integer, index, count, boolean and max/min outputs must be bit-identical;
float sums within 4*n*eps*sum|x| of the FP64 compensated-sum oracle (n = list
length); the error figures of every float-sum case are printed.
"""

import zlib

import numpy as np
import pytest

import oracle
from gpu_util import run_gpu

pytestmark = pytest.mark.gpu


def _lengths(kind, rng):
    if kind == "poisson":
        L = rng.poisson(8, 20000)
        L[rng.random(len(L)) < 0.01] = 0
        return L
    if kind == "thresholds":
        return np.array([0, 1, 31, 32, 33, 0, 4095, 4096, 4097, 2, 8191, 0, 65, 64, 63] * 3)
    if kind == "heavy":
        L = rng.poisson(6, 5000)
        L[::997] = rng.integers(5000, 300000, len(L[::997]))
        L[rng.random(len(L)) < 0.05] = 0
        return L
    if kind == "one_giant":
        return np.array([1_500_000])
    if kind == "giant_between_empty":
        return np.array([0] * 300 + [700_000] + [0] * 300 + [3] + [0] * 50)
    if kind == "all_empty":
        return np.zeros(5000, np.int64)
    raise KeyError(kind)


KINDS = ["poisson", "thresholds", "heavy", "one_giant", "giant_between_empty", "all_empty"]


def _data(kind, dtype, seed=0, base=0):
    rng = np.random.default_rng(seed)
    L = _lengths(kind, rng).astype(np.int64)
    off = (np.concatenate([[0], np.cumsum(L)]) + base).astype(np.int64)
    E = int(off[-1])
    if np.dtype(dtype).kind == "f":
        x = rng.standard_normal(E).astype(dtype)
        if E:
            starts = off[:-1][L > 0]
            pick = starts[rng.random(len(starts)) < 0.02]
            x[pick] = np.nan  # leading NaNs (argmax/argmin rule)
            x[rng.integers(0, E, max(E // 500, 1))] = np.nan
            x[rng.integers(0, E, max(E // 300, 1))] = 0.0
            x[rng.integers(0, E, max(E // 300, 1))] = -0.0
            x[rng.integers(0, E, max(E // 2000, 1))] = np.inf
            x[rng.integers(0, E, max(E // 2000, 1))] = -np.inf
    elif dtype == np.bool_:
        x = rng.random(E) < 0.3
    else:
        info = np.iinfo(dtype)
        x = rng.integers(max(info.min, -1000), min(info.max, 1000), E).astype(dtype)
    return off, x, len(L)


CASES = [
    ("awkward_reduce_sum_float64_float64_64", np.float64, np.float64, {}),
    ("awkward_reduce_max_float64_float64_64", np.float64, np.float64, {"identity": -np.inf}),
    ("awkward_reduce_min_float64_float64_64", np.float64, np.float64, {"identity": np.inf}),
    ("awkward_reduce_argmax_float64_64", np.int64, np.float64, {"starts": True}),
    ("awkward_reduce_argmin_float64_64", np.int64, np.float64, {"starts": True}),
    ("awkward_reduce_max_float32_float32_64", np.float32, np.float32, {"identity": -np.inf}),
    ("awkward_reduce_argmax_float32_64", np.int64, np.float32, {"starts": True}),
    ("awkward_reduce_sum_float64_float32_64", np.float64, np.float32, {}),
    ("awkward_reduce_sum_int64_int64_64", np.int64, np.int64, {}),
    ("awkward_reduce_max_int64_int64_64", np.int64, np.int64, {"identity": np.iinfo(np.int64).min}),
    ("awkward_reduce_argmin_int32_64", np.int64, np.int32, {"starts": True}),
    ("awkward_reduce_countnonzero_float64_64", np.int64, np.float64, {}),
    ("awkward_reduce_prod_bool_bool_64", np.bool_, np.bool_, {}),
    ("awkward_reduce_sum_bool_int8_64", np.bool_, np.int8, {}),
]


@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("name,out_dt,in_dt,extra", CASES, ids=[c[0] for c in CASES])
def test_reducer_distributions(kind, name, out_dt, in_dt, extra):
    base = 5 if kind == "thresholds" else 0  # offsets need not start at 0
    off, x, n = _data(kind, in_dt, seed=zlib.crc32(f"{kind}:{name}".encode()) % 1000, base=base)
    if base:
        x = np.concatenate([np.zeros(base, x.dtype), x])
    kw = {"toptr": np.zeros(n, out_dt), "fromptr": x, "offsets": off, "outlength": n}
    if extra.get("starts"):
        kw["starts"] = off[:-1].copy()
    if "identity" in extra:
        kw["identity"] = extra["identity"]
    exp = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in kw.items()}
    assert oracle.call(oracle.load(), name, **exp)[0] is None
    got, err = run_gpu(name, kw)
    assert err is None, err
    g, e = got["toptr"], exp["toptr"]
    if "sum_float64" in name:
        rep = oracle.sum_error_report(g, x, off)
        print(f"sum_err {name} {kind}: {rep}")
        assert rep["nonfinite_ok"] and rep["within"], rep
    elif g.dtype.kind == "f":
        gn, en = np.isnan(g), np.isnan(e)
        np.testing.assert_array_equal(gn, en)
        gi = g.view(np.int64 if g.dtype == np.float64 else np.int32)
        ei = e.view(np.int64 if e.dtype == np.float64 else np.int32)
        np.testing.assert_array_equal(gi[~en], ei[~en])  # bitwise: signed zeros
    else:
        np.testing.assert_array_equal(g, e)
