"""GPU parity of the complex reducers beyond the golden fixtures.

Against the C oracle (the CPU loops, compiled without fused multiply-adds) on
lists of every length class of the segmented reducer -- short (one lane),
33-256 (8-lane groups), longer (whole warp) and giant lists that cross warp
ranges (head/tail records and the fix-up) -- with heavy ties in both parts,
signed zeros, infinities, NaN in either part and lists whose first element has
a NaN real part (the CPU keeps that element).  max/min/argmax/argmin, the
nonzero counts and the product (computed in the CPU's order) are bit-exact;
the sums are within 4*n*eps*sum|part| per component.
"""

import numpy as np
import pytest

import oracle
from test_gpu_nonlocal_large import _gpu

pytestmark = pytest.mark.gpu


def _data(seed, dt, nan_rate):
    rng = np.random.default_rng(seed)
    L = np.minimum(rng.poisson(8, 200_000), 40)
    L[rng.random(len(L)) < 0.02] = 0
    L[::997] = rng.integers(33, 3000, len(L[::997]))
    L[12_345] = 1_500_000  # crosses warp ranges
    L[54_321] = 9_000
    off = np.concatenate([[0], np.cumsum(L)]).astype(np.int64)
    E = int(off[-1])
    v = np.round(rng.standard_normal((E, 2)), 1).astype(dt)
    k = rng.random((E, 2))
    v[k < nan_rate] = np.nan
    v[(k >= 0.4) & (k < 0.43)] = -0.0
    v[(k >= 0.43) & (k < 0.44)] = np.inf
    v[(k >= 0.44) & (k < 0.45)] = -np.inf
    first = off[:-1][(L > 0) & (rng.random(len(L)) < 0.05 if nan_rate else np.zeros(len(L), bool))]
    v[first, 0] = np.nan
    return off, v.reshape(-1), len(L)


def _run(name, kw):
    exp = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in kw.items()}
    oracle.call(oracle.load(), name, **exp)
    return _gpu(name, kw)["toptr"], exp["toptr"]


def _bits_equal(got, exp):
    gn, en = np.isnan(got), np.isnan(exp)
    np.testing.assert_array_equal(gn, en)
    w = np.uint32 if exp.dtype == np.float32 else np.uint64
    np.testing.assert_array_equal(got.view(w)[~en], exp.view(w)[~en])


@pytest.mark.parametrize("tag,dt", [("complex64", np.float32), ("complex128", np.float64)])
@pytest.mark.parametrize("nan_rate", [0.0, 0.05, 0.3])
def test_complex_extrema_and_counts(tag, dt, nan_rate):
    off, x, n = _data(7 + int(nan_rate * 100), dt, nan_rate)
    for fam in ("max", "min"):
        kw = {"toptr": np.full(2 * n, 123, dt), "fromptr": x, "offsets": off, "outlength": n,
              "identity": float(-np.inf if fam == "max" else np.inf)}
        got, exp = _run(f"awkward_reduce_{fam}_{tag}_{tag}_64", kw)
        _bits_equal(got, exp)
    for fam in ("argmax", "argmin"):
        kw = {"toptr": np.full(n, 123, np.int64), "fromptr": x, "offsets": off, "outlength": n}
        got, exp = _run(f"awkward_reduce_{fam}_{tag}_64", kw)
        np.testing.assert_array_equal(got, exp)
    got, exp = _run(f"awkward_reduce_countnonzero_{tag}_64",
                    {"toptr": np.full(n, 123, np.int64), "fromptr": x, "offsets": off,
                     "outlength": n})
    np.testing.assert_array_equal(got, exp)
    for fam in ("sum_bool", "prod_bool"):
        got, exp = _run(f"awkward_reduce_{fam}_{tag}_64",
                        {"toptr": np.zeros(n, np.bool_), "fromptr": x, "offsets": off,
                         "outlength": n})
        np.testing.assert_array_equal(got, exp)


@pytest.mark.parametrize("tag,dt", [("complex64", np.float32), ("complex128", np.float64)])
def test_complex_sum_and_prod(tag, dt):
    off, x, n = _data(3, dt, 0.0)
    kw = {"toptr": np.full(2 * n, 123, dt), "fromptr": x, "offsets": off, "outlength": n}
    got, exp = _run(f"awkward_reduce_sum_{tag}_{tag}_64", kw)
    eps = np.finfo(dt).eps
    L = np.diff(off).astype(np.float64)
    parts = np.abs(x.astype(np.float64).reshape(-1, 2))
    for c in range(2):
        g, e = got.reshape(-1, 2)[:, c].astype(np.float64), exp.reshape(-1, 2)[:, c].astype(np.float64)
        t = np.where(np.isfinite(parts[:, c]), parts[:, c], 0.0)
        cs = np.concatenate([[0.0], np.cumsum(t)])
        bound = 4 * np.maximum(L, 1) * eps * (cs[off[1:]] - cs[off[:-1]])
        fin = np.isfinite(e)
        np.testing.assert_array_equal(np.isnan(g), np.isnan(e))
        np.testing.assert_array_equal(g[~fin & ~np.isnan(e)], e[~fin & ~np.isnan(e)])
        assert np.all(np.abs(g[fin] - e[fin]) <= bound[fin])
    # the product: short lists only (long products over/underflow to 0/inf/NaN either way)
    Ls = np.minimum(np.diff(off), 12)
    offs = np.concatenate([[0], np.cumsum(Ls)]).astype(np.int64)
    xs = (1.0 + 0.05 * np.random.default_rng(4).standard_normal(2 * int(offs[-1]))).astype(dt)
    kw = {"toptr": np.full(2 * n, 123, dt), "fromptr": xs, "offsets": offs, "outlength": n}
    got, exp = _run(f"awkward_reduce_prod_{tag}_{tag}_64", kw)
    _bits_equal(got, exp)
