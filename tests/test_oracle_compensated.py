"""Pins of the FP64 compensated-sum oracle that float sums are judged against.

* Against math.fsum (Shewchuk's exactly rounded sum) on lists with wide
  magnitude ranges and heavy cancellation: the double-double result must be
  within u*|S| + 2*n*u^2*sum|x| of it (u = 2^-53).
* Against awkward-cpp's own left-to-right sums (the committed random golden
  cases of awkward_reduce_sum_float64_float64_64 and the unit vectors): their
  difference must stay within the sequential sum's error bound
  (n-1)*u*sum|x| (awkward-cpp/src/cpu-kernels/awkward_reduce_sum.cpp:17-23).
* Lists with an infinity or a NaN give the plain IEEE sum.
* The error report flags a result planted outside the 4*n*eps*sum|x| bound.
"""

import math

import numpy as np

import golden_cases as gc
import oracle

U = 2.0 ** -53


def _lists(rng, nlists=3000):
    L = rng.poisson(12, nlists)
    L[rng.random(nlists) < 0.05] = 0
    L[::97] = rng.integers(200, 3000, len(L[::97]))
    off = np.concatenate([[0], np.cumsum(L)]).astype(np.int64)
    E = int(off[-1])
    x = rng.standard_normal(E) * np.exp2(rng.integers(-60, 60, E))
    # cancellation: some lists get a huge pair that cancels exactly
    for b in range(0, nlists, 13):
        if L[b] >= 2:
            big = 2.0 ** 70 * (1 + rng.random())
            x[off[b]] = big
            x[off[b + 1] - 1] = -big
    return off, x


def test_compensated_sum_matches_fsum():
    rng = np.random.default_rng(21)
    off, x = _lists(rng)
    comp, absum = oracle.compensated_sum(x, off, nthreads=4)
    for b in range(len(off) - 1):
        seg = x[off[b]:off[b + 1]]
        exact = math.fsum(seg)
        n = len(seg)
        bound = U * abs(exact) + 2 * n * U * U * absum[b] + 1e-300
        assert abs(comp[b] - exact) <= bound, (b, comp[b], exact)
        assert absum[b] == np.sum(np.abs(seg)) or abs(absum[b] - np.sum(np.abs(seg))) <= n * U * absum[b]


def test_compensated_sum_float32_content():
    rng = np.random.default_rng(22)
    L = rng.poisson(20, 500)
    off = np.concatenate([[0], np.cumsum(L)]).astype(np.int64)
    x = (rng.standard_normal(int(off[-1])) * 1e3).astype(np.float32)
    comp, _ = oracle.compensated_sum(x, off)
    for b in range(len(L)):
        exact = math.fsum(x[off[b]:off[b + 1]].astype(np.float64))
        assert abs(comp[b] - exact) <= U * abs(exact) + 1e-300


def _sequential_cases():
    """(x, offsets, awkward-cpp's sums) of every float64 sum golden case."""
    name = "awkward_reduce_sum_float64_float64_64"
    out = []
    for nm, i in gc.random_case_ids():
        if nm == name:
            _n, kw, exp, err = gc.random_case(i)
            if err is None:
                out.append((kw["fromptr"], kw["offsets"], exp["toptr"]))
    for nm, i in gc.unit_case_ids():
        if nm == name:
            kw, exp, msg = gc.unit_case(nm, i)
            if msg is None and len(exp["toptr"]):
                m = len(exp["toptr"])
                out.append((kw["fromptr"], kw["offsets"][: m + 1], exp["toptr"]))
    return out


def test_compensated_sum_against_awkward_cpp_sequential_sums():
    cases = _sequential_cases()
    assert cases, "no float64 sum golden cases"
    for x, off, seq in cases:
        comp, absum = oracle.compensated_sum(np.asarray(x, np.float64), off)
        n = np.diff(off).astype(np.float64)
        fin = np.isfinite(seq) & np.isfinite(absum)
        with np.errstate(invalid="ignore"):
            bound = np.maximum(n - 1, 0) * U * absum * (1 + 1e-12) + 1e-300
        assert np.all(np.abs(seq[fin] - comp[fin]) <= bound[fin])
        np.testing.assert_array_equal(np.isnan(seq), np.isnan(comp))


def test_compensated_sum_nonfinite_and_empty():
    x = np.array([1.0, np.inf, 2.0, -np.inf, np.inf, np.nan, 3.0, 5.0])
    off = np.array([0, 3, 5, 6, 6, 8], np.int64)
    comp, _ = oracle.compensated_sum(x, off)
    assert comp[0] == np.inf and np.isnan(comp[1]) and np.isnan(comp[2])
    assert comp[3] == 0.0 and comp[4] == 8.0


def test_error_report_flags_a_result_outside_the_bound():
    rng = np.random.default_rng(23)
    off, x = _lists(rng, 400)
    comp, absum = oracle.compensated_sum(x, off)
    rep = oracle.sum_error_report(comp, x, off)
    assert rep["within"] and rep["nonfinite_ok"] and rep["max_ratio"] == 0.0
    bad = comp.copy()
    n = np.diff(off)
    k = int(np.argmax(n))
    bad[k] += 10 * n[k] * np.finfo(np.float64).eps * absum[k]
    rep = oracle.sum_error_report(bad, x, off)
    assert not rep["within"] and rep["worst_list"] == k
