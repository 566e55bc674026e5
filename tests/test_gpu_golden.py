"""GPU parity: every entry point against awkward's golden vectors and awkward-cpp's outputs.

Integer, index, boolean, count, offsets, carry and combinations outputs and
max/min values must be bit-identical.  Float sums (awkward_reduce_sum with a
float output) must be within 4*n*eps*sum|x| of the FP64 compensated-sum
oracle, per list (n = list length, eps of the output type).  The other
order-dependent floating-point reductions (prod, sum of squares/powers,
centered sum of squares) must be within 4*n*eps*sum|term| of awkward-cpp's
left-to-right result.  Non-finite results must match exactly.
"""

import math

import numpy as np
import pytest

import golden_cases as gc
from gpu_util import run_gpu

pytestmark = pytest.mark.gpu

UNIT = gc.unit_case_ids()
RANDOM = gc.random_case_ids()


def _terms(name, kw):
    """|term| per element as the reducer sees it (float64), for the error bound."""
    from awkward_gb300._signatures import SIGNATURES

    fam = SIGNATURES[name]["family"]
    x = np.asarray(kw["fromptr"]).astype(np.float64)
    if fam in ("awkward_reduce_sum",):
        return np.abs(x)
    if fam == "awkward_reduce_sumofsquares":
        return x * x
    if fam == "awkward_reduce_centered_sumofsquares":
        off = np.asarray(kw["offsets"])
        parents = np.repeat(np.arange(len(off) - 1), np.diff(off))
        d = x[off[0]:off[-1]] - np.asarray(kw["means"])[parents]
        out = np.zeros_like(x)
        out[off[0]:off[-1]] = d * d
        return out
    if fam == "awkward_reduce_sumofpowers":
        with np.errstate(all="ignore"):
            return np.abs(np.power(x, float(kw["n"])))
    return np.abs(x)


def check_float_sum_like(name, kw, got, exp):
    from awkward_gb300._signatures import SIGNATURES

    fam = SIGNATURES[name]["family"]
    out_t = SIGNATURES[name]["args"][0][1]
    eps = np.finfo(np.float32 if out_t == "float" else np.float64).eps
    off = np.asarray(kw["offsets"])
    got = np.asarray(got)[: len(exp)].astype(np.float64)
    exp = np.asarray(exp).astype(np.float64)
    finite = np.isfinite(exp)
    np.testing.assert_array_equal(np.isnan(got), np.isnan(exp))
    np.testing.assert_array_equal(got[np.isinf(exp)], exp[np.isinf(exp)])
    if fam == "awkward_reduce_prod":
        n = np.diff(off).astype(np.float64)[: len(exp)]
        tiny = np.finfo(np.float32 if out_t == "float" else np.float64).tiny
        bound = 4 * np.maximum(n, 1) * eps * np.abs(exp) + 64 * tiny
    elif fam == "awkward_reduce_sum":
        import oracle

        x = np.asarray(kw["fromptr"])
        x = x if x.dtype in (np.float32, np.float64) else x.astype(np.float64)
        m = len(exp)
        rep = oracle.sum_error_report(got, x, off[: m + 1], eps=float(eps))
        assert rep["nonfinite_ok"] and rep["within"], (name, rep)
        return
    else:
        with np.errstate(all="ignore"):
            t = _terms(name, kw)
            t = np.where(np.isfinite(t), t, 0.0)  # lists with non-finite terms are checked above
            cs = np.concatenate([[0.0], np.cumsum(t)])
            scale = cs[off[1:]] - cs[off[:-1]]
        n = np.diff(off).astype(np.float64)
        bound = (4 * np.maximum(n, 1) * eps * scale)[: len(exp)]
    err = np.abs(got - exp)
    bad = finite & ~(err <= bound)
    assert not bad.any(), (name, np.nonzero(bad)[0][:5], got[bad][:5], exp[bad][:5], bound[bad][:5])


def check_complex_sum(name, kw, got, exp):
    """Per list and component: within 4*n*eps*sum|part| of awkward-cpp's sum."""
    from awkward_gb300._signatures import SIGNATURES

    eps = np.finfo(np.float32 if SIGNATURES[name]["args"][0][1] == "float" else np.float64).eps
    off = np.asarray(kw["offsets"])
    n = np.diff(off).astype(np.float64)
    x = np.asarray(kw["fromptr"]).astype(np.float64).reshape(-1, 2)
    m = min(len(n), len(exp) // 2)  # unit cases may list fewer outputs than lists
    got = np.asarray(got)[: 2 * m].astype(np.float64).reshape(-1, 2)
    exp = np.asarray(exp)[: 2 * m].astype(np.float64).reshape(-1, 2)
    n, off = n[:m], off[: m + 1]
    for c in range(2):
        g, e = got[:, c], exp[:, c]
        np.testing.assert_array_equal(np.isnan(g), np.isnan(e))
        np.testing.assert_array_equal(g[np.isinf(e)], e[np.isinf(e)])
        t = np.abs(x[:, c])
        t = np.where(np.isfinite(t), t, 0.0)
        cs = np.concatenate([[0.0], np.cumsum(t)])
        bound = 4 * np.maximum(n, 1) * eps * (cs[off[1:]] - cs[off[:-1]])
        fin = np.isfinite(e)
        with np.errstate(invalid="ignore"):
            bad = fin & ~(np.abs(g - e) <= bound)
        assert not bad.any(), (name, c, np.nonzero(bad)[0][:5])


def check(name, kw, outs, expected):
    if gc.is_complex_sum(name):
        check_complex_sum(name, kw, outs["toptr"], expected["toptr"])
    elif gc.is_float_sum_like(name):
        check_float_sum_like(name, kw, outs["toptr"], expected["toptr"])
    else:
        gc.assert_outputs_equal(name, outs, expected, exact=True)


@pytest.mark.parametrize("name,index", UNIT, ids=[f"{n}-{i}" for n, i in UNIT])
def test_gpu_kernel_test_data(name, index):
    kw, expected, message = gc.unit_case(name, index)
    outs, err = run_gpu(name, kw)
    if message is not None:
        assert err is not None and err.startswith(message), (err, message)
        return
    assert err is None, err
    check(name, kw, outs, expected)


@pytest.mark.parametrize("name,index", RANDOM, ids=[f"{n}-{i}" for n, i in RANDOM])
def test_gpu_matches_awkward_cpp(name, index):
    _name, kw, expected, error = gc.random_case(index)
    outs, err = run_gpu(name, kw)
    if error is not None:
        assert err is not None and err.startswith(error), (err, error)
        return
    assert err is None, err
    check(name, kw, outs, expected)
