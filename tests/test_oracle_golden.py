"""The C oracle against awkward's golden vectors and awkward-cpp's own kernels (CPU only)."""

import numpy as np
import pytest

import golden_cases as gc
import oracle

UNIT = gc.unit_case_ids()
RANDOM = gc.random_case_ids()


@pytest.mark.parametrize("name,index", UNIT, ids=[f"{n}-{i}" for n, i in UNIT])
def test_oracle_kernel_test_data(name, index):
    kw, expected, message = gc.unit_case(name, index)
    msg, _identity, _attempt = oracle.call(oracle.load(), name, **kw)
    if message is not None:
        assert msg == message
        return
    assert msg is None, msg
    gc.assert_outputs_equal(name, kw, expected, exact=True)


@pytest.mark.parametrize("name,index", RANDOM, ids=[f"{n}-{i}" for n, i in RANDOM])
def test_oracle_matches_awkward_cpp(name, index):
    _name, kw, expected, error = gc.random_case(index)
    msg, _identity, _attempt = oracle.call(oracle.load(), name, **kw)
    assert msg == error
    gc.assert_outputs_equal(name, kw, expected, exact=True)


def test_oracle_matches_awkward_cpp_live():
    """When awkward-cpp's kernels are built here, re-run a few cases against them live."""
    ref = oracle.load_ref() if oracle._build.os.path.exists(oracle._build.REF_SO) else None
    if ref is None:
        pytest.skip("awkward-cpp CPU kernels not built on this machine")
    rng = np.random.default_rng(7)
    L = rng.poisson(8, 5000)
    L[rng.random(5000) < 0.01] = 0
    off = np.concatenate([[0], np.cumsum(L)]).astype(np.int64)
    x = rng.standard_normal(int(off[-1]))
    for name in ["awkward_reduce_sum_float64_float64_64", "awkward_reduce_argmax_float64_64"]:
        outs = []
        for lib in (oracle.load(), ref):
            dt = np.float64 if "sum" in name else np.int64
            t = np.zeros(len(L), dt)
            kw = dict(toptr=t, fromptr=x, offsets=off, outlength=len(L))
            if "argmax" in name:
                kw["starts"] = off[:-1].copy()
            assert oracle.call(lib, name, **kw)[0] is None
            outs.append(t)
        np.testing.assert_array_equal(outs[0], outs[1])
