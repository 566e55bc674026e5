"""Golden cases shared by the oracle tests and the GPU parity tests.

Two sources, both committed under tests/golden/ by make_golden.py:

* awkward's own kernel unit tests (kernel-test-data.json), expanded per
  dtype specialization exactly as awkward's test generator does
  (dev/generate-tests.py:1440-1663): outputs pre-filled with 123, values cast
  to the specialization's dtypes, cases skipped when a value does not fit the
  dtype (``checkuint``/``checkintrange``, dev/generate-tests.py:280-309), and
  only the first ``len(expected)`` output entries compared;
* seeded random cases whose expected outputs come from awkward-cpp's own CPU
  kernels.
"""

from __future__ import annotations

import json
import os

import numpy as np

from awkward_gb300._signatures import SIGNATURES

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")

NP = {
    "bool": np.bool_, "int8_t": np.int8, "uint8_t": np.uint8, "int16_t": np.int16,
    "uint16_t": np.uint16, "int32_t": np.int32, "uint32_t": np.uint32,
    "int64_t": np.int64, "uint64_t": np.uint64, "float": np.float32, "double": np.float64,
}

_UNIT = None
_RANDOM = None


def _unit():
    global _UNIT
    if _UNIT is None:
        with open(os.path.join(GOLDEN, "kernel_test_data_subset.json")) as f:
            _UNIT = json.load(f)
    return _UNIT


def _fits(base, values):
    if base in ("float", "double", "bool"):
        return True
    info = np.iinfo(NP[base])
    return all(int(info.min) <= int(v) <= int(info.max) for v in values)


def unit_case_ids():
    """(specialization, index) of every applicable kernel-test-data case."""
    out = []
    fams = _unit()
    for name, rec in SIGNATURES.items():
        fam = rec["family"]
        if fam not in fams:
            continue
        args = {a[0]: a for a in rec["args"]}
        for i, t in enumerate(fams[fam]["tests"]):
            vals = dict(t["inputs"])
            vals.update(t["outputs"])
            ok = True
            for an, v in vals.items():
                if an not in args:
                    ok = False
                    break
                base, depth = args[an][1], args[an][3]
                flat = v if depth == 1 else [x for row in v for x in row] if depth == 2 else [v]
                if base.startswith("uint") and any(x < 0 for x in flat):
                    ok = False
                if not t["error"] and not _fits(base, flat):
                    ok = False
            if ok:
                out.append((name, i))
    return out


def unit_case(name, index):
    """Inputs (numpy, outputs pre-filled with 123) and expectations of one case."""
    rec = SIGNATURES[name]
    t = _unit()[rec["family"]]["tests"][index]
    kw = {}
    expected = {}
    # Output buffers get room beyond the expected prefix: awkward's error
    # cases list empty expected outputs, while the kernels write their full
    # output (e.g. len+1 offsets) before the error is known.  Only the
    # expected prefix is compared.
    pad = 16 + max([len(v) for v in t["inputs"].values() if isinstance(v, list)] + [0])
    for (an, base, d, depth, _c, _r) in rec["args"]:
        dt = NP[base]
        if an in t["inputs"]:
            v = t["inputs"][an]
            if depth == 0:
                kw[an] = bool(v) if base == "bool" else (float(v) if base in ("float", "double") else int(v))
            elif depth == 1:
                kw[an] = np.array(v, dtype=dt) if len(v) else np.zeros(0, dt)
            else:
                kw[an] = [np.array(r, dtype=dt) for r in v]
        elif an in t["outputs"]:
            v = t["outputs"][an]
            fill = True if base == "bool" else (123.0 if base in ("float", "double") else 123)
            if depth == 1:
                kw[an] = np.full(len(v) + pad, fill, dtype=dt)
            elif depth == 2:
                kw[an] = [np.full(len(r) + pad, fill, dtype=dt) for r in v]
            else:
                raise AssertionError("scalar output")
        else:
            raise AssertionError(f"missing argument {an}")
        if an in t["outputs"]:
            v = t["outputs"][an]
            if depth == 1:
                expected[an] = np.array([min(x, 1) if base == "bool" else x for x in v], dtype=dt) if len(v) else np.zeros(0, dt)
            else:
                expected[an] = [np.array(r, dtype=dt) for r in v]
    return kw, expected, (t["message"] if t["error"] else None)


def _random():
    global _RANDOM
    if _RANDOM is None:
        z = np.load(os.path.join(GOLDEN, "ref_random.npz"))
        manifest = json.loads(bytes(z["manifest"]).decode())
        _RANDOM = (z, manifest)
    return _RANDOM


def random_case_ids():
    _z, manifest = _random()
    return [(m["name"], i) for i, m in enumerate(manifest)]


def random_case(index):
    """Inputs (fresh numpy copies), expected outputs and error of one random case."""
    z, manifest = _random()
    m = manifest[index]
    kw = dict(m["scalars"])
    expected = {}
    for an in m["arrays"]:
        kw[an] = z[f"{index}:in:{an}"].copy()
    for an, nrows in m["lists"].items():
        kw[an] = [z[f"{index}:in:{an}:{r}"].copy() for r in range(nrows)]
        expected[an] = [z[f"{index}:out:{an}:{r}"] for r in range(nrows)]
    for an in m["outs"]:
        if an not in m["lists"]:
            expected[an] = z[f"{index}:out:{an}"]
    return m["name"], kw, expected, m["error"]


def is_float_sum_like(name):
    """True for float-output specializations whose result depends on summation order."""
    fam = SIGNATURES[name]["family"]
    out = SIGNATURES[name]["args"][0][1]
    return out in ("float", "double") and fam in (
        "awkward_reduce_sum", "awkward_reduce_prod", "awkward_reduce_sumofsquares",
        "awkward_reduce_sumofpowers", "awkward_reduce_centered_sumofsquares")


def is_complex_sum(name):
    """The complex sums: two order-dependent float outputs per list."""
    return SIGNATURES[name]["family"] == "awkward_reduce_sum_complex"


def assert_outputs_equal(name, got, expected, exact=True):
    """Compare outputs; ``exact`` demands bit-for-bit equality (NaN == NaN)."""
    for an, exp in expected.items():
        g = got[an]
        if isinstance(exp, list):
            assert len(g) >= len(exp), an
            for r, (gr, er) in enumerate(zip(g, exp)):
                np.testing.assert_array_equal(np.asarray(gr)[: len(er)], er, err_msg=f"{name}:{an}[{r}]")
            continue
        g = np.asarray(g)[: len(exp)]
        if exact or exp.dtype.kind not in "f":
            if exp.dtype.kind == "f":
                # bitwise (distinguishes -0.0 from +0.0); any NaN payload matches NaN
                gn, en = np.isnan(g), np.isnan(exp)
                np.testing.assert_array_equal(gn, en, err_msg=f"{name}:{an} NaN positions")
                gi = g.view(np.uint32 if exp.dtype == np.float32 else np.uint64)
                ei = exp.view(np.uint32 if exp.dtype == np.float32 else np.uint64)
                np.testing.assert_array_equal(gi[~en], ei[~en], err_msg=f"{name}:{an}")
            else:
                np.testing.assert_array_equal(g, exp, err_msg=f"{name}:{an}")
        else:
            np.testing.assert_allclose(g, exp, rtol=1e-5 if exp.dtype == np.float32 else 1e-12,
                                       atol=1e-5 if exp.dtype == np.float32 else 1e-12,
                                       equal_nan=True, err_msg=f"{name}:{an}")
