"""GPU parity of segmented sort / argsort beyond the golden fixtures.

Bit-exact against the C oracle (a stable merge sort with awkward-cpp's
comparators) on seeded inputs that exercise every segment class of the GPU
path: segments of 0..32 elements (one warp), 33..2048 (one CTA in shared
memory) and longer ones (runs of 2048 merged pass by pass, up to 300,000
elements), in both directions, with heavy ties (the stable order must hold),
NaN, +-0.0 and +-inf for floating point, and offsets that end before or run
past `length`.
"""

import zlib

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

NP_T = {"bool": np.bool_, "int8": np.int8, "uint8": np.uint8, "int16": np.int16,
        "uint16": np.uint16, "int32": np.int32, "uint32": np.uint32, "int64": np.int64,
        "uint64": np.uint64, "float32": np.float32, "float64": np.float64}
NP_U = {"int32": np.int32, "uint32": np.uint32, "int64": np.int64, "uint64": np.uint64}


def _lengths(kind, rng):
    if kind == "short":
        return rng.integers(0, 33, 20_000)
    if kind == "medium":
        return rng.integers(30, 2100, 400)
    if kind == "long":
        return np.array([2049, 4096, 5000, 0, 1, 70_001, 300_000, 2048, 33, 16_385])
    if kind == "mixed":
        L = np.minimum(rng.poisson(6, 50_000), 40)
        L[::5000] = rng.integers(2000, 20_000, len(L[::5000]))
        return L
    raise KeyError(kind)


def _values(tname, n, rng, ties):
    t = NP_T[tname]
    if tname == "bool":
        return rng.random(n) < 0.5
    if tname.startswith("float"):
        x = np.round(rng.standard_normal(n), 1 if ties else 6).astype(t)
        k = rng.random(n)
        x[k < 0.03] = np.nan
        x[(k >= 0.03) & (k < 0.05)] = -0.0
        x[(k >= 0.05) & (k < 0.07)] = 0.0
        x[(k >= 0.07) & (k < 0.08)] = np.inf
        x[(k >= 0.08) & (k < 0.09)] = -np.inf
        return x
    info = np.iinfo(t)
    if ties:
        lo, hi = max(info.min, -5), min(info.max, 5)
        return rng.integers(lo, hi + 1, n).astype(t)
    return rng.integers(info.min, info.max, n, dtype=t, endpoint=True)


def _oracle_sort(arg, tname, uname, x, off, length, asc):
    lib = oracle.load()
    if arg:
        out = np.zeros(length, np.int64)
        oracle.call(lib, f"awkward_argsort_{tname}_{uname}", toptr=out, fromptr=x,
                    length=length, offsets=off, offsetslength=len(off), ascending=asc,
                    stable=True)
    else:
        out = np.zeros(length, NP_T[tname])
        oracle.call(lib, f"awkward_sort_{tname}", toptr=out, fromptr=x, length=length,
                    offsets=off, offsetslength=len(off), ascending=asc, stable=True)
    return out


def _gpu_sort(arg, tname, uname, x, off, length, asc):
    import torch

    import awkward_gb300

    be = awkward_gb300.backend()
    xd = torch.from_numpy(x.copy()).cuda()
    od = torch.from_numpy(off.copy()).cuda()
    if arg:
        out = torch.zeros(length, dtype=torch.int64, device="cuda")
        be.by_name(f"awkward_argsort_{tname}_{uname}")(out, xd, length, od, len(off), asc, True)
    else:
        out = torch.zeros(length, dtype=xd.dtype, device="cuda")
        be.by_name(f"awkward_sort_{tname}")(out, xd, length, od, len(off), asc, True)
    be.synchronize()
    return out.cpu().numpy()


def _case(kind, tname, ties, seed):
    rng = np.random.default_rng(seed)
    L = _lengths(kind, rng)
    off = np.concatenate([[0], np.cumsum(L)]).astype(np.int64)
    x = _values(tname, int(off[-1]), rng, ties)
    return off, x


def _same(got, exp):
    if got.dtype.kind == "f":
        np.testing.assert_array_equal(got.view(np.uint8), exp.view(np.uint8))
    else:
        np.testing.assert_array_equal(got, exp)


@pytest.mark.parametrize("kind", ["short", "medium", "long", "mixed"])
@pytest.mark.parametrize("tname", ["float64", "float32", "int64", "int32"])
@pytest.mark.parametrize("asc", [True, False])
def test_argsort_matches_oracle(kind, tname, asc):
    off, x = _case(kind, tname, ties=True, seed=zlib.crc32(f"{kind}{tname}{asc}".encode()))
    exp = _oracle_sort(True, tname, "int64", x, off, len(x), asc)
    got = _gpu_sort(True, tname, "int64", x, off, len(x), asc)
    _same(got, exp)


@pytest.mark.parametrize("kind", ["short", "medium", "long"])
@pytest.mark.parametrize("tname", list(NP_T))
def test_sort_matches_oracle_every_type(kind, tname):
    off, x = _case(kind, tname, ties=tname not in ("uint64",), seed=7 + len(tname))
    for asc in (True, False):
        _same(_gpu_sort(False, tname, "int64", x, off, len(x), asc),
              _oracle_sort(False, tname, "int64", x, off, len(x), asc))


@pytest.mark.parametrize("uname", list(NP_U))
def test_argsort_offset_types(uname):
    off, x = _case("mixed", "int16", ties=True, seed=99)
    off = off.astype(NP_U[uname])
    for asc in (True, False):
        _same(_gpu_sort(True, "int16", uname, x, off, len(x), asc),
              _oracle_sort(True, "int16", uname, x, off, len(x), asc))


@pytest.mark.parametrize("arg", [True, False])
def test_offsets_past_length_and_short_of_it(arg):
    rng = np.random.default_rng(3)
    off = np.array([0, 5, 40, 3000, 3100, 9000], np.int64)
    x = _values("float64", 5000, rng, ties=True)
    for length in (5000, 2500, 3050):
        for o in (off, off[:4]):
            _same(_gpu_sort(arg, "float64", "int64", x[:length], o, length, True),
                  _oracle_sort(arg, "float64", "int64", x[:length], o, length, True))


def test_unstable_distinct_values_sorted():
    """stable=False may return any order of ties; with distinct values it is unique."""
    rng = np.random.default_rng(11)
    L = rng.integers(0, 5000, 300)
    off = np.concatenate([[0], np.cumsum(L)]).astype(np.int64)
    x = rng.permutation(int(off[-1])).astype(np.float64)
    import torch

    import awkward_gb300

    be = awkward_gb300.backend()
    out = torch.zeros(len(x), dtype=torch.int64, device="cuda")
    be.by_name("awkward_argsort_float64_int64")(out, torch.from_numpy(x).cuda(), len(x),
                                               torch.from_numpy(off).cuda(), len(off), False,
                                               False)
    be.synchronize()
    exp = _oracle_sort(True, "float64", "int64", x, off, len(x), False)
    np.testing.assert_array_equal(out.cpu().numpy(), exp)
