"""GPU parity of the fused map + segmented reduction (awkward_gb300.fused).

The oracle is the reference computation unfused: the mapped values
(x*y, x*x, |x|, x) materialised with numpy (IEEE products, rounded once,
like an elementwise kernel), then awkward-cpp's reducers restated in C.
max/min/argmax/argmin must match bit for bit; sums must lie within
4*n*eps*sum|v| of the FP64 compensated-sum oracle over the mapped values.
Length distributions cover the staged rounds (short lists), long lists
reduced by the whole warp, giant lists crossing warp ranges, empty lists,
offsets not starting at 0, and NaN / signed zeros / infinities.
"""

import zlib

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

KINDS = ["poisson", "long", "giant", "empty", "shifted"]
MAPS = ["x", "x*y", "x*x", "abs"]
REDS = ["sum", "max", "min", "argmax", "argmin"]


def _case(kind, seed):
    rng = np.random.default_rng(seed)
    if kind == "poisson":
        L = rng.poisson(8, 30000)
        L[rng.random(len(L)) < 0.01] = 0
    elif kind == "long":
        L = rng.poisson(8, 3000)
        L[::37] = rng.integers(33, 5000, len(L[::37]))
    elif kind == "giant":
        L = np.array([0] * 40 + [600_000] + [3] * 100 + [0] * 10)
    elif kind == "empty":
        L = np.zeros(4000, np.int64)
    else:
        L = rng.poisson(5, 20000)
    base = 7 if kind == "shifted" else 0
    off = (np.concatenate([[0], np.cumsum(L)]) + base).astype(np.int64)
    E = int(off[-1])
    x = rng.standard_normal(E)
    y = rng.standard_normal(E) * 3
    if E > base:
        x[rng.integers(base, E, max(E // 700, 1))] = np.nan
        x[rng.integers(base, E, max(E // 300, 1))] = -0.0
        x[rng.integers(base, E, max(E // 300, 1))] = 0.0
        y[rng.integers(base, E, max(E // 2000, 1))] = np.inf
        starts = off[:-1][L > 0]
        x[starts[rng.random(len(starts)) < 0.02]] = np.nan
    return off, x, y


def _mapped(map_, x, y):
    with np.errstate(all="ignore"):
        return {"x": x, "x*y": x * y, "x*x": x * x, "abs": np.abs(x)}[map_]


def _oracle(red, v, off):
    lib = oracle.load()
    n = len(off) - 1
    if red in ("argmax", "argmin"):
        out = np.zeros(n, np.int64)
        oracle.call(lib, f"awkward_reduce_{red}_float64_64", toptr=out, fromptr=v, offsets=off,
                    starts=off[:-1].copy(), outlength=n)
    else:
        out = np.zeros(n)
        ident = {"max": -np.inf, "min": np.inf}.get(red)
        kw = {"identity": ident} if ident is not None else {}
        oracle.call(lib, f"awkward_reduce_{red}_float64_float64_64", toptr=out, fromptr=v,
                    offsets=off, outlength=n, **kw)
    return out


@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("map_", MAPS)
def test_fused_reduce_matches_materialised_oracle(kind, map_):
    import torch

    from awkward_gb300.fused import segment_reduce

    off, x, y = _case(kind, zlib.crc32(f"{kind}:{map_}".encode()) % 1000)
    v = _mapped(map_, x, y)
    dx, dy, doff = (torch.from_numpy(a).cuda() for a in (x, y, off))
    for red in REDS:
        got = segment_reduce(dx, doff, map=map_, y=dy if map_ == "x*y" else None,
                             reduce=red).cpu().numpy()
        if red == "sum":
            rep = oracle.sum_error_report(got, v, off)
            assert rep["within"] and rep["nonfinite_ok"], (kind, map_, rep)
        else:
            exp = _oracle(red, v, off)
            if red.startswith("arg"):
                np.testing.assert_array_equal(got, exp, err_msg=f"{kind} {map_} {red}")
            else:
                np.testing.assert_array_equal(got.view(np.int64), exp.view(np.int64),
                                              err_msg=f"{kind} {map_} {red}")


def test_fused_rejects_bad_arguments():
    import torch

    from awkward_gb300 import _abi

    f = _abi.ext_cfunc("awkward_gb300_fused_reduce_float64")
    x = torch.zeros(4, dtype=torch.float64, device="cuda")
    off = torch.tensor([0, 2, 4], dtype=torch.int64, device="cuda")
    out = torch.empty(2, dtype=torch.float64, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    assert f(out.data_ptr(), x.data_ptr(), None, off.data_ptr(), 2, 1, 0, 0, None, s) == 1
    assert f(out.data_ptr(), x.data_ptr(), None, off.data_ptr(), 2, 0, 7, 0, None, s) == 1
    assert f(out.data_ptr(), x.data_ptr(), None, off.data_ptr(), 2, 9, 0, 0, None, s) == 1
