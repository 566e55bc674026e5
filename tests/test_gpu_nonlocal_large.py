"""GPU parity of the non-local / option-type reduction kernels beyond the golden fixtures.

Bit-exact against the C oracle on seeded inputs large enough to span many
tiles of every kernel: the bin-major regrouping of one bin of 300,000 rows
(the axis=0 reduction of a jagged array) and of 20,000 bins (several radix
passes), its nextshifts, the option-type compactions over millions of
entries, and the permutation of local_preparenext.
"""

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

S = 777


def _gpu(name, kw):
    """Run `name` on the GPU with numpy inputs; returns the outputs as numpy."""
    import torch

    import awkward_gb300
    from awkward_gb300._signatures import SIGNATURES

    be = awkward_gb300.backend()
    args, dev = [], {}
    for (an, _base, _d, depth, _c, _r) in SIGNATURES[name]["args"]:
        v = kw[an]
        if depth == 0:
            args.append(v)
        else:
            dev[an] = torch.from_numpy(np.ascontiguousarray(v).copy()).cuda()
            args.append(dev[an])
    be.by_name(name)(*args)
    be.synchronize()
    return {k: t.cpu().numpy() for k, t in dev.items()}


def _cpu(name, kw):
    kw = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in kw.items()}
    oracle.call(oracle.load(), name, **kw)
    return kw


def _check(name, kw, outs):
    exp = _cpu(name, kw)
    got = _gpu(name, kw)
    for o in outs:
        np.testing.assert_array_equal(got[o], exp[o], err_msg=f"{name}:{o}")
    return exp


def _two_level(rng, nbins, lam_rows, lam_len, long_row=0):
    R = rng.poisson(lam_rows, nbins).astype(np.int64)
    R[rng.random(nbins) < 0.05] = 0
    outer = np.concatenate([[0], np.cumsum(R)]).astype(np.int64)
    L = rng.poisson(lam_len, int(outer[-1])).astype(np.int64)
    L[rng.random(len(L)) < 0.1] = 0
    if long_row and len(L):
        L[rng.integers(0, len(L))] = long_row
    off = np.concatenate([[0], np.cumsum(L)]).astype(np.int64)
    return outer, off, L


@pytest.mark.parametrize("nbins,lam_rows,lam_len,long_row",
                         [(1, 300_000, 6, 0), (20_000, 6, 5, 0), (300, 40, 3, 5000)])
def test_preparenext_and_nextshifts(nbins, lam_rows, lam_len, long_row):
    rng = np.random.default_rng(nbins)
    outer, off, L = _two_level(rng, nbins, lam_rows, lam_len, long_row)
    nrows, E = len(L), int(off[-1])
    M = int(L.max()) if nrows else 0
    nb = nbins * M
    kw = {"nextcarry": np.full(E, S, np.int64), "nextoffsets": np.full(nb + 1, S, np.int64),
          "nextlen": E, "maxnextparents": np.full(1, S, np.int64),
          "distincts": np.full(nb, S, np.int64), "distinctslen": nb,
          "offsetscopy": np.full(nrows + 1, S, np.int64), "offsets": off, "length": nrows,
          "outer_offsets": outer, "outlength": nbins, "maxcount": M}
    exp = _check("awkward_ListOffsetArray_reduce_nonlocal_preparenext_64", kw,
                 ["nextcarry", "nextoffsets", "maxnextparents", "distincts"])
    kw2 = {"nummissing": np.full(M, S, np.int64), "missing": np.full(E, S, np.int64),
           "nextshifts": np.full(E, S, np.int64), "offsets": off, "length": nrows,
           "starts": off[:-1].copy(), "outer_offsets": outer, "outlength": nbins,
           "maxcount": M, "nextlen": E, "nextcarry": exp["nextcarry"]}
    _check("awkward_ListOffsetArray_reduce_nonlocal_nextshifts_64", kw2,
           ["nummissing", "missing", "nextshifts"])
    out = {"outstarts": np.full(nbins, S, np.int64), "outstops": np.full(nbins, S, np.int64),
           "distincts": exp["distincts"], "lendistincts": nb, "outlength": nbins}
    _check("awkward_ListOffsetArray_reduce_nonlocal_outstartsstops_64", out,
           ["outstarts", "outstops"])


def test_maxcount_and_local_nextparents():
    rng = np.random.default_rng(5)
    L = rng.poisson(7, 2_000_000).astype(np.int64)
    L[12345] = 100_000
    off = np.concatenate([[0], np.cumsum(L)]).astype(np.int64)
    n = len(L)
    _check("awkward_ListOffsetArray_reduce_nonlocal_maxcount_offsetscopy_64",
           {"maxcount": np.full(1, S, np.int64), "offsetscopy": np.full(n + 1, S, np.int64),
            "offsets": off, "length": n}, ["maxcount", "offsetscopy"])
    for C, tag in ((np.int64, "64"), (np.int32, "32"), (np.uint32, "U32")):
        o = (off + 11).astype(C)
        E = int(off[-1])
        _check(f"awkward_ListOffsetArray{tag}_reduce_local_nextparents_64",
               {"nextparents": np.full(E, S, C), "offsets": o, "length": n,
                "nextparents_length": E - 1000}, ["nextparents"])


def test_regular_array_kernels():
    rng = np.random.default_rng(6)
    R = rng.poisson(5, 400_000).astype(np.int64)
    R[::997] = 0
    off = np.concatenate([[0], np.cumsum(R)]).astype(np.int64)
    rows, size = int(off[-1]), 7
    _check("awkward_RegularArray_reduce_nonlocal_preparenext_64",
           {"nextcarry": np.full(rows * size, S, np.int64),
            "nextoffsets": np.full(len(R) * size + 1, S, np.int64), "offsets": off, "size": size,
            "length": rows, "outlength": len(R)}, ["nextcarry", "nextoffsets"])
    _check("awkward_RegularArray_reduce_local_nextparents_64",
           {"nextparents": np.full(rows * size, S, np.int64), "size": size, "length": rows},
           ["nextparents"])


@pytest.mark.parametrize("tag,T", [("32", np.int32), ("U32", np.uint32), ("64", np.int64)])
def test_indexed_compactions(tag, T):
    rng = np.random.default_rng(7)
    L = rng.poisson(4, 1_500_000).astype(np.int64)
    L[rng.random(len(L)) < 0.2] = 0
    off = np.concatenate([[0], np.cumsum(L)]).astype(np.int64)
    E = int(off[-1])
    idx = rng.integers(0, 1 << 30, E)
    if T != np.uint32:
        idx[rng.random(E) < 0.3] = -1
    idx = idx.astype(T)
    _check(f"awkward_IndexedArray{tag}_reduce_next_64",
           {"nextcarry": np.full(E, S, np.int64), "nextoffsets": np.full(len(L) + 1, S, np.int64),
            "outindex": np.full(E, S, np.int64), "index": idx, "offsets": off, "outlength": len(L)},
           ["nextcarry", "nextoffsets", "outindex"])
    _check(f"awkward_IndexedArray{tag}_reduce_next_nonlocal_nextshifts_64",
           {"nextshifts": np.full(E, S, np.int64), "index": idx, "length": E}, ["nextshifts"])
    _check(f"awkward_IndexedArray{tag}_reduce_next_nonlocal_nextshifts_fromshifts_64",
           {"nextshifts": np.full(E, S, np.int64), "index": idx, "length": E,
            "shifts": rng.integers(0, 50, E).astype(np.int64)}, ["nextshifts"])


@pytest.mark.parametrize("validwhen", [True, False])
def test_bytemasked_compactions(validwhen):
    rng = np.random.default_rng(8)
    L = rng.poisson(5, 1_000_000).astype(np.int64)
    off = np.concatenate([[0], np.cumsum(L)]).astype(np.int64)
    E = int(off[-1])
    m = (rng.random(E) < 0.7).astype(np.int8) * 3
    _check("awkward_ByteMaskedArray_reduce_next_64",
           {"nextcarry": np.full(E, S, np.int64), "nextoffsets": np.full(len(L) + 1, S, np.int64),
            "outindex": np.full(E, S, np.int64), "mask": m, "offsets": off, "outlength": len(L),
            "validwhen": validwhen}, ["nextcarry", "nextoffsets", "outindex"])
    _check("awkward_ByteMaskedArray_reduce_next_nonlocal_nextshifts_64",
           {"nextshifts": np.full(E, S, np.int64), "mask": m, "length": E,
            "valid_when": validwhen}, ["nextshifts"])
    _check("awkward_ByteMaskedArray_reduce_next_nonlocal_nextshifts_fromshifts_64",
           {"nextshifts": np.full(E, S, np.int64), "mask": m, "length": E,
            "valid_when": validwhen, "shifts": rng.integers(0, 50, E).astype(np.int64)},
           ["nextshifts"])


def test_local_preparenext_and_indexed_local():
    rng = np.random.default_rng(9)
    n = 3_000_000
    _check("awkward_ListOffsetArray_local_preparenext_64",
           {"tocarry": np.full(n, S, np.int64),
            "fromindex": rng.permutation(n).astype(np.int64) * 3 - 1000, "length": n}, ["tocarry"])
    Lo = rng.poisson(5, 500_000).astype(np.int64)
    off = np.concatenate([[0], np.cumsum(Lo)]).astype(np.int64)
    Li = np.minimum(Lo, rng.poisson(3, len(Lo)))
    _check("awkward_IndexedArray_local_preparenext_64",
           {"tocarry": np.full(int(off[-1]), S, np.int64), "starts": off[:-1].copy(),
            "offsets": off, "nextoffsets": np.concatenate([[0], np.cumsum(Li)]).astype(np.int64),
            "outlength": len(Lo)}, ["tocarry"])
    st = np.sort(rng.integers(0, 1 << 40, 1_000_000)).astype(np.int64)
    _check("awkward_IndexedArray_reduce_next_fix_offsets_64",
           {"outoffsets": np.full(len(st) + 1, S, np.int64), "starts": st,
            "startslength": len(st), "outindexlength": 1 << 41}, ["outoffsets"])
