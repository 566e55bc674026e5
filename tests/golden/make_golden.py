"""Regenerate the committed golden fixtures (run by hand, where awkward's sources are).

    python tests/golden/make_golden.py [/path/to/awkward]

Writes two files next to this script:

* ``kernel_test_data_subset.json`` -- the unit tests of awkward's
  ``kernel-test-data.json`` for every kernel family libawkward_gb300 exports
  (inputs, expected outputs, error flag and message), unchanged.
* ``ref_random.npz`` -- seeded random cases for every family (including the
  three with no unit tests: sumofsquares, sumofpowers, centered_sumofsquares),
  each run through awkward-cpp's OWN CPU kernels compiled by
  ``oracle/build.py``; stores inputs, the outputs after the call and the
  returned error.  A JSON manifest (key ``manifest``) lists the cases.

Both pin the C restatement in ``oracle/`` and are the fixtures of the GPU
parity tests.  Nothing here runs at test time.
"""

from __future__ import annotations

import json
import os
import sys
import zlib

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from awkward_gb300._signatures import SIGNATURES  # noqa: E402
from awkward_gb300.gen_signatures import FAMILIES  # noqa: E402

import oracle  # noqa: E402
from oracle import NP_DTYPES  # noqa: E402

SLICE_NONE = np.iinfo(np.int64).max


def extract_unit_tests(awkward_src):
    with open(os.path.join(awkward_src, "kernel-test-data.json")) as f:
        data = json.load(f)["unit-tests"]
    out = {}
    for rec in data:
        if rec["name"] in FAMILIES:
            out[rec["name"]] = {"status": rec["status"], "tests": rec["tests"]}
    with open(os.path.join(HERE, "kernel_test_data_subset.json"), "w") as f:
        json.dump(out, f, separators=(",", ":"))
    return sum(len(v["tests"]) for v in out.values())


# ---------------------------------------------------------------- random inputs
def _lengths(rng, n, lam, p_empty=0.05, longs=(33, 257, 1025)):
    L = rng.poisson(lam, n).astype(np.int64)
    L[rng.random(n) < p_empty] = 0
    for k, ln in enumerate(longs):
        if n > 3 * (k + 1):
            L[rng.integers(0, n)] = ln
    return L


def _offsets(L):
    return np.concatenate([[0], np.cumsum(L)]).astype(np.int64)


def _values(rng, base, n):
    dt = NP_DTYPES[base]
    if base == "bool":
        return rng.random(n) < 0.5
    if base in ("float", "double"):
        x = rng.standard_normal(n).astype(dt)
        # exercise the comparison rules: NaN, signed zeros, infinities, ties
        k = max(n // 40, 1)
        for special in (np.nan, 0.0, -0.0, np.inf, -np.inf, 1.0):
            idx = rng.integers(0, n, k) if n else np.zeros(0, np.int64)
            x[idx] = special
        return x
    info = np.iinfo(dt)
    lo = max(int(info.min), -100)
    hi = min(int(info.max), 100)
    x = rng.integers(lo, hi + 1, n).astype(dt)
    if n:
        x[rng.integers(0, n, max(n // 50, 1))] = 0
    return x


def reducer_case(rng, name):
    rec = SIGNATURES[name]
    args = {a[0]: a for a in rec["args"]}
    L = _lengths(rng, 300, 4)
    off = _offsets(L)
    E = int(off[-1])
    kw = {"offsets": off, "outlength": len(L)}
    if "fromptr" in args:
        base = args["fromptr"][1]
        kw["fromptr"] = _values(rng, base, E)
        if name.startswith(("awkward_reduce_max", "awkward_reduce_min")) and rng.random() < 0.5:
            kw["fromptr"][: min(E, 5)] = kw["fromptr"][0] if E else 0
    if "starts" in args:
        kw["starts"] = off[:-1].copy()
    if "identity" in args:
        base = args["identity"][1]
        if base in ("float", "double"):
            kw["identity"] = float(-np.inf if "max" in name else np.inf)
        else:
            info = np.iinfo(NP_DTYPES[base])
            kw["identity"] = int(info.min if "max" in name else info.max)
    if "means" in args:
        kw["means"] = rng.standard_normal(len(L))
    if "n" in args:
        kw["n"] = int(rng.choice([0, 1, 2, 3, -1]))
    base = args["toptr"][1]
    if name == "awkward_NumpyArray_reduce_adjust_starts_64":
        kw["toptr"] = np.where(L > 0, off[:-1] + (L > 0) * (rng.integers(0, 1 << 20, len(L)) % np.maximum(L, 1)), -1).astype(np.int64)
        kw["starts"] = off[:-1].copy()
    else:
        kw["toptr"] = np.full(len(L), 123, dtype=NP_DTYPES[base])
    return kw


def jagged_case(rng, name):
    rec = SIGNATURES[name]
    fam = rec["family"]
    args = {a[0]: a for a in rec["args"]}
    n = 200
    if fam == "awkward_ListArray_getitem_jagged_apply":
        C = NP_DTYPES[args["fromstarts"][1]]
        L = _lengths(rng, n, 5, longs=(40,))
        off = _offsets(L)
        K = np.where(L > 0, rng.poisson(3, n), 0)
        soff = _offsets(K)
        idx = np.concatenate([rng.integers(-l, l, k) if k else np.zeros(0, np.int64) for l, k in zip(L, K)]).astype(np.int64)
        return {"tooffsets": np.full(n + 1, 123, np.int64), "tocarry": np.full(len(idx), 123, np.int64),
                "slicestarts": soff[:-1].copy(), "slicestops": soff[1:].copy(), "sliceouterlen": n,
                "sliceindex": idx, "sliceinnerlen": len(idx), "fromstarts": off[:-1].astype(C),
                "fromstops": off[1:].astype(C), "contentlen": int(off[-1])}
    if fam == "awkward_ListArray_getitem_jagged_carrylen":
        L = _lengths(rng, n, 5)
        off = _offsets(L)
        return {"carrylen": np.full(1, 123, np.int64), "slicestarts": off[:-1].copy(),
                "slicestops": off[1:].copy(), "sliceouterlen": n}
    if fam == "awkward_ListArray_getitem_jagged_descend":
        C = NP_DTYPES[args["fromstarts"][1]]
        L = _lengths(rng, n, 5)
        off = _offsets(L) + 7
        return {"tooffsets": np.full(n + 1, 123, np.int64), "slicestarts": off[:-1].copy(),
                "slicestops": off[1:].copy(), "sliceouterlen": n,
                "fromstarts": (off[:-1] * 2).astype(C), "fromstops": (off[:-1] * 2 + L).astype(C)}
    if fam == "awkward_ListArray_getitem_jagged_expand":
        C = NP_DTYPES[args["fromstarts"][1]]
        js = 4
        starts = (np.arange(n) * 9).astype(C)
        single = _offsets(rng.poisson(2, js))
        return {"multistarts": np.full(n * js, 123, np.int64), "multistops": np.full(n * js, 123, np.int64),
                "singleoffsets": single, "tocarry": np.full(n * js, 123, np.int64),
                "fromstarts": starts, "fromstops": (starts + js).astype(C), "jaggedsize": js, "length": n}
    if fam == "awkward_ListArray_getitem_jagged_numvalid":
        L = _lengths(rng, n, 5)
        off = _offsets(L)
        missing = np.where(rng.random(int(off[-1])) < 0.3, -1, np.arange(int(off[-1]))).astype(np.int64)
        return {"numvalid": np.full(1, 123, np.int64), "slicestarts": off[:-1].copy(),
                "slicestops": off[1:].copy(), "length": n, "missing": missing,
                "missinglength": len(missing)}
    if fam == "awkward_ListArray_getitem_jagged_shrink":
        L = _lengths(rng, n, 5)
        off = _offsets(L)
        missing = np.where(rng.random(int(off[-1])) < 0.3, -1, np.arange(int(off[-1]))).astype(np.int64)
        nv = int((missing >= 0).sum())
        return {"tocarry": np.full(nv, 123, np.int64), "tosmalloffsets": np.full(n + 1, 123, np.int64),
                "tolargeoffsets": np.full(n + 1, 123, np.int64), "slicestarts": off[:-1].copy(),
                "slicestops": off[1:].copy(), "length": n, "missing": missing}
    if fam == "awkward_RegularArray_getitem_jagged_expand":
        size, length = 5, 60
        single = _offsets(rng.poisson(3, size))
        return {"multistarts": np.full(size * length, 123, np.int64),
                "multistops": np.full(size * length, 123, np.int64), "singleoffsets": single,
                "regularsize": size, "regularlength": length}
    if fam == "awkward_ListArray_localindex":
        C = NP_DTYPES[args["offsets"][1]]
        L = _lengths(rng, n, 5)
        off = _offsets(L)
        return {"toindex": np.full(int(off[-1]), 123, np.int64), "offsets": off.astype(C), "length": n}
    raise KeyError(fam)


def range_cases(rng, name):
    rec = SIGNATURES[name]
    fam = rec["family"]
    args = {a[0]: a for a in rec["args"]}
    out = []
    slices = [(1, SLICE_NONE, 1), (SLICE_NONE, SLICE_NONE, 2), (-3, SLICE_NONE, 1),
              (SLICE_NONE, -1, 1), (SLICE_NONE, SLICE_NONE, -1), (5, 1, -2), (2, 100, 3),
              (-100, 100, 7), (SLICE_NONE, 2, -3)]
    if fam == "awkward_RegularArray_getitem_next_range":
        for (rs, step, length, size, nextsize) in [(1, 1, 50, 6, 5), (5, -2, 30, 6, 3), (0, 3, 10, 9, 3)]:
            out.append({"tocarry": np.full(length * nextsize, 123, np.int64), "regular_start": rs,
                        "step": step, "length": length, "size": size, "nextsize": nextsize})
        return out
    C = NP_DTYPES[args["fromstarts"][1]]
    for (a, b, c) in slices:
        n = 150
        L = _lengths(rng, n, 5, longs=(20,))
        off = _offsets(L)
        starts = off[:-1].astype(C)
        stops = off[1:].astype(C)
        if fam == "awkward_ListArray_getitem_next_range_carrylength":
            out.append({"carrylength": np.full(1, 123, np.int64), "fromstarts": starts, "fromstops": stops,
                        "lenstarts": n, "start": a, "stop": b, "step": c})
        else:
            total = int(off[-1])
            out.append({"tooffsets": np.full(n + 1, 123, C), "tocarry": np.full(total, 123, np.int64),
                        "fromstarts": starts, "fromstops": stops, "lenstarts": n,
                        "start": a, "stop": b, "step": c})
    return out


def combinations_cases(rng, name):
    rec = SIGNATURES[name]
    fam = rec["family"]
    C = NP_DTYPES[{a[0]: a for a in rec["args"]}["starts"][1]]
    out = []
    for n_, repl in [(2, False), (3, False), (2, True), (3, True), (1, False), (4, False)]:
        n = 120
        L = np.minimum(rng.poisson(4, n), 9).astype(np.int64)
        L[rng.random(n) < 0.05] = 0
        off = _offsets(L)
        starts, stops = off[:-1].astype(C), off[1:].astype(C)
        if fam == "awkward_ListArray_combinations_length":
            out.append({"totallen": np.full(1, 123, np.int64), "tooffsets": np.full(n + 1, 123, np.int64),
                        "n": n_, "replacement": repl, "starts": starts, "stops": stops, "length": n})
        else:
            tmp_total = np.zeros(1, np.int64)
            oracle.call(oracle.load_ref(), name.replace("_combinations_64", "_combinations_length_64"),
                        totallen=tmp_total, tooffsets=np.zeros(n + 1, np.int64), n=n_,
                        replacement=repl, starts=starts, stops=stops, length=n)
            total = int(tmp_total[0])
            out.append({"tocarry": [np.full(total, 123, np.int64) for _ in range(n_)],
                        "toindex": np.full(n_, 123, np.int64), "fromindex": np.zeros(n_, np.int64),
                        "n": n_, "replacement": repl, "starts": starts, "stops": stops, "length": n})
    return out


def regular_combinations_cases(rng, name):
    out = []
    for n_, repl, size in [(2, False, 5), (3, False, 6), (2, True, 4), (3, True, 3), (1, False, 4),
                           (4, False, 7), (2, False, 1), (3, False, 0)]:
        length = 40
        tmp_total = np.zeros(1, np.int64)
        starts = (np.arange(length) * size).astype(np.int64)
        oracle.call(oracle.load_ref(), "awkward_ListArray64_combinations_length_64",
                    totallen=tmp_total, tooffsets=np.zeros(length + 1, np.int64), n=n_,
                    replacement=repl, starts=starts, stops=starts + size, length=length)
        total = int(tmp_total[0])
        out.append({"tocarry": [np.full(total, 123, np.int64) for _ in range(n_)],
                    "toindex": np.full(n_, 123, np.int64), "fromindex": np.zeros(n_, np.int64),
                    "n": n_, "replacement": repl, "size": size, "length": length})
    return out


def broadcast_cases(rng, name):
    C = NP_DTYPES[{a[0]: a for a in SIGNATURES[name]["args"]}["fromstarts"][1]]
    out = []
    for variant in ("valid", "gaps", "mismatch"):
        n = 200
        L = _lengths(rng, n, 5, longs=(40,))
        off = _offsets(L) + 3
        if variant == "gaps":  # a ListArray whose lists are not contiguous
            starts = np.cumsum(L + rng.integers(0, 3, n)) - L
        else:
            starts = off[:-1] - 3
        stops = starts + L
        if variant == "mismatch":
            stops = stops.copy()
            stops[rng.integers(0, n)] += 1
        lencontent = int(stops.max()) + 2 if n else 0
        out.append({"tocarry": np.full(int(off[-1] - off[0]) + 4, 123, np.int64), "fromoffsets": off,
                    "offsetslength": n + 1, "fromstarts": starts.astype(C),
                    "fromstops": stops.astype(C), "lencontent": lencontent})
    return out


def sort_cases(rng, name):
    rec = SIGNATURES[name]
    args = {a[0]: a for a in rec["args"]}
    base = args["fromptr"][1]
    U = NP_DTYPES[args["offsets"][1]]
    out = []
    for ascending, stable in [(True, True), (False, True), (True, False), (False, False)]:
        if not stable and base in ("bool", "int8_t", "uint8_t"):
            continue  # too few distinct values for a tie-free unstable case
        n = 120
        # the merged path (segments past 2048 elements) in the 64-bit cases only
        wide = base in ("double", "int64_t") and args["offsets"][1] == "int64_t"
        L = _lengths(rng, n, 6, longs=(33, 257, 2050, 5000) if wide else (33, 257))
        off = _offsets(L)
        E = int(off[-1])
        if stable:
            x = _values(rng, base, E)
        else:  # distinct values: std::sort's order is then unique
            dt = NP_DTYPES[base]
            if base in ("float", "double"):
                x = (rng.permutation(E) - E / 2).astype(dt) / 7
            else:
                info = np.iinfo(dt)
                span = min(int(info.max) - int(info.min), 1 << 40)
                x = (rng.permutation(E) % span + (int(info.min) if int(info.min) < 0 else 0)).astype(dt)
        length = E + 3
        xx = np.concatenate([x, np.zeros(3, x.dtype)]) if E else np.zeros(3, NP_DTYPES[base])
        if name.startswith("awkward_argsort"):
            out.append({"toptr": np.full(length, 123, np.int64), "fromptr": xx, "length": length,
                        "offsets": off.astype(U), "offsetslength": n + 1,
                        "ascending": ascending, "stable": stable})
        else:
            out.append({"toptr": np.full(length, 123, NP_DTYPES[base]), "fromptr": xx,
                        "length": length, "offsets": off, "offsetslength": n + 1,
                        "ascending": ascending, "stable": stable})
    return out


def _two_level(rng, nbins, lam_rows, lam_len, longs=(), p_empty_bin=0.1):
    """Outer bins of rows and rows of elements: (outer_offsets, offsets, L)."""
    R = rng.poisson(lam_rows, nbins).astype(np.int64)
    R[rng.random(nbins) < p_empty_bin] = 0
    outer = _offsets(R)
    L = _lengths(rng, int(outer[-1]), lam_len, p_empty=0.1, longs=longs)
    return outer, _offsets(L), L


def nonlocal_cases(rng, name):
    """Seeded inputs of the non-local / option-type reduction kernels."""
    rec = SIGNATURES[name]
    fam = rec["family"]
    args = {a[0]: a for a in rec["args"]}
    out = []
    S = 777  # untouched output slots keep this value
    if fam == "awkward_ListOffsetArray_reduce_nonlocal_maxcount_offsetscopy_64":
        for n in (0, 1, 150):
            off = _offsets(_lengths(rng, n, 5, longs=(40,)))
            out.append({"maxcount": np.full(1, S, np.int64), "offsetscopy": np.full(n + 1, S, np.int64),
                        "offsets": off, "length": n})
    elif fam in ("awkward_ListOffsetArray_reduce_nonlocal_preparenext_64",
                 "awkward_ListOffsetArray_reduce_nonlocal_nextshifts_64"):
        ref = oracle.load()
        for nbins, lr, ll, longs in ((1, 60, 4, ()), (40, 3, 3, ()), (25, 4, 2, (30,)), (0, 1, 1, ())):
            outer, off, L = _two_level(rng, nbins, lr, ll, longs)
            nrows = len(L)
            M = int(L.max()) if nrows else 0
            E = int(off[-1])
            nbinsM = nbins * M
            prep = {"nextcarry": np.full(E, S, np.int64), "nextoffsets": np.full(nbinsM + 1, S, np.int64),
                    "nextlen": E, "maxnextparents": np.full(1, S, np.int64),
                    "distincts": np.full(nbinsM, S, np.int64), "distinctslen": nbinsM,
                    "offsetscopy": np.full(nrows + 1, S, np.int64), "offsets": off, "length": nrows,
                    "outer_offsets": outer, "outlength": nbins, "maxcount": M}
            if fam.endswith("preparenext_64"):
                out.append(prep)
                continue
            kw = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in prep.items()}
            oracle.call(ref, "awkward_ListOffsetArray_reduce_nonlocal_preparenext_64", **kw)
            out.append({"nummissing": np.full(max(M, 1), S, np.int64), "missing": np.full(E, S, np.int64),
                        "nextshifts": np.full(E, S, np.int64), "offsets": off, "length": nrows,
                        "starts": off[:-1].copy(), "outer_offsets": outer, "outlength": nbins,
                        "maxcount": M, "nextlen": E, "nextcarry": kw["nextcarry"]})
    elif fam == "awkward_ListOffsetArray_reduce_nonlocal_outstartsstops_64":
        for outlength, M in ((0, 3), (3, 0), (1, 7), (30, 5), (12, 1)):
            n = outlength * M
            d = np.where(rng.random(n) < 0.4, -1, rng.integers(0, 50, n)).astype(np.int64)
            d[: M] = -1  # one sublist without any entry
            out.append({"outstarts": np.full(outlength, S, np.int64), "outstops": np.full(outlength, S, np.int64),
                        "distincts": d, "lendistincts": n, "outlength": outlength})
    elif fam == "awkward_ListOffsetArray_reduce_local_nextparents_64":
        C = NP_DTYPES[args["offsets"][1]]
        for n, first, trim in ((0, 0, 0), (120, 0, 0), (90, 17, 0), (80, 5, 30)):
            off = _offsets(_lengths(rng, n, 4, longs=(33,))) + first
            E = int(off[-1] - off[0])
            out.append({"nextparents": np.full(E, S, C), "offsets": off.astype(C), "length": n,
                        "nextparents_length": max(E - trim, 0)})
    elif fam == "awkward_ListOffsetArray_local_preparenext_64":
        for n in (0, 1, 300):
            out.append({"tocarry": np.full(n, S, np.int64),
                        "fromindex": rng.permutation(3 * n)[:n].astype(np.int64), "length": n})
    elif fam == "awkward_RegularArray_reduce_local_nextparents_64":
        for size, length in ((0, 5), (3, 0), (4, 37), (1, 10)):
            out.append({"nextparents": np.full(size * length, S, np.int64), "size": size, "length": length})
    elif fam == "awkward_RegularArray_reduce_nonlocal_preparenext_64":
        for nbins, size in ((0, 3), (1, 4), (20, 3), (15, 0), (9, 1)):
            R = rng.poisson(3, nbins).astype(np.int64)
            R[rng.random(nbins) < 0.15] = 0
            off = _offsets(R)
            rows = int(off[-1])
            out.append({"nextcarry": np.full(rows * size, S, np.int64),
                        "nextoffsets": np.full(nbins * size + 1, S, np.int64), "offsets": off,
                        "size": size, "length": rows, "outlength": nbins})
    elif fam == "awkward_IndexedArray_reduce_next_64":
        T = NP_DTYPES[args["index"][1]]
        for nbins in (0, 1, 60):
            off = _offsets(_lengths(rng, nbins, 4, p_empty=0.15, longs=(40,)))
            E = int(off[-1])
            idx = rng.integers(0, 1000, E)
            if T != np.uint32:
                idx[rng.random(E) < 0.25] = -1
            out.append({"nextcarry": np.full(E, S, np.int64), "nextoffsets": np.full(nbins + 1, S, np.int64),
                        "outindex": np.full(E, S, np.int64), "index": idx.astype(T), "offsets": off,
                        "outlength": nbins})
    elif fam == "awkward_IndexedArray_reduce_next_fix_offsets_64":
        for n in (0, 1, 50):
            st = np.sort(rng.integers(0, 500, n)).astype(np.int64)
            out.append({"outoffsets": np.full(n + 1, S, np.int64), "starts": st, "startslength": n,
                        "outindexlength": 500 + n})
    elif fam in ("awkward_IndexedArray_reduce_next_nonlocal_nextshifts_64",
                 "awkward_IndexedArray_reduce_next_nonlocal_nextshifts_fromshifts_64"):
        T = NP_DTYPES[args["index"][1]]
        for n in (0, 1, 400):
            idx = rng.integers(0, 1000, n)
            if T != np.uint32:
                idx[rng.random(n) < 0.3] = -1
            kw = {"nextshifts": np.full(n, S, np.int64), "index": idx.astype(T), "length": n}
            if "shifts" in args:
                kw["shifts"] = rng.integers(0, 20, n).astype(np.int64)
            out.append(kw)
    elif fam == "awkward_IndexedArray_local_preparenext_64":
        for nbins in (0, 1, 70):
            Lo = _lengths(rng, nbins, 4, p_empty=0.15, longs=(40,))
            off = _offsets(Lo)
            Li = np.array([rng.integers(0, x + 1) for x in Lo], np.int64)
            out.append({"tocarry": np.full(int(off[-1]), S, np.int64), "starts": off[:-1].copy(),
                        "offsets": off, "nextoffsets": _offsets(Li), "outlength": nbins})
    elif fam == "awkward_ByteMaskedArray_reduce_next_64":
        for nbins, vw in ((0, True), (1, False), (60, True), (45, False)):
            off = _offsets(_lengths(rng, nbins, 4, p_empty=0.15, longs=(40,)))
            E = int(off[-1])
            m = (rng.random(E) < 0.6).astype(np.int8) * rng.integers(1, 5, E).astype(np.int8)
            out.append({"nextcarry": np.full(E, S, np.int64), "nextoffsets": np.full(nbins + 1, S, np.int64),
                        "outindex": np.full(E, S, np.int64), "mask": m, "offsets": off,
                        "outlength": nbins, "validwhen": vw})
    elif fam in ("awkward_ByteMaskedArray_reduce_next_nonlocal_nextshifts_64",
                 "awkward_ByteMaskedArray_reduce_next_nonlocal_nextshifts_fromshifts_64"):
        for n, vw in ((0, True), (1, True), (300, True), (300, False)):
            m = (rng.random(n) < 0.6).astype(np.int8)
            kw = {"nextshifts": np.full(n, S, np.int64), "mask": m, "length": n, "valid_when": vw}
            if "shifts" in args:
                kw["shifts"] = rng.integers(0, 20, n).astype(np.int64)
            out.append(kw)
    else:
        raise KeyError(fam)
    return out


def complex_cases(rng, name):
    """Seeded inputs of the complex reducers: interleaved (re, im) values with
    ties, signed zeros, infinities and NaN in either part (some lists start
    with a NaN real part), lists up to 1025 elements."""
    rec = SIGNATURES[name]
    args = {a[0]: a for a in rec["args"]}
    base = args["fromptr"][1]
    dt = NP_DTYPES[base]
    out = []
    for lam, nan_rate in ((4, 0.0), (4, 0.08), (2, 0.3)):
        L = _lengths(rng, 250, lam)
        off = _offsets(L)
        E = int(off[-1])
        v = np.round(rng.standard_normal((E, 2)), 1).astype(dt)  # ties in both parts
        k = rng.random((E, 2))
        v[k < nan_rate] = np.nan
        v[(k >= 0.5) & (k < 0.53)] = 0.0
        v[(k >= 0.53) & (k < 0.55)] = -0.0
        v[(k >= 0.55) & (k < 0.56)] = np.inf
        v[(k >= 0.56) & (k < 0.57)] = -np.inf
        if nan_rate:
            first = off[:-1][(L > 0) & (rng.random(len(L)) < 0.1)]
            v[first, 0] = np.nan
        kw = {"fromptr": v.reshape(-1), "offsets": off, "outlength": len(L)}
        out_t = args["toptr"][1]
        width = 2 if out_t in ("float", "double") else 1
        kw["toptr"] = np.full(width * len(L), 123, NP_DTYPES[out_t])
        if "identity" in args:
            kw["identity"] = float(-np.inf if "max" in name else np.inf)
        out.append(kw)
    return out


def layout_cases(rng, name):
    """Seeded inputs of compact_offsets and the RegularArray carries."""
    rec = SIGNATURES[name]
    fam = rec["family"]
    args = {a[0]: a for a in rec["args"]}
    S = 777
    out = []
    if fam == "awkward_ListArray_compact_offsets":
        C = NP_DTYPES[args["fromstarts"][1]]
        for n, bad in ((0, False), (1, False), (300, False), (120, True)):
            L = _lengths(rng, n, 5, longs=(40,))
            starts = rng.integers(0, 1000, n)
            stops = starts + L
            if bad and n:
                stops[n // 2] = starts[n // 2] - 1 if starts[n // 2] > 0 else starts[n // 2]
                if stops[n // 2] == starts[n // 2]:
                    starts[n // 2] += 1
            out.append({"tooffsets": np.full(n + 1, S, np.int64), "fromstarts": starts.astype(C),
                        "fromstops": stops.astype(C), "length": n})
    elif fam == "awkward_RegularArray_getitem_carry":
        for lencarry, size in ((0, 3), (5, 0), (200, 4), (37, 1)):
            out.append({"tocarry": np.full(lencarry * size, S, np.int64),
                        "fromcarry": rng.integers(0, 500, lencarry).astype(np.int64),
                        "lencarry": lencarry, "size": size})
    elif fam == "awkward_RegularArray_localindex":
        for size, length in ((0, 5), (3, 0), (5, 70), (1, 9)):
            out.append({"toindex": np.full(size * length, S, np.int64), "size": size,
                        "length": length})
    else:
        raise KeyError(fam)
    return out


def sibling_cases(rng, name):
    """Seeded inputs of the small siblings (adjust_starts_shifts, localindex,
    range counts / spreads, missing-value jagged helpers)."""
    rec = SIGNATURES[name]
    fam = rec["family"]
    args = {a[0]: a for a in rec["args"]}
    S = 777
    out = []
    if fam == "awkward_NumpyArray_reduce_adjust_starts_shifts_64":
        for n in (0, 1, 200):
            starts = np.sort(rng.integers(0, 500, n)).astype(np.int64)
            toptr = np.where(rng.random(n) < 0.2, -1, starts + rng.integers(0, 5, n)).astype(np.int64)
            out.append({"toptr": toptr, "outlength": n, "offsets": np.zeros(n + 1, np.int64),
                        "starts": starts, "shifts": rng.integers(0, 9, 600).astype(np.int64)})
    elif fam == "awkward_localindex":
        for n in (0, 1, 300):
            out.append({"toindex": np.full(n, S, np.int64), "length": n})
    elif fam == "awkward_ListArray_getitem_next_range_counts":
        C = NP_DTYPES[args["fromoffsets"][1]]
        for n in (0, 1, 150):
            off = _offsets(_lengths(rng, n, 4, longs=(40,))) + 3
            out.append({"total": np.full(1, S, np.int64), "fromoffsets": off.astype(C),
                        "lenstarts": n})
    elif fam == "awkward_ListArray_getitem_next_range_spreadadvanced":
        C = NP_DTYPES[args["fromoffsets"][1]]
        for n in (0, 1, 150):
            off = _offsets(_lengths(rng, n, 4, longs=(40,)))
            out.append({"toadvanced": np.full(int(off[-1]), S, np.int64),
                        "fromadvanced": rng.integers(0, 1000, n).astype(np.int64),
                        "fromoffsets": off.astype(C), "lenstarts": n})
    elif fam == "awkward_RegularArray_getitem_next_range_spreadadvanced":
        for length, size in ((0, 3), (4, 0), (90, 5), (30, 1)):
            out.append({"toadvanced": np.full(length * size, S, np.int64),
                        "fromadvanced": rng.integers(0, 1000, length).astype(np.int64),
                        "length": length, "nextsize": size})
    elif fam == "awkward_Content_getitem_next_missing_jagged_getmaskstartstop":
        for n in (0, 1, 250):
            idx = np.where(rng.random(n) < 0.3, -1, np.arange(n)).astype(np.int64)
            valid = int((idx >= 0).sum())
            offs = _offsets(_lengths(rng, valid, 3))
            out.append({"index_in": idx, "offsets_in": offs, "mask_out": np.full(n, S, np.int64),
                        "starts_out": np.full(n, S, np.int64), "stops_out": np.full(n, S, np.int64),
                        "length": n})
    elif fam == "awkward_MaskedArray_getitem_next_jagged_project":
        T = NP_DTYPES[args["index"][1]]
        for n in (0, 1, 250):
            idx = rng.integers(0, 1000, n)
            if T != np.uint32:
                idx[rng.random(n) < 0.3] = -1
            st = rng.integers(0, 500, n).astype(np.int64)
            out.append({"index": idx.astype(T), "starts_in": st, "stops_in": st + rng.integers(0, 9, n),
                        "starts_out": np.full(n, S, np.int64), "stops_out": np.full(n, S, np.int64),
                        "length": n})
    else:
        raise KeyError(fam)
    return out


SIBLING_FAMILIES = (
    "awkward_NumpyArray_reduce_adjust_starts_shifts_64", "awkward_localindex",
    "awkward_ListArray_getitem_next_range_counts",
    "awkward_ListArray_getitem_next_range_spreadadvanced",
    "awkward_RegularArray_getitem_next_range_spreadadvanced",
    "awkward_Content_getitem_next_missing_jagged_getmaskstartstop",
    "awkward_MaskedArray_getitem_next_jagged_project")


LAYOUT_FAMILIES = ("awkward_ListArray_compact_offsets", "awkward_RegularArray_getitem_carry",
                   "awkward_RegularArray_localindex")


NONLOCAL_PREFIXES = ("awkward_ListOffsetArray_reduce_", "awkward_ListOffsetArray_local_",
                     "awkward_RegularArray_reduce_", "awkward_IndexedArray_",
                     "awkward_ByteMaskedArray_")


def make_random():
    ref = oracle.load_ref()
    ref = oracle.load_ref()
    if ref is None:
        raise SystemExit("awkward-cpp CPU kernels not built (oracle/build.py)")
    manifest = []
    arrays = {}
    for name, rec in SIGNATURES.items():
        fam = rec["family"]
        # one generator per specialization: adding a family leaves the others' cases unchanged
        rng = np.random.default_rng([20241203, zlib.crc32(name.encode())])
        if fam in ("awkward_argsort", "awkward_sort"):
            cases = sort_cases(rng, name)
        elif fam.startswith("awkward_reduce") and fam.endswith("_complex"):
            cases = complex_cases(rng, name)
        elif fam in LAYOUT_FAMILIES:
            cases = layout_cases(rng, name)
        elif fam in SIBLING_FAMILIES:
            cases = sibling_cases(rng, name)
        elif fam.startswith(NONLOCAL_PREFIXES):
            cases = nonlocal_cases(rng, name)
        elif fam == "awkward_RegularArray_combinations_64":
            cases = regular_combinations_cases(rng, name)
        elif fam == "awkward_ListArray_broadcast_tooffsets":
            cases = broadcast_cases(rng, name)
        elif fam.startswith(("awkward_reduce", "awkward_NumpyArray_reduce")):
            cases = [reducer_case(rng, name)]
        elif "next_range" in fam:
            cases = range_cases(rng, name)
        elif "combinations" in fam:
            cases = combinations_cases(rng, name)
        else:
            cases = [jagged_case(rng, name)]
        for kw in cases:
            inputs = {k: (v.copy() if isinstance(v, np.ndarray) else [r.copy() for r in v] if isinstance(v, list) else v)
                      for k, v in kw.items()}
            err = oracle.call(ref, name, **kw)
            i = len(manifest)
            entry = {"name": name, "scalars": {}, "arrays": [], "lists": {}, "outs": [], "error": err[0],
                     "identity": int(err[1]), "attempt": int(err[2])}
            for (an, base, d, depth, _c, _r) in rec["args"]:
                v = inputs[an]
                if depth == 0:
                    entry["scalars"][an] = v if not isinstance(v, (np.generic,)) else v.item()
                elif depth == 1:
                    arrays[f"{i}:in:{an}"] = v
                    entry["arrays"].append(an)
                    if d == "out":
                        arrays[f"{i}:out:{an}"] = kw[an]
                        entry["outs"].append(an)
                else:
                    entry["lists"][an] = len(v)
                    for r, row in enumerate(v):
                        arrays[f"{i}:in:{an}:{r}"] = row
                        arrays[f"{i}:out:{an}:{r}"] = kw[an][r]
                    entry["outs"].append(an)
            manifest.append(entry)
    arrays["manifest"] = np.frombuffer(json.dumps(manifest).encode(), dtype=np.uint8)
    np.savez_compressed(os.path.join(HERE, "ref_random.npz"), **arrays)
    return len(manifest)


if __name__ == "__main__":
    src = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("AWKWARD_SRC", "/root/reference")
    from oracle import build

    build.build_oracle()
    build.build_ref(src)
    print("unit tests:", extract_unit_tests(src))
    print("random cases:", make_random())
