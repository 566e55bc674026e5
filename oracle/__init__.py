"""CPU oracle for the GB300 jagged hot path -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this package; the product (``awkward_gb300``) never does.

``load()`` returns the plain-C restatement (``awkward_oracle.c``);
``load_ref()`` returns awkward-cpp's own CPU kernels when they were built
from the reference sources (None otherwise).  ``call()`` runs one
specialization on numpy arrays, in place, following the argument table in
``awkward_gb300/_signatures.py``, and returns the kernel's ``struct Error``
as ``(message or None, identity, attempt)``.  ``compensated_sum()`` and
``sum_error_report()`` give the FP64 compensated per-list sums that float sums
are judged against, and the error figures of a float-sum result.
"""

from __future__ import annotations

import ctypes
import os

import numpy as np

from awkward_gb300._signatures import SIGNATURES

from . import build as _build

_CTYPES = {
    "bool": ctypes.c_bool, "int8_t": ctypes.c_int8, "uint8_t": ctypes.c_uint8,
    "int16_t": ctypes.c_int16, "uint16_t": ctypes.c_uint16, "int32_t": ctypes.c_int32,
    "uint32_t": ctypes.c_uint32, "int64_t": ctypes.c_int64, "uint64_t": ctypes.c_uint64,
    "float": ctypes.c_float, "double": ctypes.c_double,
}
NP_DTYPES = {
    "bool": np.bool_, "int8_t": np.int8, "uint8_t": np.uint8, "int16_t": np.int16,
    "uint16_t": np.uint16, "int32_t": np.int32, "uint32_t": np.uint32,
    "int64_t": np.int64, "uint64_t": np.uint64, "float": np.float32, "double": np.float64,
}


class Error(ctypes.Structure):
    _fields_ = [("str", ctypes.c_char_p), ("filename", ctypes.c_char_p),
                ("identity", ctypes.c_int64), ("attempt", ctypes.c_int64)]


_LIBS = {}


def load():
    if "oracle" not in _LIBS:
        _LIBS["oracle"] = ctypes.CDLL(_build.build_oracle())
    return _LIBS["oracle"]


def load_ref():
    if "ref" not in _LIBS:
        path = _build.REF_SO if os.path.exists(_build.REF_SO) else _build.build_ref()
        _LIBS["ref"] = ctypes.CDLL(path) if path else None
    return _LIBS["ref"]


def _fn(lib, name):
    f = getattr(lib, name)
    if getattr(f, "_gb_ready", False):
        return f
    argtypes = []
    for (_an, base, _d, depth, _c, _r) in SIGNATURES[name]["args"]:
        t = _CTYPES[base]
        for _ in range(depth):
            t = ctypes.POINTER(t)
        argtypes.append(t)
    f.argtypes = argtypes
    f.restype = Error
    f._gb_ready = True
    return f


def call(lib, name, **kwargs):
    """Run ``name`` from ``lib`` on numpy arrays (modified in place).

    List arguments must be C-contiguous numpy arrays of the spec dtype;
    List[List[T]] arguments are sequences of such arrays.  Returns
    ``(message or None, identity, attempt)``.
    """
    f = _fn(lib, name)
    cargs = []
    keep = []
    for (an, base, _d, depth, _c, _r) in SIGNATURES[name]["args"]:
        v = kwargs[an]
        ct = _CTYPES[base]
        if depth == 0:
            cargs.append(ct(v))
        elif depth == 1:
            assert isinstance(v, np.ndarray) and v.dtype == NP_DTYPES[base], (an, getattr(v, "dtype", None))
            assert v.flags.c_contiguous
            cargs.append(v.ctypes.data_as(ctypes.POINTER(ct)))
        else:
            rows = (ctypes.POINTER(ct) * max(len(v), 1))()
            for i, row in enumerate(v):
                assert row.dtype == NP_DTYPES[base] and row.flags.c_contiguous
                rows[i] = row.ctypes.data_as(ctypes.POINTER(ct))
            keep.append(rows)
            cargs.append(ctypes.cast(rows, ctypes.POINTER(ctypes.POINTER(ct))))
    err = f(*cargs)
    msg = err.str.decode() if err.str else None
    return msg, err.identity, err.attempt


def parallel_reduce(name, toptr, fromptr, offsets, outlength, nthreads, identity=None):
    """Run a reducer of the restatement over ``nthreads`` list ranges (pthreads).

    ``identity`` is the float64 max/min identity argument (those reducers
    take it after ``outlength``); the arg-reducers take ``starts``, unused.
    """
    lib = load()
    f = getattr(lib, name)
    if "argmax" in name or "argmin" in name:
        kind = 5
    elif "_max_" in name or "_min_" in name:
        if identity is None or "float64_float64" not in name:
            raise ValueError("max/min: float64 content with an identity only")
        kind = 6
    else:
        kind = 4
    drv = lib.oracle_parallel_reduce_ident
    drv.restype = ctypes.c_int
    drv.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t,
                    ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int,
                    ctypes.c_double]
    rc = drv(ctypes.cast(f, ctypes.c_void_p), kind, toptr.ctypes.data, toptr.itemsize,
             fromptr.ctypes.data, offsets.ctypes.data, outlength, nthreads,
             0.0 if identity is None else float(identity))
    if rc != 0:
        raise RuntimeError("oracle_parallel_reduce failed")


def compensated_sum(fromptr, offsets, nthreads=None):
    """Per-list FP64 compensated sums and sum|x| (float64 or float32 content).

    Double-double accumulation (TwoSum) in the C restatement, split over
    ``nthreads`` list ranges; returns ``(sums, abs_sums)`` as float64 arrays.
    """
    fromptr = np.ascontiguousarray(fromptr)
    offsets = np.ascontiguousarray(offsets, dtype=np.int64)
    n = len(offsets) - 1
    out = np.zeros((max(n, 0), 2), np.float64)
    if n <= 0:
        return out[:, 0], out[:, 1]
    kind = {np.dtype(np.float64): "float64", np.dtype(np.float32): "float32"}[fromptr.dtype]
    lib = load()
    f = getattr(lib, f"oracle_sum_compensated_{kind}")
    drv = lib.oracle_parallel_reduce
    drv.restype = ctypes.c_int
    drv.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t,
                    ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int]
    threads = nthreads or min(os.cpu_count() or 1, max(1, n // 100_000))
    if drv(ctypes.cast(f, ctypes.c_void_p), 4, out.ctypes.data, 16, fromptr.ctypes.data,
           offsets.ctypes.data, n, threads) != 0:
        raise RuntimeError("oracle_parallel_reduce failed")
    return out[:, 0].copy(), out[:, 1].copy()


def sum_error_report(got, fromptr, offsets, eps=None, nthreads=None):
    """Error figures of per-list float sums ``got`` against the compensated oracle.

    Per list with finite oracle sum: err = |got - comp|; ``ratio`` =
    err / (n * eps * sum|x|) (the bound's unit; a list with sum|x| = 0 must
    have err = 0) and ``rel`` = err / |comp| where comp != 0.  Non-finite
    oracle sums must be matched exactly (NaN by NaN, infinities by sign).
    Returns a dict: lists, max/p99 of ratio and rel, the index of the worst
    list, ``within`` (every ratio <= 4, i.e. err <= 4*n*eps*sum|x|) and
    ``nonfinite_ok``.
    """
    got = np.asarray(got, dtype=np.float64)
    comp, absum = compensated_sum(fromptr, offsets, nthreads)
    if eps is None:
        eps = float(np.finfo(np.float64).eps)
    n = np.diff(np.asarray(offsets, dtype=np.int64)).astype(np.float64)
    fin = np.isfinite(comp)
    nonfinite_ok = bool(np.array_equal(np.isnan(got), np.isnan(comp)) and
                        np.array_equal(got[np.isinf(comp)], comp[np.isinf(comp)]))
    err = np.abs(got[fin] - comp[fin])
    unit = np.maximum(n[fin], 1) * eps * absum[fin]
    with np.errstate(divide="ignore", invalid="ignore"):
        ratio = np.where(unit > 0, err / unit, np.where(err == 0, 0.0, np.inf))
        nz = comp[fin] != 0
        rel = err[nz] / np.abs(comp[fin][nz])
    worst = int(np.flatnonzero(fin)[np.argmax(ratio)]) if ratio.size else -1
    q = lambda a, p: float(np.quantile(a, p)) if a.size else 0.0
    return {"lists": int(len(got)), "max_ratio": float(ratio.max()) if ratio.size else 0.0,
            "p99_ratio": q(ratio, 0.99), "max_rel": float(rel.max()) if rel.size else 0.0,
            "p99_rel": q(rel, 0.99), "worst_list": worst,
            "within": bool(ratio.size == 0 or ratio.max() <= 4.0), "nonfinite_ok": nonfinite_ok}
