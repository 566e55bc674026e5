"""CPU oracle for the GB300 jagged hot path -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this package; the product (``awkward_gb300``) never does.

``load()`` returns the plain-C restatement (``awkward_oracle.c``);
``load_ref()`` returns awkward-cpp's own CPU kernels when they were built
from the reference sources (None otherwise).  ``call()`` runs one
specialization on numpy arrays, in place, following the argument table in
``awkward_gb300/_signatures.py``, and returns the kernel's ``struct Error``
as ``(message or None, identity, attempt)``.
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


def parallel_reduce(name, toptr, fromptr, offsets, outlength, nthreads):
    """Run a reducer of the restatement over ``nthreads`` list ranges (pthreads)."""
    lib = load()
    f = getattr(lib, name)
    kind = 5 if ("argmax" in name or "argmin" in name) else 4
    drv = lib.oracle_parallel_reduce
    drv.restype = ctypes.c_int
    drv.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t,
                    ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int]
    rc = drv(ctypes.cast(f, ctypes.c_void_p), kind, toptr.ctypes.data, toptr.itemsize,
             fromptr.ctypes.data, offsets.ctypes.data, outlength, nthreads)
    if rc != 0:
        raise RuntimeError("oracle_parallel_reduce failed")
