"""ctypes binding of libawkward_gb300.so (the C ABI declared in include/awkward_gb300.h).

Every entry point takes the kernel-specification.yml arguments in spec order
(pointers are device addresses, passed as integers) followed by
``(invocation_index, err_code, stream)`` and returns the launch's
``cudaError_t``.  There is no fallback: if the library has not been built,
``load_library()`` raises.
"""

from __future__ import annotations

import ctypes
import os
import threading

from ._signatures import SIGNATURES

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libawkward_gb300.so")

_SCALAR_CTYPES = {
    "bool": ctypes.c_bool, "int8_t": ctypes.c_int8, "uint8_t": ctypes.c_uint8,
    "int16_t": ctypes.c_int16, "uint16_t": ctypes.c_uint16, "int32_t": ctypes.c_int32,
    "uint32_t": ctypes.c_uint32, "int64_t": ctypes.c_int64, "uint64_t": ctypes.c_uint64,
    "float": ctypes.c_float, "double": ctypes.c_double,
}

_lock = threading.Lock()
_lib = None
_funcs = {}


class LibraryNotBuilt(RuntimeError):
    pass


def load_library():
    """Load (once) and return the CDLL; raises if the CUDA library is missing."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise LibraryNotBuilt(
                    f"{LIB_PATH} is missing: build it with "
                    "`python -c 'import awkward_gb300; awkward_gb300.build()'` (needs nvcc)")
            _lib = ctypes.CDLL(LIB_PATH)
            _lib.awkward_gb300_version.restype = ctypes.c_char_p
        return _lib


def version():
    return load_library().awkward_gb300_version().decode()


def argtypes_of(name):
    out = []
    for (_an, base, _d, depth, _c, _r) in SIGNATURES[name]["args"]:
        out.append(ctypes.c_void_p if depth else _SCALAR_CTYPES[base])
    return out + [ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p]


def cfunc(name):
    """The typed ctypes function for one specialization."""
    f = _funcs.get(name)
    if f is None:
        lib = load_library()
        f = getattr(lib, name)
        f.argtypes = argtypes_of(name)
        f.restype = ctypes.c_int
        _funcs[name] = f
    return f


_EXT_CTYPES = {"int64_t": ctypes.c_int64, "uint64_t": ctypes.c_uint64, "int32_t": ctypes.c_int32,
               "uint32_t": ctypes.c_uint32}


def ext_cfunc(name):
    """The typed ctypes function of one extension entry point (_extensions.py)."""
    from ._extensions import EXTENSIONS

    f = _funcs.get(name)
    if f is None:
        lib = load_library()
        f = getattr(lib, name)
        args, _group = EXTENSIONS[name]
        f.argtypes = [ctypes.c_void_p if t.endswith("*") else _EXT_CTYPES[t] for t, _a in args]
        f.restype = ctypes.c_int
        _funcs[name] = f
    return f


def exported_symbols():
    """Names declared in include/awkward_gb300.h that the loaded library exports."""
    lib = load_library()
    return [n for n in SIGNATURES if hasattr(lib, n)]
