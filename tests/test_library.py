"""CPU-side checks of the C ABI: the library builds for sm_103a, loads, and exports every declaration."""

import re

import numpy as np

import awkward_gb300
from awkward_gb300 import _abi
from awkward_gb300._signatures import SIGNATURES
from awkward_gb300.kernel_table import GB300Backend, kernel_key


from awkward_gb300._extensions import EXTENSIONS

# Entry points without a kernel-specification.yml counterpart.
EXTRA = set(EXTENSIONS)


def _header_names():
    import os

    here = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    txt = open(os.path.join(here, "include", "awkward_gb300.h")).read()
    return re.findall(r"^int (\w+)\(", txt, flags=re.M)


def test_header_matches_signature_table():
    assert sorted(_header_names()) == sorted(set(SIGNATURES) | EXTRA)


def test_library_builds_loads_and_exports_every_declaration():
    awkward_gb300.build()
    lib = _abi.load_library()
    missing = [n for n in _header_names() if not hasattr(lib, n)]
    assert not missing, missing
    assert "sm_103a" in _abi.version()
    for n in SIGNATURES:  # argtypes resolve for every entry point
        _abi.cfunc(n)
    for n in EXTENSIONS:
        _abi.ext_cfunc(n)


def test_kernel_keys_follow_awkward_scheme():
    be = GB300Backend()
    k = ("awkward_reduce_sum", np.float64, np.float64, np.int64)
    assert k in be
    assert kernel_key("awkward_reduce_argmax_float64_64") == (
        "awkward_reduce_argmax", np.int64, np.float64, np.int64, np.int64)
    assert kernel_key("awkward_ListArray64_combinations_64")[:2] == (
        "awkward_ListArray_combinations", np.int64)
    # one key per specialization
    assert len(set(be.keys())) == len(SIGNATURES)
