"""GB300-native kernels for Awkward Array's jagged hot path.

``libawkward_gb300.so`` (CUDA, sm_103a) implements awkward's segmented
reducers over ListOffsetArray offsets, the jagged getitem kernels and the
carries they feed, range slices on lists and ListArray combinations, under
the names and argument lists of awkward's kernel-specification.yml.

Entry points for Python callers:

* ``backend()`` -- the kernel table ``backend[(family, *dtypes)]`` over torch
  CUDA tensors, with awkward's error protocol (see ``kernel_table.py``);
* ``cupy_adapter.install()`` -- registers the same kernels in awkward's own
  cupy kernel table;
* ``build()`` -- compiles the library in-tree with nvcc.
"""

from __future__ import annotations

from ._abi import LibraryNotBuilt, load_library, version  # noqa: F401
from ._signatures import SIGNATURES  # noqa: F401


def build(force=False, verbose=False):
    """Compile libawkward_gb300.so in-tree (nvcc, sm_103a) and return its path."""
    from . import _build

    return _build.build(force=force, verbose=verbose)


def backend():
    """The process-wide kernel table over torch CUDA tensors."""
    from .kernel_table import backend as _backend

    return _backend()
