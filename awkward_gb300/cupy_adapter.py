"""Install libawkward_gb300 into awkward's own CUDA (cupy) kernel table.

awkward's cupy backend looks kernels up in ``awkward._connect.cuda.kernel``,
a dict keyed by ``(family, *pointer-argument dtypes)`` whose values are
called as ``f(grid, block, args)`` with
``args = (*spec_args, invocation_index, err_code)`` by ``CupyKernel.__call__``
(src/awkward/_kernels.py:185-232; the wrapper shape with ``.dir`` and
``.is_ptr`` is dev/generate-kernel-signatures.py:443-476).  A non-None entry
takes precedence over the cuda.compute fallback
(src/awkward/_backends/cupy.py:30-57), so replacing the entries of the hot
path families routes ``ak.sum/max/argmax``, jagged getitem and
``ak.combinations`` on cupy arrays through this library.

Each adapted entry ignores ``grid`` and ``block`` (the library sizes its own
launches), reads device addresses from the cupy arguments (``List[List[T]]``
arrives as awkward's device array of row pointers, passed through
unchanged), and launches on cupy's current stream.  Error codes follow the
``// message:`` order of awkward's CUDA kernel of the same family, so the
table ``kernel_errors`` keeps working; the library's own "bounded wait gave
up" code (32) is appended to each family's message list.
"""

from __future__ import annotations

from . import _abi
from ._messages import TIMEOUT_CODE, messages
from ._signatures import SIGNATURES
from .kernel_table import kernel_key


class CudaLaunchError(RuntimeError):
    """A launch through the C ABI returned a non-zero cudaError_t."""


def _address(x):
    """Device address of a cupy array (or an integer address)."""
    if isinstance(x, int):
        return x
    data = getattr(x, "data", None)
    if data is not None and hasattr(data, "ptr"):
        return int(data.ptr)
    ptr = getattr(x, "ptr", None)
    if ptr is not None:
        return int(ptr)
    raise TypeError(f"expected a device array, got {type(x).__name__}")


def _scalar(x):
    return x.item() if hasattr(x, "item") else x


class AdaptedKernel:
    """``f(grid, block, args)`` wrapper of one specialization of the C ABI."""

    def __init__(self, name, cfunc, current_stream_ptr):
        rec = SIGNATURES[name]
        self.name = name
        self.dir = [a[2] for a in rec["args"]]
        self.is_ptr = [a[3] > 0 for a in rec["args"]]
        self._f = cfunc
        self._stream = current_stream_ptr

    def __repr__(self):
        return f"<awkward_gb300 {self.name}>"

    def __call__(self, grid, block, args):
        del grid, block
        *spec, invocation_index, err_code = args
        if len(spec) != len(self.is_ptr):
            raise TypeError(f"{self.name}: expected {len(self.is_ptr)} arguments, got {len(spec)}")
        cargs = [_address(v) if p else _scalar(v) for v, p in zip(spec, self.is_ptr)]
        rc = self._f(*cargs, int(invocation_index), _address(err_code), self._stream())
        if rc != 0:
            raise CudaLaunchError(f"{self.name}: launch failed with cudaError {rc}")


def _cupy_stream_ptr():
    import cupy

    return cupy.cuda.get_current_stream().ptr


def adapted_kernels(cfunc=None, current_stream_ptr=None):
    """``{key: AdaptedKernel}`` for every specialization of the library."""
    cfunc = cfunc or _abi.cfunc
    current_stream_ptr = current_stream_ptr or _cupy_stream_ptr
    return {kernel_key(n): AdaptedKernel(n, cfunc(n), current_stream_ptr) for n in SIGNATURES}


def install(kernel_table=None, kernel_errors=None, cfunc=None, current_stream_ptr=None):
    """Replace awkward's CUDA kernels of the hot-path families with this library's.

    With no arguments this initialises awkward's table
    (``awkward._connect.cuda.initialize_cuda_kernels``) and edits it and
    ``awkward._connect.cuda.kernel_errors`` in place.  The arguments let a
    caller (or a test) pass the two dicts, the ctypes function factory and the
    current-stream getter explicitly.  Returns the installed keys.
    """
    if kernel_table is None or kernel_errors is None:
        import awkward._connect.cuda as ak_cuda

        cupy = ak_cuda.import_cupy("awkward_gb300")
        if kernel_table is None:
            kernel_table = ak_cuda.initialize_cuda_kernels(cupy)
        if kernel_errors is None:
            kernel_errors = ak_cuda.kernel_errors
    table = adapted_kernels(cfunc, current_stream_ptr)
    for key, fn in table.items():
        kernel_table[key] = fn
    for fam in {k[0] for k in table}:
        msgs = messages(fam)
        assert len(msgs) == TIMEOUT_CODE + 1
        kernel_errors[fam] = msgs
    return sorted(table, key=lambda k: (k[0], [t.__name__ for t in k[1:]]))
