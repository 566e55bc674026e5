"""Kernel table over libawkward_gb300 with awkward's key scheme and error protocol.

This mirrors the part of awkward's CUDA backend that sits on the accelerated
path, for callers holding torch CUDA tensors (the cupy adapter in
``cupy_adapter.py`` installs the same entry points into awkward itself):

* ``backend[(family, *dtypes)]`` returns a kernel, keyed exactly like
  ``CupyBackend.__getitem__`` (src/awkward/_backends/cupy.py:30-57): the
  family name followed by the numpy dtype of every pointer argument in spec
  order (dev/generate-kernel-signatures.py:225-236, 419-422);
* calling the kernel with the spec's arguments launches it asynchronously on
  the current torch stream, appending ``(invocation_index, err_code)`` like
  ``CupyKernel.__call__`` (src/awkward/_kernels.py:185-232);
* ``backend.synchronize()`` waits for the stream and raises
  ``ValueError("<message> in compiled CUDA code (<family>)")`` for the first
  failing invocation, like ``synchronize_cuda``
  (src/awkward/_connect/cuda/__init__.py:257-294).

Arguments: List[T] -> a contiguous CUDA tensor of dtype T (bool as
torch.bool); List[List[T]] -> a sequence of such tensors; scalars -> Python
numbers.

Fault injection (host side, for testing callers' error handling): with
``AWKWARD_GB300_FAULT="<specialization or family>:<code>"`` every call of a
matching kernel still launches, and then the stream's error word records
``invocation_index * 256 + code`` exactly as a failing kernel would, so the
next ``synchronize()`` raises that code's message (code 32: the library's
"bounded wait gave up").  No kernel is made to fail on the GPU.
"""

from __future__ import annotations

import collections
import os

import numpy as np
import torch

from . import _abi
from ._messages import messages
from ._signatures import SIGNATURES

ERROR_BITS = 8
NO_ERROR = (1 << 64) - 1
MAX_PENDING_INVOCATIONS = 8192

NP_OF_C = {
    "bool": np.bool_, "int8_t": np.int8, "uint8_t": np.uint8, "int16_t": np.int16,
    "uint16_t": np.uint16, "int32_t": np.int32, "uint32_t": np.uint32,
    "int64_t": np.int64, "uint64_t": np.uint64, "float": np.float32, "double": np.float64,
}
TORCH_OF_C = {
    "bool": torch.bool, "int8_t": torch.int8, "uint8_t": torch.uint8, "int16_t": torch.int16,
    "uint16_t": torch.uint16, "int32_t": torch.int32, "uint32_t": torch.uint32,
    "int64_t": torch.int64, "uint64_t": torch.uint64, "float": torch.float32,
    "double": torch.float64,
}


def kernel_key(name):
    """(family, *numpy dtype types of the pointer arguments) of a specialization."""
    rec = SIGNATURES[name]
    return (rec["family"],) + tuple(NP_OF_C[a[1]] for a in rec["args"] if a[3] > 0)


FAULT_ENV = "AWKWARD_GB300_FAULT"


def injected_fault(name, family, env=None):
    """The error code AWKWARD_GB300_FAULT forces on kernel ``name``, or None.

    The variable holds ``<specialization or family>:<code>`` with code in
    0..255; anything else is ignored.
    """
    spec = (os.environ if env is None else env).get(FAULT_ENV, "")
    target, sep, code = spec.rpartition(":")
    if not sep or target not in (name, family):
        return None
    try:
        c = int(code)
    except ValueError:
        return None
    return c if 0 <= c < (1 << ERROR_BITS) else None


class _Invocation:
    __slots__ = ("name", "keepalive")

    def __init__(self, name, keepalive):
        self.name = name
        self.keepalive = keepalive


class _StreamContext:
    """Error word and pending invocations of one stream."""

    def __init__(self, device):
        self.err = torch.full((1,), -1, dtype=torch.int64, device=device)  # NO_ERROR
        self.pending = []

    def record_error(self, invocation, code, stream):
        """Lower the error word to invocation*256 + code on `stream` (as atomicMin does)."""
        word = invocation * (1 << ERROR_BITS) + code
        with torch.cuda.stream(stream):
            w = torch.full_like(self.err, word)
            self.err.copy_(torch.where((self.err < 0) | (self.err > w), w, self.err))


# Device arrays of row pointers (the int64_t** arguments), by device and
# addresses: uploading one is a blocking host-to-device copy, so a repeated
# call with the same rows reuses the array (it holds nothing but those
# addresses, so a cached array is right whatever tensors now live there).
_PTR_ARRAYS: collections.OrderedDict = collections.OrderedDict()
_PTR_ARRAYS_MAX = 256


def _pointer_array(dev, addresses):
    key = (dev.index, addresses)
    arr = _PTR_ARRAYS.get(key)
    if arr is None:
        arr = torch.tensor(list(addresses) or [0], dtype=torch.int64, device=dev)
        _PTR_ARRAYS[key] = arr
        if len(_PTR_ARRAYS) > _PTR_ARRAYS_MAX:
            _PTR_ARRAYS.popitem(last=False)
    else:
        _PTR_ARRAYS.move_to_end(key)
    return arr


class GB300Kernel:
    """One specialization, callable with the spec's arguments."""

    def __init__(self, backend, name):
        self.backend = backend
        self.name = name
        self.family = SIGNATURES[name]["family"]
        self.args = SIGNATURES[name]["args"]
        self.dir = [a[2] for a in self.args]
        self.is_ptr = [a[3] > 0 for a in self.args]
        self._f = _abi.cfunc(name)

    def __repr__(self):
        return f"<GB300Kernel {self.name}>"

    def _convert(self, args):
        cargs = []
        keep = []
        device = None
        for (an, base, _d, depth, _c, _r), v in zip(self.args, args, strict=True):
            if depth == 0:
                cargs.append(v.item() if hasattr(v, "item") else v)
                continue
            if depth == 1:
                t = v
                if not isinstance(t, torch.Tensor) or not t.is_cuda:
                    raise TypeError(f"{self.name}: argument {an} must be a CUDA tensor")
                if t.dtype != TORCH_OF_C[base]:
                    raise TypeError(f"{self.name}: argument {an} must have dtype "
                                    f"{TORCH_OF_C[base]}, not {t.dtype}")
                if not t.is_contiguous():
                    raise ValueError(f"{self.name}: argument {an} must be contiguous")
                device = t.device
                cargs.append(t.data_ptr())
                keep.append(t)
                continue
            rows = list(v)
            for t in rows:
                if not isinstance(t, torch.Tensor) or not t.is_cuda or t.dtype != TORCH_OF_C[base]:
                    raise TypeError(f"{self.name}: rows of {an} must be CUDA {TORCH_OF_C[base]} tensors")
                device = t.device
            dev = device if device is not None else torch.device("cuda", torch.cuda.current_device())
            ptrs = _pointer_array(dev, tuple(t.data_ptr() for t in rows))
            keep.extend(rows)
            keep.append(ptrs)
            cargs.append(ptrs.data_ptr())
        return cargs, keep, device

    def __call__(self, *args):
        cargs, keep, device = self._convert(args)
        if device is None:
            device = torch.device("cuda", torch.cuda.current_device())
        stream = torch.cuda.current_stream(device)
        ctx = self.backend._context(stream)
        if len(ctx.pending) >= MAX_PENDING_INVOCATIONS:
            self.backend.synchronize(stream)
            ctx = self.backend._context(stream)
        invocation = len(ctx.pending)
        ctx.pending.append(_Invocation(self.family, keep))
        rc = self._f(*cargs, invocation, ctx.err.data_ptr(), stream.cuda_stream)
        if rc != 0:
            raise RuntimeError(f"{self.name}: CUDA launch failed with cudaError {rc}")
        code = injected_fault(self.name, self.family)
        if code is not None:
            ctx.record_error(invocation, code, stream)


class GB300Backend:
    """Kernel table ``backend[(family, *dtypes)]`` over libawkward_gb300."""

    def __init__(self):
        self._by_key = {kernel_key(n): n for n in SIGNATURES}
        self._kernels = {}
        self._contexts = {}

    def keys(self):
        return list(self._by_key)

    def __contains__(self, key):
        return self._norm(key) in self._by_key

    @staticmethod
    def _norm(key):
        return (key[0],) + tuple(np.dtype(k).type for k in key[1:])

    def __getitem__(self, key):
        k = self._norm(key)
        name = self._by_key.get(k)
        if name is None:
            raise KeyError(f"no GB300 kernel for {key}")
        kern = self._kernels.get(name)
        if kern is None:
            kern = self._kernels[name] = GB300Kernel(self, name)
        return kern

    def by_name(self, name):
        return self[kernel_key(name)]

    def _context(self, stream):
        key = (stream.device, stream.cuda_stream)
        ctx = self._contexts.get(key)
        if ctx is None:
            ctx = self._contexts[key] = _StreamContext(stream.device)
        return ctx

    def selftest_lookback_timeout(self, spin_limit=1000):
        """Launch the look-back self-test (awkward_gb300_selftest_lookback_timeout)
        on the current stream as one more invocation: its wait on a tile that
        never publishes runs out after `spin_limit` polls, so the next
        synchronize() raises the "bounded wait gave up" ValueError."""
        stream = torch.cuda.current_stream()
        ctx = self._context(stream)
        invocation = len(ctx.pending)
        ctx.pending.append(_Invocation("awkward_gb300_selftest_lookback_timeout", []))
        rc = _abi.ext_cfunc("awkward_gb300_selftest_lookback_timeout")(
            int(spin_limit), invocation, ctx.err.data_ptr(), stream.cuda_stream)
        if rc != 0:
            raise RuntimeError(f"look-back self-test: CUDA launch failed with cudaError {rc}")

    def synchronize(self, stream=None):
        """Wait for the stream; raise ValueError for the first failed invocation."""
        if stream is None:
            stream = torch.cuda.current_stream()
        stream.synchronize()
        key = (stream.device, stream.cuda_stream)
        ctx = self._contexts.get(key)
        if ctx is None:
            return
        word = int(ctx.err.item()) & NO_ERROR
        pending = ctx.pending
        self._contexts[key] = _StreamContext(stream.device)
        if word == NO_ERROR:
            return
        inv = pending[word >> ERROR_BITS]
        code = word & ((1 << ERROR_BITS) - 1)
        raise ValueError(f"{messages(inv.name)[code]} in compiled CUDA code ({inv.name})")


_BACKEND = None


def backend():
    """The process-wide kernel table."""
    global _BACKEND
    if _BACKEND is None:
        _BACKEND = GB300Backend()
    return _BACKEND
