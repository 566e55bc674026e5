"""Differentiable jagged operations: torch.autograd.Function over the GB300 kernels.

A jagged array here is ``(values, offsets)``: ``values`` a 1-D CUDA tensor
(float32 or float64) and ``offsets`` an int64 CUDA tensor of ``nlists + 1``
entries (the ListOffsetArray layout; offsets need not start at 0, elements
are indexed globally).  Every forward and backward pass runs this library's
CUDA kernels; there is no fallback.

* ``segment_sum(values, offsets)``   -> per-list sums (float32 accumulates in
  float32 in list order, float64 as a fixed-point sum rounded once, within
  n*eps*sum|x| of the exact sum); backward broadcasts the
  output gradient to every element of its list.
* ``segment_max(values, offsets)``   -> per-list maxima (``-inf`` for an empty
  list; NaN ignored, as ak.max); backward routes each list's gradient to the
  element awkward's argmax selects (first maximum), zero elsewhere.
* ``jagged_softmax(values, offsets)`` -> ``exp(x - max) / sum(exp(x - max))``
  per list (equal to ak.softmax's ``exp(x) / sum(exp(x))``, without its
  overflow); backward applies the softmax Jacobian in one fused kernel.  The
  forward keeps ``y`` for the backward only while ``y`` plus the per-list
  maxima and normalisers fit ``activation_budget`` bytes; otherwise the
  backward recomputes them from ``x`` (no extra activation memory).
"""

from __future__ import annotations

import numpy as np
import torch

from . import _abi
from .kernel_table import backend

DEFAULT_ACTIVATION_BUDGET = 256 * 2**20

_SUFFIX = {torch.float32: "float32", torch.float64: "float64"}
_NP = {torch.float32: np.float32, torch.float64: np.float64}


def _check(values, offsets):
    if values.dtype not in _SUFFIX:
        raise TypeError(f"values must be float32 or float64, not {values.dtype}")
    if not (values.is_cuda and offsets.is_cuda):
        raise TypeError("values and offsets must be CUDA tensors")
    if offsets.dtype != torch.int64 or offsets.dim() != 1 or offsets.numel() < 1:
        raise TypeError("offsets must be a 1-D int64 tensor of nlists + 1 entries")
    if values.dim() != 1 or not values.is_contiguous() or not offsets.is_contiguous():
        raise ValueError("values and offsets must be contiguous 1-D tensors")


def _stream(t):
    return torch.cuda.current_stream(t.device).cuda_stream


def _launch(name, *args):
    rc = _abi.ext_cfunc(name)(*args)
    if rc != 0:
        raise RuntimeError(f"{name}: CUDA launch failed with cudaError {rc}")


def _reduce(family, out, values, offsets, *extra):
    dt = _NP[values.dtype]
    key = {"sum": ("awkward_reduce_sum", dt, dt, np.int64),
           "max": ("awkward_reduce_max", dt, dt, np.int64),
           "argmax": ("awkward_reduce_argmax", np.int64, dt, np.int64, np.int64)}[family]
    backend()[key](out, values, offsets, *extra)


class SegmentSum(torch.autograd.Function):
    @staticmethod
    def forward(ctx, values, offsets):
        _check(values, offsets)
        n = offsets.numel() - 1
        out = torch.empty(n, dtype=values.dtype, device=values.device)
        _reduce("sum", out, values, offsets, n)
        ctx.save_for_backward(offsets)
        ctx.nvalues = values.numel()
        return out

    @staticmethod
    def backward(ctx, grad_out):
        (offsets,) = ctx.saved_tensors
        g = grad_out.contiguous()
        gx = torch.empty(ctx.nvalues, dtype=g.dtype, device=g.device)  # every element written
        _launch(f"awkward_gb300_segment_sum_backward_{_SUFFIX[g.dtype]}", gx.data_ptr(),
                g.data_ptr(), offsets.data_ptr(), offsets.numel() - 1, ctx.nvalues, _stream(g))
        return gx, None


class SegmentMax(torch.autograd.Function):
    @staticmethod
    def forward(ctx, values, offsets):
        _check(values, offsets)
        n = offsets.numel() - 1
        out = torch.empty(n, dtype=values.dtype, device=values.device)
        arg = torch.empty(n, dtype=torch.int64, device=values.device)
        _reduce("max", out, values, offsets, n, -np.inf)
        _reduce("argmax", arg, values, offsets, offsets[:-1].contiguous(), n)
        ctx.save_for_backward(arg)
        ctx.nvalues = values.numel()
        return out

    @staticmethod
    def backward(ctx, grad_out):
        (arg,) = ctx.saved_tensors
        g = grad_out.contiguous()
        gx = torch.empty(ctx.nvalues, dtype=g.dtype, device=g.device)
        _launch(f"awkward_gb300_segment_max_backward_{_SUFFIX[g.dtype]}", gx.data_ptr(),
                g.data_ptr(), arg.data_ptr(), ctx.nvalues, arg.numel(), _stream(g))
        return gx, None


class JaggedSoftmax(torch.autograd.Function):
    @staticmethod
    def forward(ctx, values, offsets, activation_budget=DEFAULT_ACTIVATION_BUDGET):
        _check(values, offsets)
        n = offsets.numel() - 1
        y = torch.empty_like(values)  # elements outside the offsets' span are set to 0
        _launch(f"awkward_gb300_jagged_softmax_forward_{_SUFFIX[values.dtype]}", y.data_ptr(),
                values.data_ptr(), offsets.data_ptr(), n, values.numel(), _stream(values))
        itemsize = values.element_size()
        keep_y = (values.numel() + 2 * n) * itemsize <= activation_budget
        ctx.keep_y = keep_y
        if keep_y:
            ctx.save_for_backward(values, offsets, y)
        else:
            ctx.save_for_backward(values, offsets)
        return y

    @staticmethod
    def backward(ctx, grad_y):
        saved = ctx.saved_tensors
        values, offsets = saved[0], saved[1]
        y = saved[2] if ctx.keep_y else None
        g = grad_y.contiguous()
        gx = torch.empty_like(values)  # every element written (0 outside the lists)
        _launch(f"awkward_gb300_jagged_softmax_backward_{_SUFFIX[g.dtype]}", gx.data_ptr(),
                g.data_ptr(), values.data_ptr(), y.data_ptr() if y is not None else None,
                offsets.data_ptr(), offsets.numel() - 1, values.numel(), _stream(g))
        return gx, None, None


def segment_sum(values, offsets):
    return SegmentSum.apply(values, offsets)


def segment_max(values, offsets):
    return SegmentMax.apply(values, offsets)


def jagged_softmax(values, offsets, activation_budget=DEFAULT_ACTIVATION_BUDGET):
    return JaggedSoftmax.apply(values, offsets, activation_budget)
