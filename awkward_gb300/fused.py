"""Elementwise map fused into the float64 segmented reduction.

``segment_reduce(x, offsets, map="x*y", y=y, reduce="sum")`` computes, per
list of ``offsets``, the reduction of the mapped values -- what awkward
computes as ``ak.sum(x * y, axis=-1)`` with an elementwise kernel that
materialises ``x * y`` followed by ``awkward_reduce_sum`` -- in one pass
over x and y (awkward_gb300_fused_reduce_float64).  Maps: "x", "x*y", "x*x",
"abs"; reductions: "sum", "max", "min", "argmax", "argmin".  Launches on the
current torch stream; there is no CPU fallback.
"""

from __future__ import annotations

import torch

from . import _abi

MAPS = {"x": 0, "x*y": 1, "x*x": 2, "abs": 3}
REDUCTIONS = {"sum": 0, "max": 1, "min": 2, "argmax": 3, "argmin": 4}


def segment_reduce(x, offsets, map="x", y=None, reduce="sum", out=None):
    if map not in MAPS or reduce not in REDUCTIONS:
        raise ValueError(f"map must be one of {list(MAPS)}, reduce one of {list(REDUCTIONS)}")
    for name, t in (("x", x), ("offsets", offsets)) + ((("y", y),) if y is not None else ()):
        if not (isinstance(t, torch.Tensor) and t.is_cuda and t.dim() == 1 and t.is_contiguous()):
            raise TypeError(f"{name} must be a contiguous 1-D CUDA tensor")
    if x.dtype != torch.float64 or (y is not None and y.dtype != torch.float64):
        raise TypeError("x and y must be float64")
    if offsets.dtype != torch.int64 or offsets.numel() < 1:
        raise TypeError("offsets must be int64 with nlists + 1 entries")
    if map == "x*y" and (y is None or y.numel() != x.numel()):
        raise ValueError("map 'x*y' needs y with the length of x")
    n = offsets.numel() - 1
    dt = torch.int64 if reduce.startswith("arg") else torch.float64
    if out is None:
        out = torch.empty(n, dtype=dt, device=x.device)
    err = torch.full((1,), -1, dtype=torch.int64, device=x.device)
    if y is not None and y.numel() == 0:  # no element is read; any valid address will do
        y = torch.empty(1, dtype=torch.float64, device=x.device)
    rc = _abi.ext_cfunc("awkward_gb300_fused_reduce_float64")(
        out.data_ptr(), x.data_ptr(), y.data_ptr() if y is not None else None,
        offsets.data_ptr(), n, MAPS[map], REDUCTIONS[reduce], 0, err.data_ptr(),
        torch.cuda.current_stream(x.device).cuda_stream)
    if rc != 0:
        raise RuntimeError(f"fused reduce: CUDA launch failed with cudaError {rc}")
    return out
