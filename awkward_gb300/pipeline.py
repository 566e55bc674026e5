"""Reductions of jagged arrays held in host memory, with overlapped transfers.

``reduce_host(x, offsets)`` returns the per-list float64 sum, max and argmax
(the results of ak.sum, ak.max and ak.argmax with axis=-1 before their
option masks) of a ListOffsetArray whose content and offsets are CPU tensors
(pinned for the copies to overlap).  The work is enqueued on the current
CUDA stream and the outputs are pinned CPU tensors that are valid once that
stream has been synchronised.  A ``Workspace`` keeps the device buffers
between calls.
"""

from __future__ import annotations

import torch

from . import _abi


class Workspace:
    def __init__(self, nlists, nelements, device="cuda"):
        self.nlists, self.nelements = nlists, nelements
        self.x = torch.empty(max(nelements, 1), dtype=torch.float64, device=device)
        self.offsets = torch.empty(nlists + 1, dtype=torch.int64, device=device)
        self.sum = torch.empty(max(nlists, 1), dtype=torch.float64, device=device)
        self.max = torch.empty(max(nlists, 1), dtype=torch.float64, device=device)
        self.argmax = torch.empty(max(nlists, 1), dtype=torch.int64, device=device)

    def fits(self, nlists, end):
        return nlists <= self.nlists and end <= self.x.numel()


def reduce_host(x, offsets, chunks=8, workspace=None, out=None):
    """(sum, max, argmax) pinned CPU tensors of the float64 jagged array (x, offsets)."""
    if x.dtype != torch.float64 or offsets.dtype != torch.int64:
        raise TypeError("x must be float64 and offsets int64")
    if x.is_cuda or offsets.is_cuda:
        raise TypeError("reduce_host takes CPU (preferably pinned) tensors")
    x, offsets = x.contiguous(), offsets.contiguous()
    n = offsets.numel() - 1
    end = int(offsets[-1]) if n >= 0 else 0
    if workspace is None or not workspace.fits(n, end):
        workspace = Workspace(n, end)
    if out is None:
        out = (torch.empty(max(n, 1), dtype=torch.float64).pin_memory(),
               torch.empty(max(n, 1), dtype=torch.float64).pin_memory(),
               torch.empty(max(n, 1), dtype=torch.int64).pin_memory())
    w = workspace
    rc = _abi.ext_cfunc("awkward_gb300_reduce_sum_max_argmax_host_float64")(
        out[0].data_ptr(), out[1].data_ptr(), out[2].data_ptr(), x.data_ptr(),
        offsets.data_ptr(), n, w.x.data_ptr(), w.offsets.data_ptr(), w.sum.data_ptr(),
        w.max.data_ptr(), w.argmax.data_ptr(), chunks,
        torch.cuda.current_stream(w.x.device).cuda_stream)
    if rc != 0:
        raise RuntimeError(f"awkward_gb300_reduce_sum_max_argmax_host_float64: cudaError {rc}")
    return out[0][:n], out[1][:n], out[2][:n]
