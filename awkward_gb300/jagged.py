"""Jagged getitem on (offsets, content) pairs, following awkward's own call sequence.

Host-side mirror of the parts of awkward's getitem path on this library's
kernels, for CUDA tensors:

* ``getitem_jagged_mask``  -- ``array[mask]`` with a jagged boolean mask of the
  same offsets: the mask becomes a jagged local index
  (src/awkward/_slicing.py:476-530), which is applied with
  ``awkward_ListArray_getitem_jagged_apply`` (src/awkward/contents/listarray.py:573-616)
  and the content carried (``NumpyArray._carry``);
* ``getitem_jagged_index`` -- ``array[idx]`` with a jagged int64 index
  (same apply + carry); ``index_select`` does it in one kernel (the apply
  with the content gathered at each carry), ``mask_select`` the same for
  ``array[mask]``;
* ``getitem_inner_range``  -- ``array[..., start:stop:step]`` on the innermost
  list level of a two-level ListOffsetArray:
  ``awkward_ListArray_getitem_next_range_carrylength``, the carry allocation,
  ``awkward_ListArray_getitem_next_range`` and the carry
  (src/awkward/contents/listarray.py:795-862).

Sizes that depend on data are read back from the device exactly where
awkward reads them (the carry length, the total of true mask entries).
Errors follow awkward's protocol and surface as ``ValueError``.
"""

from __future__ import annotations

import numpy as np
import torch

from . import _abi
from .kernel_table import backend

SLICE_NONE = np.iinfo(np.int64).max  # awkward's kSliceNone


def _stream(t):
    return torch.cuda.current_stream(t.device).cuda_stream


def _err_word(device):
    return torch.full((1,), -1, dtype=torch.int64, device=device)


def _raise_if(err, what):
    word = int(err.item()) & ((1 << 64) - 1)
    if word != (1 << 64) - 1:
        raise ValueError(f"index out of range in compiled CUDA code ({what})")


def take(content, carry, check=True):
    """content[carry] (a gather); raises ValueError for a carry outside the content."""
    out = torch.empty(carry.numel(), dtype=content.dtype, device=content.device)
    err = _err_word(content.device)
    rc = _abi.ext_cfunc("awkward_gb300_take")(
        out.data_ptr(), content.data_ptr(), content.element_size(), carry.data_ptr(),
        carry.numel(), content.numel(), 0, err.data_ptr(), _stream(content))
    if rc != 0:
        raise RuntimeError(f"awkward_gb300_take: cudaError {rc}")
    if check:
        _raise_if(err, "take")
    return out


def jagged_mask_to_index(offsets, mask):
    """(index offsets, local index) of the true entries of a jagged boolean mask."""
    n = offsets.numel() - 1
    span = int(offsets[-1].item() - offsets[0].item()) if n > 0 else 0
    tooffsets = torch.empty(n + 1, dtype=torch.int64, device=offsets.device)
    toindex = torch.empty(max(span, 1), dtype=torch.int64, device=offsets.device)
    m = mask.view(torch.uint8) if mask.dtype == torch.bool else mask
    err = _err_word(offsets.device)
    rc = _abi.ext_cfunc("awkward_gb300_jagged_mask_to_index")(
        tooffsets.data_ptr(), toindex.data_ptr(), m.data_ptr(), offsets.data_ptr(), n,
        err.data_ptr(), _stream(offsets))
    if rc != 0:
        raise RuntimeError(f"awkward_gb300_jagged_mask_to_index: cudaError {rc}")
    k = int(tooffsets[-1].item())
    return tooffsets, toindex[:k]


def mask_select(offsets, content, mask, with_carry=False):
    """array[mask] in one pass (awkward_gb300_jagged_mask_select): the new
    offsets, the selected content and, with `with_carry`, the carry (each
    selected element's position in the content) -- the same outputs as
    getitem_jagged_mask without its intermediate local index."""
    n = offsets.numel() - 1
    span = int(offsets[-1].item() - offsets[0].item()) if n > 0 else 0
    tooffsets = torch.empty(n + 1, dtype=torch.int64, device=offsets.device)
    out = torch.empty(max(span, 1), dtype=content.dtype, device=content.device)
    carry = torch.empty(max(span, 1), dtype=torch.int64, device=offsets.device) if with_carry else None
    m = mask.view(torch.uint8) if mask.dtype == torch.bool else mask
    err = _err_word(offsets.device)
    rc = _abi.ext_cfunc("awkward_gb300_jagged_mask_select")(
        tooffsets.data_ptr(), out.data_ptr(), carry.data_ptr() if with_carry else None,
        m.data_ptr(), offsets.data_ptr(), content.data_ptr(), content.element_size(), n,
        err.data_ptr(), _stream(offsets))
    if rc != 0:
        raise RuntimeError(f"awkward_gb300_jagged_mask_select: cudaError {rc}")
    k = int(tooffsets[-1].item()) if n > 0 else 0
    if with_carry:
        return tooffsets, out[:k], carry[:k]
    return tooffsets, out[:k]


def index_select(offsets, content, index_offsets, index, with_carry=False):
    """array[idx] with a jagged int64 index in one pass
    (awkward_gb300_jagged_index_select): the new offsets, the gathered
    content and, with `with_carry`, the carry -- the same outputs as
    getitem_jagged_index without writing and re-reading the carry.  Errors
    are jagged_apply's, raised as ValueError."""
    from ._messages import messages

    n = offsets.numel() - 1
    k = index.numel()
    tooffsets = torch.empty(n + 1, dtype=torch.int64, device=offsets.device)
    out = torch.empty(max(k, 1), dtype=content.dtype, device=content.device)
    carry = torch.empty(max(k, 1), dtype=torch.int64, device=offsets.device) if with_carry else None
    # a one-element stand-in keeps the pointers valid when the content is empty
    src = content if content.numel() > 0 else torch.zeros(1, dtype=content.dtype,
                                                          device=content.device)
    err = _err_word(offsets.device)
    rc = _abi.ext_cfunc("awkward_gb300_jagged_index_select")(
        tooffsets.data_ptr(), out.data_ptr(), carry.data_ptr() if with_carry else None,
        index_offsets.data_ptr(), index.data_ptr(), k, offsets.data_ptr(), src.data_ptr(),
        content.element_size(), content.numel(), n, err.data_ptr(), _stream(offsets))
    if rc != 0:
        raise RuntimeError(f"awkward_gb300_jagged_index_select: cudaError {rc}")
    word = int(err.item()) & ((1 << 64) - 1)
    if word != (1 << 64) - 1:
        msg = messages("awkward_ListArray_getitem_jagged_apply")[word & 255]
        raise ValueError(f"{msg} in compiled CUDA code (awkward_gb300_jagged_index_select)")
    m = int(tooffsets[-1].item()) if n > 0 else 0
    if with_carry:
        return tooffsets, out[:m], carry[:m]
    return tooffsets, out[:m]


def jagged_apply(offsets, index_offsets, index, contentlen):
    """(tooffsets, tocarry) of a jagged int index applied to lists with these offsets."""
    be = backend()
    n = offsets.numel() - 1
    tooffsets = torch.empty(n + 1, dtype=torch.int64, device=offsets.device)
    tocarry = torch.empty(max(index.numel(), 1), dtype=torch.int64, device=offsets.device)
    be["awkward_ListArray_getitem_jagged_apply", np.int64, np.int64, np.int64, np.int64,
       np.int64, np.int64, np.int64](
        tooffsets, tocarry, index_offsets[:-1].contiguous(), index_offsets[1:].contiguous(), n,
        index, index.numel(), offsets[:-1].contiguous(), offsets[1:].contiguous(), contentlen)
    be.synchronize()
    return tooffsets, tocarry[: index.numel()]


def getitem_jagged_index(offsets, content, index_offsets, index):
    tooffsets, tocarry = jagged_apply(offsets, index_offsets, index, content.numel())
    return tooffsets, take(content, tocarry)


def getitem_jagged_mask(offsets, content, mask):
    index_offsets, index = jagged_mask_to_index(offsets, mask)
    return getitem_jagged_index(offsets, content, index_offsets, index)


def inner_range(inner_offsets, start=None, stop=None, step=None):
    """(nextoffsets, nextcarry) of [start:stop:step] on every list of one level."""
    be = backend()
    n = inner_offsets.numel() - 1
    st, sp = inner_offsets[:-1].contiguous(), inner_offsets[1:].contiguous()
    a = SLICE_NONE if start is None else start
    b = SLICE_NONE if stop is None else stop
    c = 1 if step is None else step
    carrylength = torch.empty(1, dtype=torch.int64, device=inner_offsets.device)
    be["awkward_ListArray_getitem_next_range_carrylength", np.int64, np.int64, np.int64](
        carrylength, st, sp, n, a, b, c)
    be.synchronize()
    nextcarry = torch.empty(max(int(carrylength.item()), 1), dtype=torch.int64,
                            device=inner_offsets.device)
    nextoffsets = torch.empty(n + 1, dtype=torch.int64, device=inner_offsets.device)
    be["awkward_ListArray_getitem_next_range", np.int64, np.int64, np.int64, np.int64](
        nextoffsets, nextcarry, st, sp, n, a, b, c)
    be.synchronize()
    return nextoffsets, nextcarry[: int(carrylength.item())]


def getitem_inner_range(outer_offsets, inner_offsets, content, start=None, stop=None, step=None):
    """array[..., start:stop:step] of a two-level ListOffsetArray: the outer offsets
    are unchanged; returns (outer_offsets, new inner offsets, new content)."""
    nextoffsets, nextcarry = inner_range(inner_offsets, start, stop, step)
    return outer_offsets, nextoffsets, take(content, nextcarry)
