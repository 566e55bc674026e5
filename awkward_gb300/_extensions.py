"""Entry points of libawkward_gb300 that have no kernel-specification.yml counterpart.

One table serves the header generator (gen_signatures.py), the ctypes loader
(_abi.py) and the export test.  Each entry: name -> (C argument list as
(type, name) pairs, comment for the header).  All return int (cudaError_t).
"""

from __future__ import annotations

_NOALLOC_COMMENT = """no-alloc variant.  No counterpart in awkward: an extra entry point
of this library for callers that may not allocate device memory while
they run, e.g. code embedded in a process whose GPU memory is owned by
another framework's pooling allocator (cudaMalloc then fails or goes
around the pool, and the caller has no handle to the pool).
Same arguments and results as awkward_ListArray64_getitem_jagged_apply_64;
its tile-state scratch is a fixed 512 KiB device array inside the
library (held on every GPU that loads it until exit) instead of a
pool allocation.  sliceouterlen above AWKWARD_GB300_NOALLOC_MAX_LISTS
returns cudaErrorInvalidValue (1) and launches nothing.  All calls
share the array: calls that overlap on the GPU (other streams or
threads) race and must be ordered by the caller.  The first call in
each CUDA context looks up the array's device address (cached per
device and context), so make it before any stream capture there."""

_AUTOGRAD_COMMENT = """backward kernels of differentiable jagged operations (torch.autograd
in awkward_gb300/autograd.py).  No counterpart in awkward, which has no
CUDA backward kernels.  Pointers are device pointers; offsets are int64
[nlists + 1] (need not start at 0); element arrays are indexed globally;
nvalues is the length of the element arrays: elements no list covers are
set to 0, the others written by the kernels (no prior clearing needed).
  segment_sum_backward:   grad_x[j] = grad_out[list of j]
  segment_max_backward:   grad_x = 0; grad_x[argmax[l]] = grad_out[l] for
                          argmax[l] in [0, nelements) (global indices, -1 empty)
  jagged_softmax_forward: y = exp(x - max) / sum(exp(x - max)) per list
  jagged_softmax_backward: grad_x = y * (grad_y - sum(grad_y * y)) per list,
                          y from y_saved, or recomputed from x when NULL"""

EXTENSIONS = {
    "awkward_ListArray64_getitem_jagged_apply_64_noalloc": (
        [("int64_t*", "tooffsets"), ("int64_t*", "tocarry"), ("const int64_t*", "slicestarts"),
         ("const int64_t*", "slicestops"), ("int64_t", "sliceouterlen"),
         ("const int64_t*", "sliceindex"), ("int64_t", "sliceinnerlen"),
         ("const int64_t*", "fromstarts"), ("const int64_t*", "fromstops"),
         ("int64_t", "contentlen"), ("uint64_t", "invocation_index"), ("uint64_t*", "err_code"),
         ("void*", "stream")],
        "noalloc"),
}

for _suffix, _t in (("float32", "float"), ("float64", "double")):
    EXTENSIONS[f"awkward_gb300_segment_sum_backward_{_suffix}"] = (
        [(f"{_t}*", "grad_x"), (f"const {_t}*", "grad_out"), ("const int64_t*", "offsets"),
         ("int64_t", "nlists"), ("int64_t", "nvalues"), ("void*", "stream")], "autograd")
    EXTENSIONS[f"awkward_gb300_segment_max_backward_{_suffix}"] = (
        [(f"{_t}*", "grad_x"), (f"const {_t}*", "grad_out"), ("const int64_t*", "argmax"),
         ("int64_t", "nelements"), ("int64_t", "nlists"), ("void*", "stream")], "autograd")
    EXTENSIONS[f"awkward_gb300_jagged_softmax_forward_{_suffix}"] = (
        [(f"{_t}*", "y"), (f"const {_t}*", "x"), ("const int64_t*", "offsets"),
         ("int64_t", "nlists"), ("int64_t", "nvalues"), ("void*", "stream")], "autograd")
    EXTENSIONS[f"awkward_gb300_jagged_softmax_backward_{_suffix}"] = (
        [(f"{_t}*", "grad_x"), (f"const {_t}*", "grad_y"), (f"const {_t}*", "x"),
         (f"const {_t}*", "y_saved"), ("const int64_t*", "offsets"), ("int64_t", "nlists"),
         ("int64_t", "nvalues"), ("void*", "stream")], "autograd")

_JAGGED_COMMENT = """jagged getitem steps that awkward performs with cupy array operations
instead of kernels of its specification (no counterpart in
kernel-specification.yml):
  jagged_mask_to_index: jagged boolean mask (uint8, one byte per element,
    indexed globally over offsets[0]..offsets[nlists]) -> new offsets
    [nlists + 1] and, for each true entry in order, its position within its
    list (src/awkward/_slicing.py:476-530: localindex + compaction + cumsum);
  jagged_mask_select: array[mask] in one pass -- the new offsets, the
    selected content (itemsize 1, 2, 4 or 8) and optionally the carry
    (NULL to skip), without the local index of the chain;
  jagged_index_select: array[index] with a jagged int64 index in one pass
    -- jagged_apply with the content gathered at each carry (itemsize 1, 2,
    4 or 8; tocarry NULL to skip), errors as jagged_apply's;
  take: out[i] = content[carry[i]] for itemsize 1, 2, 4 or 8 bytes
    (NumpyArray._carry); a carry outside [0, contentlen) sets err_code to
    invocation_index*256 + 0 ("index out of range")."""

EXTENSIONS["awkward_gb300_jagged_mask_to_index"] = (
    [("int64_t*", "tooffsets"), ("int64_t*", "toindex"), ("const uint8_t*", "mask"),
     ("const int64_t*", "offsets"), ("int64_t", "nlists"), ("uint64_t*", "err_code"),
     ("void*", "stream")], "jagged")
EXTENSIONS["awkward_gb300_jagged_mask_select"] = (
    [("int64_t*", "tooffsets"), ("void*", "tocontent"), ("int64_t*", "tocarry"),
     ("const uint8_t*", "mask"), ("const int64_t*", "offsets"), ("const void*", "content"),
     ("int64_t", "itemsize"), ("int64_t", "nlists"), ("uint64_t*", "err_code"),
     ("void*", "stream")], "jagged")
EXTENSIONS["awkward_gb300_jagged_index_select"] = (
    [("int64_t*", "tooffsets"), ("void*", "tocontent"), ("int64_t*", "tocarry"),
     ("const int64_t*", "index_offsets"), ("const int64_t*", "index"), ("int64_t", "indexlen"),
     ("const int64_t*", "offsets"), ("const void*", "content"), ("int64_t", "itemsize"),
     ("int64_t", "contentlen"), ("int64_t", "nlists"), ("uint64_t*", "err_code"),
     ("void*", "stream")], "jagged")
EXTENSIONS["awkward_gb300_take"] = (
    [("void*", "out"), ("const void*", "content"), ("int64_t", "itemsize"),
     ("const int64_t*", "carry"), ("int64_t", "n"), ("int64_t", "contentlen"),
     ("uint64_t", "invocation_index"), ("uint64_t*", "err_code"), ("void*", "stream")], "jagged")

_BATCH_COMMENT = """batched execution (no counterpart in awkward): sum, max, argmax and
count (axis=-1) and array[mask] of many float64 ListOffsetArrays in one
launch per operation.  plan_create (set-up: allocates and uploads the
work-queue tables, synchronous) takes host arrays of narrays entries:
list counts, element counts (offsets[n] - offsets[0]) and the device
pointers of each array's content, offsets, uint8 mask and outputs
(out_sum/out_max [n] float64, out_argmax/out_count [n] int64,
sel_offsets [n + 1] int64, sel_content [elements] float64).  Tuning
knobs: order_mode (0 array order, 1 largest ranges first),
occupancy_div (persistent CTAs per SM = occupancy / div), range_min
(items per range of arrays with no list above 4096 elements, >= 512),
block (threads per reducer CTA, 128 or 256).  Reducer results are
bit-identical to the per-array entry points.  plan_run only
launches (capturable in a CUDA graph); plan_destroy frees the plan."""

EXTENSIONS["awkward_gb300_batch_plan_create"] = (
    [("void**", "plan"), ("int64_t", "narrays"), ("const int64_t*", "nlists"),
     ("const int64_t*", "nelements"), ("const int64_t*", "maxlen"), ("const double* const*", "x"),
     ("const int64_t* const*", "offsets"), ("const uint8_t* const*", "mask"),
     ("double* const*", "out_sum"), ("double* const*", "out_max"),
     ("int64_t* const*", "out_argmax"), ("int64_t* const*", "out_count"),
     ("int64_t* const*", "sel_offsets"), ("double* const*", "sel_content"),
     ("int64_t", "order_mode"), ("int64_t", "occupancy_div"), ("int64_t", "range_min"),
     ("int64_t", "block"), ("uint64_t*", "err_code")], "batch")
EXTENSIONS["awkward_gb300_batch_plan_run"] = ([("void*", "plan"), ("void*", "stream")], "batch")
EXTENSIONS["awkward_gb300_batch_plan_destroy"] = ([("void*", "plan")], "batch")

_PIPELINE_COMMENT = """host-buffer reduction with overlapped transfers (no counterpart in
awkward): segmented sum, max (identity -inf) and argmax of a float64
ListOffsetArray in pinned host memory.  Lists are cut into `chunks`
(1..64) at list boundaries; copies in of chunk c+1, the reductions of
chunk c and copies back of chunk c-1 overlap.  Device workspace: d_x
(element j at d_x[j]), d_offsets [nlists + 1], three outputs [nlists].
Returns after enqueueing; `stream` waits for the last copy back."""

EXTENSIONS["awkward_gb300_reduce_sum_max_argmax_host_float64"] = (
    [("double*", "h_sum"), ("double*", "h_max"), ("int64_t*", "h_argmax"),
     ("const double*", "h_x"), ("const int64_t*", "h_offsets"), ("int64_t", "nlists"),
     ("double*", "d_x"), ("int64_t*", "d_offsets"), ("double*", "d_sum"), ("double*", "d_max"),
     ("int64_t*", "d_argmax"), ("int64_t", "chunks"), ("void*", "stream")], "pipeline")

_FUSED_COMMENT = """elementwise map fused into the segmented reduction (no counterpart in
kernel-specification.yml; awkward evaluates such chains as an elementwise
kernel followed by a reducer, or through its lazy fusion backend).
float64 content x (and y), int64 offsets [nlists + 1] (need not start at
0), indexed globally.  map: 0 x, 1 x*y, 2 x*x, 3 |x| (y may be NULL unless
map is 1).  reduce: 0 sum, 1 max (identity -inf), 2 min (identity +inf)
into double out[nlists]; 3 argmax, 4 argmin into int64 out[nlists]
(global indices, -1 for empty lists).  Equal to awkward_reduce_* on the
materialised mapped values (sums within the reducers' bound).  Other
map or reduce values, or map 1 without y, return cudaErrorInvalidValue."""

EXTENSIONS["awkward_gb300_fused_reduce_float64"] = (
    [("void*", "out"), ("const double*", "x"), ("const double*", "y"),
     ("const int64_t*", "offsets"), ("int64_t", "nlists"), ("int64_t", "map"),
     ("int64_t", "reduce"), ("uint64_t", "invocation_index"), ("uint64_t*", "err_code"),
     ("void*", "stream")], "fused")

_SELFTEST_COMMENT = """self-test of the failure report (no counterpart in awkward): one warp
runs the decoupled look-back of the scan kernels on tile 1 of a fresh
scan whose tile 0 never publishes, with a spin limit of `spin_limit`
polls (clamped to 1..2^22; each poll sleeps at most 256 ns).  The wait
runs out and the kernel sets err_code to invocation_index*256 + 32, the
library's "bounded wait gave up" code, then returns; the GPU stays
usable.  It is how the tests check that a stalled look-back ends with an
error the host can read instead of a hang."""

EXTENSIONS["awkward_gb300_selftest_lookback_timeout"] = (
    [("uint32_t", "spin_limit"), ("uint64_t", "invocation_index"), ("uint64_t*", "err_code"),
     ("void*", "stream")], "selftest")

GROUP_COMMENTS = {"noalloc": _NOALLOC_COMMENT, "autograd": _AUTOGRAD_COMMENT,
                  "jagged": _JAGGED_COMMENT, "batch": _BATCH_COMMENT,
                  "pipeline": _PIPELINE_COMMENT, "fused": _FUSED_COMMENT,
                  "selftest": _SELFTEST_COMMENT}
GROUP_DEFINES = {"noalloc": ["#define AWKWARD_GB300_NOALLOC_MAX_LISTS 67108864LL"]}


def header_lines():
    """Declarations of the extension entry points, grouped, for the C header."""
    out = []
    for group in ("noalloc", "jagged", "autograd", "batch", "pipeline", "fused", "selftest"):
        out.append("")
        text = GROUP_COMMENTS[group].splitlines()
        out.append(f"/* ---- {text[0]}")
        out.extend(f" * {t}".rstrip() for t in text[1:])
        out[-1] = out[-1] + " */"
        out.extend(GROUP_DEFINES.get(group, []))
        for name, (args, g) in EXTENSIONS.items():
            if g == group:
                out.append(f"int {name}({', '.join(f'{t} {a}' for t, a in args)});")
    return out
