"""Error messages of every kernel family, indexed by the code a kernel raises.

Codes 0.. follow the ``// message:`` order of awkward's CUDA kernel of the
same family (src/awkward/_connect/cuda/cuda_kernels/<family>.cu), whose text
is the awkward-cpp CPU message; code 32 is this library's own "a bounded
wait gave up" failure.  ``messages(family)`` returns a list indexable by
code, which is the shape awkward's ``kernel_errors[name]`` table uses
(src/awkward/_connect/cuda/__init__.py:171-185).
"""

TIMEOUT_CODE = 32
TIMEOUT_MESSAGE = "GPU kernel gave up waiting for a predecessor tile (bounded wait exceeded)"

_FAMILY_MESSAGES = {
    # awkward_ListArray_getitem_jagged_apply.cu:14-20
    "awkward_ListArray_getitem_jagged_apply": [
        "jagged slice's stops[i] < starts[i]",
        "jagged slice's offsets extend beyond its content",
        "stops[i] < starts[i]",
        "stops[i] > len(content)",
        "index out of range",
    ],
    # awkward_ListArray_getitem_jagged_descend.cu:14-16
    "awkward_ListArray_getitem_jagged_descend": [
        "jagged slice inner length differs from array inner length",
    ],
    # awkward_ListArray_getitem_jagged_expand.cu:3-6
    "awkward_ListArray_getitem_jagged_expand": [
        "stops[i] < starts[i]",
        "cannot fit jagged slice into nested list",
    ],
    # awkward_ListArray_broadcast_tooffsets.cu:18-22
    "awkward_ListArray_broadcast_tooffsets": [
        "stops[i] > len(content)",
        "broadcast's offsets must be monotonically increasing",
        "cannot broadcast nested list",
    ],
    # awkward_ListArray_compact_offsets.cu:15
    "awkward_ListArray_compact_offsets": [
        "stops[i] < starts[i]",
    ],
    # awkward_ListArray_getitem_jagged_numvalid.cu:14-17
    "awkward_ListArray_getitem_jagged_numvalid": [
        "jagged slice's stops[i] < starts[i]",
        "jagged slice's offsets extend beyond its content",
    ],
}


def messages(family):
    """Message list indexable by error code (unused codes hold a placeholder)."""
    base = list(_FAMILY_MESSAGES.get(family, []))
    out = base + [f"unknown error code {i}" for i in range(len(base), TIMEOUT_CODE)]
    out.append(TIMEOUT_MESSAGE)
    return out
