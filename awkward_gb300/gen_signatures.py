"""Regenerate the kernel signature table and the C header from awkward's kernel spec.

This is a maintainer step, run by hand in a checkout that has the awkward
sources next to it::

    python -m awkward_gb300.gen_signatures /path/to/awkward

It reads ``kernel-specification.yml`` (the contract every awkward kernel
backend implements; one ``- name:`` entry per kernel family, one nested
``- name:`` per dtype specialization, each with ``{name, type, dir, role}``
argument records) and writes two files that are committed:

* ``awkward_gb300/_signatures.py`` -- the Python table the ctypes loader
  uses (argument names, C types, directions, list depth), plus the spec
  line of every specialization for citation;
* ``include/awkward_gb300.h`` -- the ``extern "C"`` declarations of every
  entry point of ``libawkward_gb300.so``: the spec's arguments in spec order,
  followed by ``(uint64_t invocation_index, uint64_t* err_code, void* stream)``.

The YAML is parsed with regular expressions (the spec's layout is regular),
so no YAML library is needed.  Nothing at run time reads the spec.
"""

from __future__ import annotations

import os
import re
import sys

# Kernel families on the accelerated path, with the awkward-cpp CPU file and
# line of the template each family restates.
FAMILIES = {
    # segmented reducers over ListOffsetArray offsets
    "awkward_reduce_sum": ("awkward_reduce_sum.cpp", 12),
    "awkward_reduce_sum_bool": ("awkward_reduce_sum_bool.cpp", 18),
    "awkward_reduce_sum_int32_bool_64": ("awkward_reduce_sum_int32_bool_64.cpp", 7),
    "awkward_reduce_sum_int64_bool_64": ("awkward_reduce_sum_int64_bool_64.cpp", 7),
    "awkward_reduce_prod": ("awkward_reduce_prod.cpp", 12),
    "awkward_reduce_prod_bool": ("awkward_reduce_prod_bool.cpp", 10),
    "awkward_reduce_max": ("awkward_reduce_max.cpp", 9),
    "awkward_reduce_min": ("awkward_reduce_min.cpp", 26),
    "awkward_reduce_argmax": ("awkward_reduce_argmax.cpp", 9),
    "awkward_reduce_argmin": ("awkward_reduce_argmin.cpp", 25),
    "awkward_reduce_count_64": ("awkward_reduce_count_64.cpp", 7),
    "awkward_reduce_countnonzero": ("awkward_reduce_countnonzero.cpp", 14),
    "awkward_reduce_sumofsquares": ("awkward_reduce_sumofsquares.cpp", 12),
    "awkward_reduce_sumofpowers": ("awkward_reduce_sumofpowers.cpp", 39),
    "awkward_reduce_centered_sumofsquares": ("awkward_reduce_centered_sumofsquares.cpp", 15),
    "awkward_reduce_sum_complex": ("awkward_reduce_sum_complex.cpp", 7),
    "awkward_reduce_prod_complex": ("awkward_reduce_prod_complex.cpp", 9),
    "awkward_reduce_max_complex": ("awkward_reduce_max_complex.cpp", 7),
    "awkward_reduce_min_complex": ("awkward_reduce_min_complex.cpp", 7),
    "awkward_reduce_argmax_complex": ("awkward_reduce_argmax_complex.cpp", 7),
    "awkward_reduce_argmin_complex": ("awkward_reduce_argmin_complex.cpp", 7),
    "awkward_reduce_countnonzero_complex": ("awkward_reduce_countnonzero_complex.cpp", 7),
    "awkward_reduce_sum_bool_complex": ("awkward_reduce_sum_bool_complex.cpp", 7),
    "awkward_reduce_prod_bool_complex": ("awkward_reduce_prod_bool_complex.cpp", 7),
    "awkward_NumpyArray_reduce_adjust_starts_64": ("awkward_NumpyArray_reduce_adjust_starts_64.cpp", 7),
    "awkward_NumpyArray_reduce_mask_ByteMaskedArray_64": ("awkward_NumpyArray_reduce_mask_ByteMaskedArray_64.cpp", 7),
    # jagged getitem and the carries it feeds
    "awkward_ListArray_getitem_jagged_apply": ("awkward_ListArray_getitem_jagged_apply.cpp", 8),
    "awkward_ListArray_getitem_jagged_carrylen": ("awkward_ListArray_getitem_jagged_carrylen.cpp", 8),
    "awkward_ListArray_getitem_jagged_descend": ("awkward_ListArray_getitem_jagged_descend.cpp", 8),
    "awkward_ListArray_getitem_jagged_expand": ("awkward_ListArray_getitem_jagged_expand.cpp", 8),
    "awkward_ListArray_getitem_jagged_numvalid": ("awkward_ListArray_getitem_jagged_numvalid.cpp", 8),
    "awkward_ListArray_getitem_jagged_shrink": ("awkward_ListArray_getitem_jagged_shrink.cpp", 8),
    "awkward_RegularArray_getitem_jagged_expand": ("awkward_RegularArray_getitem_jagged_expand.cpp", 8),
    "awkward_ListArray_localindex": ("awkward_ListArray_localindex.cpp", 8),
    "awkward_ListArray_getitem_next_range": ("awkward_ListArray_getitem_next_range.cpp", 9),
    "awkward_ListArray_getitem_next_range_carrylength": ("awkward_ListArray_getitem_next_range_carrylength.cpp", 9),
    "awkward_RegularArray_getitem_next_range": ("awkward_RegularArray_getitem_next_range.cpp", 8),
    # combinations
    "awkward_ListArray_combinations_length": ("awkward_ListArray_combinations_length.cpp", 8),
    "awkward_ListArray_combinations": ("awkward_ListArray_combinations.cpp", 9),
    # siblings of combinations and jagged broadcasting
    "awkward_RegularArray_combinations_64": ("awkward_RegularArray_combinations_64.cpp", 8),
    "awkward_ListArray_broadcast_tooffsets": ("awkward_ListArray_broadcast_tooffsets.cpp", 8),
    # segmented sort
    "awkward_argsort": ("awkward_argsort.cpp", 62),
    "awkward_sort": ("awkward_sort.cpp", 62),
    # reductions above the innermost axis (non-local) and through option types
    "awkward_ListOffsetArray_reduce_nonlocal_maxcount_offsetscopy_64": ("awkward_ListOffsetArray_reduce_nonlocal_maxcount_offsetscopy_64.cpp", 7),
    "awkward_ListOffsetArray_reduce_nonlocal_preparenext_64": ("awkward_ListOffsetArray_reduce_nonlocal_preparenext_64.cpp", 7),
    "awkward_ListOffsetArray_reduce_nonlocal_outstartsstops_64": ("awkward_ListOffsetArray_reduce_nonlocal_outstartsstops_64.cpp", 10),
    "awkward_ListOffsetArray_reduce_nonlocal_nextshifts_64": ("awkward_ListOffsetArray_reduce_nonlocal_nextshifts_64.cpp", 7),
    "awkward_ListOffsetArray_reduce_local_nextparents_64": ("awkward_ListOffsetArray_reduce_local_nextparents_64.cpp", 14),
    "awkward_ListOffsetArray_local_preparenext_64": ("awkward_ListOffsetArray_local_preparenext_64.cpp", 11),
    "awkward_RegularArray_reduce_local_nextparents_64": ("awkward_RegularArray_reduce_local_nextparents_64.cpp", 14),
    "awkward_RegularArray_reduce_nonlocal_preparenext_64": ("awkward_RegularArray_reduce_nonlocal_preparenext_64.cpp", 7),
    "awkward_IndexedArray_reduce_next_64": ("awkward_IndexedArray_reduce_next_64.cpp", 7),
    "awkward_IndexedArray_reduce_next_fix_offsets_64": ("awkward_IndexedArray_reduce_next_fix_offsets_64.cpp", 7),
    "awkward_IndexedArray_reduce_next_nonlocal_nextshifts_64": ("awkward_IndexedArray_reduce_next_nonlocal_nextshifts_64.cpp", 7),
    "awkward_IndexedArray_reduce_next_nonlocal_nextshifts_fromshifts_64": ("awkward_IndexedArray_reduce_next_nonlocal_nextshifts_fromshifts_64.cpp", 7),
    "awkward_IndexedArray_local_preparenext_64": ("awkward_IndexedArray_local_preparenext_64.cpp", 7),
    "awkward_ByteMaskedArray_reduce_next_64": ("awkward_ByteMaskedArray_reduce_next_64.cpp", 7),
    "awkward_ByteMaskedArray_reduce_next_nonlocal_nextshifts_64": ("awkward_ByteMaskedArray_reduce_next_nonlocal_nextshifts_64.cpp", 7),
    "awkward_ByteMaskedArray_reduce_next_nonlocal_nextshifts_fromshifts_64": ("awkward_ByteMaskedArray_reduce_next_nonlocal_nextshifts_fromshifts_64.cpp", 7),
    # list-layout conversions on the same path (ListArray -> offsets, regular carries)
    "awkward_ListArray_compact_offsets": ("awkward_ListArray_compact_offsets.cpp", 7),
    "awkward_RegularArray_getitem_carry": ("awkward_RegularArray_getitem_carry.cpp", 7),
    "awkward_RegularArray_localindex": ("awkward_RegularArray_localindex.cpp", 7),
    # small siblings on the same driver paths (argmax through option types,
    # axis-0 local index, range slices with advanced indexing, jagged slices
    # with missing values)
    "awkward_NumpyArray_reduce_adjust_starts_shifts_64": ("awkward_NumpyArray_reduce_adjust_starts_shifts_64.cpp", 7),
    "awkward_localindex": ("awkward_localindex.cpp", 8),
    "awkward_ListArray_getitem_next_range_counts": ("awkward_ListArray_getitem_next_range_counts.cpp", 7),
    "awkward_ListArray_getitem_next_range_spreadadvanced": ("awkward_ListArray_getitem_next_range_spreadadvanced.cpp", 7),
    "awkward_RegularArray_getitem_next_range_spreadadvanced": ("awkward_RegularArray_getitem_next_range_spreadadvanced.cpp", 7),
    "awkward_Content_getitem_next_missing_jagged_getmaskstartstop": ("awkward_Content_getitem_next_missing_jagged_getmaskstartstop.cpp", 7),
    "awkward_MaskedArray_getitem_next_jagged_project": ("awkward_MaskedArray_getitem_next_jagged_project.cpp", 7),
}

_C_TYPES = {
    "bool": "bool", "int8_t": "int8_t", "uint8_t": "uint8_t", "int16_t": "int16_t",
    "uint16_t": "uint16_t", "int32_t": "int32_t", "uint32_t": "uint32_t",
    "int64_t": "int64_t", "uint64_t": "uint64_t", "float": "float", "double": "double",
}


def parse_spec(path):
    kernels = []
    cur = spec = None
    with open(path, encoding="utf-8") as f:
        for ln, line in enumerate(f, 1):
            m = re.match(r"^  - name: (\S+)", line)
            if m:
                cur = {"name": m.group(1), "line": ln, "specs": []}
                kernels.append(cur)
                spec = None
                continue
            m = re.match(r"^      - name: (\S+)", line)
            if m and cur is not None:
                spec = {"name": m.group(1), "line": ln, "args": []}
                cur["specs"].append(spec)
                continue
            m = re.match(
                r'^          - \{name: (\w+), type: "([^"]+)", dir: (\w+)(?:, role: ([\w-]+))?\}',
                line,
            )
            if m and spec is not None:
                spec["args"].append(
                    (m.group(1), m.group(2), m.group(3), m.group(4) or "")
                )
    return kernels


def split_type(t):
    const = t.startswith("Const[")
    if const:
        t = t[len("Const["):-1]
    depth = 0
    while t.startswith("List["):
        depth += 1
        t = t[len("List["):-1]
    return const, depth, t


def c_decl(argname, t):
    const, depth, base = split_type(t)
    ctype = _C_TYPES[base]
    if depth == 0:
        return f"{ctype} {argname}"
    if depth == 1:
        return f"{'const ' if const else ''}{ctype}* {argname}"
    return f"{ctype}** {argname}"


def main(refroot):
    here = os.path.dirname(os.path.abspath(__file__))
    repo = os.path.dirname(here)
    kernels = parse_spec(os.path.join(refroot, "kernel-specification.yml"))
    table = {}
    order = []
    for k in kernels:
        if k["name"] not in FAMILIES:
            continue
        cpu_file, cpu_line = FAMILIES[k["name"]]
        for s in k["specs"]:
            args = []
            for (an, at, ad, role) in s["args"]:
                const, depth, base = split_type(at)
                args.append((an, base, ad, depth, const, role))
            table[s["name"]] = {
                "family": k["name"],
                "spec_line": s["line"],
                "cpu": f"awkward-cpp/src/cpu-kernels/{cpu_file}:{cpu_line}",
                "args": args,
            }
            order.append(s["name"])
    missing = set(FAMILIES) - {v["family"] for v in table.values()}
    if missing:
        raise SystemExit(f"families not found in spec: {sorted(missing)}")

    # ---- Python table
    out = [
        '"""Signatures of every entry point of libawkward_gb300.so (generated).',
        "",
        "Generated by ``awkward_gb300/gen_signatures.py`` from awkward's",
        "``kernel-specification.yml``; do not edit by hand.  Each record holds the",
        "kernel family, the spec line of the specialization, the awkward-cpp CPU",
        "template it restates, and its arguments as",
        "``(name, base C type, direction, list depth, const, role)``.",
        '"""',
        "",
        "SIGNATURES = {",
    ]
    for name in order:
        r = table[name]
        out.append(f"    {name!r}: {{")
        out.append(f"        'family': {r['family']!r},")
        out.append(f"        'spec_line': {r['spec_line']},")
        out.append(f"        'cpu': {r['cpu']!r},")
        out.append("        'args': [")
        for a in r["args"]:
            out.append(f"            {a!r},")
        out.append("        ],")
        out.append("    },")
    out.append("}")
    out.append("")
    with open(os.path.join(here, "_signatures.py"), "w", encoding="utf-8") as f:
        f.write("\n".join(out))

    # ---- C header
    h = [
        "/* libawkward_gb300: GB300 (sm_103a) kernels for awkward's jagged hot path.",
        " *",
        " * Generated by awkward_gb300/gen_signatures.py from awkward's",
        " * kernel-specification.yml; do not edit by hand.",
        " *",
        " * Every entry point keeps the name and the argument list of one",
        " * specialization of kernel-specification.yml (cited per declaration as",
        " * kernel-specification.yml:<line>, with the awkward-cpp CPU template it",
        " * replaces), so a ctypes adapter can install it into awkward's cupy",
        " * kernel table keyed by (family, *dtypes).  Differences from the spec:",
        " *   - every pointer is a DEVICE pointer; List[List[T]] is a device array",
        " *     of device pointers;",
        " *   - three trailing arguments follow the spec's arguments:",
        " *       uint64_t  invocation_index  index of this call in the caller's",
        " *                                   pending-invocation list;",
        " *       uint64_t* err_code          device word; a failing kernel does",
        " *                                   atomicMin(err_code,",
        " *                                     invocation_index*256 + message)",
        " *                                   (awkward's RawModule protocol) and",
        " *                                   kernels skip work when it is set;",
        " *       void*     stream            cudaStream_t to launch on (0 = legacy).",
        " *   - the return value is the cudaError_t of the launch (0 = success);",
        " *     data errors are reported only through err_code.",
        " * Outputs are preallocated by the caller.  Temporary buffers (tile",
        " * states of the single-pass scans) come from a stream-ordered pool owned",
        " * by the library and are released in stream order.",
        " */",
        "#ifndef AWKWARD_GB300_H_",
        "#define AWKWARD_GB300_H_",
        "",
        "#include <stdint.h>",
        "#include <stdbool.h>",
        "",
        "#ifdef __cplusplus",
        'extern "C" {',
        "#endif",
        "",
        "#define AWKWARD_GB300_ERROR_BITS 8",
        "#define AWKWARD_GB300_NO_ERROR 0xffffffffffffffffULL",
        "",
    ]
    fam = None
    for name in order:
        r = table[name]
        if r["family"] != fam:
            fam = r["family"]
            h.append(f"/* ---- {fam}: replaces {r['cpu']} */")
        decl = ", ".join(
            c_decl(a[0], (("Const[" if a[4] else "") + "List[" * a[3] + a[1] + "]" * a[3] + ("]" if a[4] else "")))
            for a in r["args"]
        )
        h.append(f"/* kernel-specification.yml:{r['spec_line']} */")
        h.append(
            f"int {name}({decl}, uint64_t invocation_index, uint64_t* err_code, void* stream);"
        )
    from ._extensions import header_lines

    h += header_lines()
    h += [
        "",
        "#ifdef __cplusplus",
        "}",
        "#endif",
        "",
        "#endif /* AWKWARD_GB300_H_ */",
        "",
    ]
    with open(os.path.join(repo, "include", "awkward_gb300.h"), "w", encoding="utf-8") as f:
        f.write("\n".join(h))
    print(f"{len(order)} specializations in {len(FAMILIES)} families")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.environ.get("AWKWARD_SRC", "."))
