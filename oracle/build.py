"""Build recipe for the CPU oracle (test infrastructure only).

Two libraries:

* ``oracle/liboracle.so`` -- ``awkward_oracle.c``, the plain-C restatement of
  the awkward-cpp kernels on the accelerated path.  Built everywhere (here
  and on the GPU host) with ``gcc -O2 -ffp-contract=off -shared -fPIC``.
* ``oracle/_ref/libawkward-cpu-kernels.so`` -- awkward-cpp's OWN CPU kernels
  for the same families, compiled directly from the reference sources where
  they lie (``<awkward>/awkward-cpp/src/cpu-kernels/*.cpp``), used only to pin
  the restatement.  It is built only when the awkward sources are present
  (``AWKWARD_SRC`` or the default checkout path below).  Upstream's
  ``kernels.h`` is produced by its own build from kernel-specification.yml;
  this recipe instead writes a declaration-only header with the same
  ``extern "C"`` prototypes from ``awkward_gb300/_signatures.py`` into
  ``oracle/_ref/include``.  Nothing is copied from the reference tree.
"""

from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
DEFAULT_AWKWARD_SRC = "/root/reference"

ORACLE_SO = os.path.join(HERE, "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")
REF_SO = os.path.join(REF_DIR, "libawkward-cpu-kernels.so")


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build_oracle(force=False):
    src = os.path.join(HERE, "awkward_oracle.c")
    if force or _stale(ORACLE_SO, [src]):
        # no fused multiply-adds: the same roundings on x86 and Arm hosts
        cmd = ["gcc", "-O2", "-std=c11", "-ffp-contract=off", "-shared", "-fPIC", "-pthread", src,
               "-o", ORACLE_SO + ".tmp", "-lm"]
        subprocess.check_call(cmd)
        os.replace(ORACLE_SO + ".tmp", ORACLE_SO)
    return ORACLE_SO


def _ctype(base, depth, const):
    t = base + "*" * depth
    return ("const " + t) if (const and depth) else t


def _write_ref_header(path):
    sys.path.insert(0, REPO)
    from awkward_gb300._signatures import SIGNATURES

    lines = [
        "/* Declarations of the awkward-cpp CPU kernels compiled for the oracle",
        " * (written by oracle/build.py from awkward_gb300/_signatures.py). */",
        "#ifndef AWKWARD_KERNELS_H_",
        "#define AWKWARD_KERNELS_H_",
        '#include "awkward/common.h"',
        'extern "C" {',
    ]
    for name, rec in SIGNATURES.items():
        args = ", ".join(f"{_ctype(a[1], a[3], a[4])} {a[0]}" for a in rec["args"])
        lines.append(f"  EXPORT_SYMBOL ERROR {name}({args});")
    lines += ["}", "#endif", ""]
    os.makedirs(os.path.dirname(path), exist_ok=True)
    with open(path, "w") as f:
        f.write("\n".join(lines))


def build_ref(awkward_src=None, force=False):
    """Compile awkward-cpp's own CPU kernels for the accelerated families."""
    awkward_src = awkward_src or os.environ.get("AWKWARD_SRC", DEFAULT_AWKWARD_SRC)
    kdir = os.path.join(awkward_src, "awkward-cpp", "src", "cpu-kernels")
    inc = os.path.join(awkward_src, "awkward-cpp", "include")
    if not os.path.isdir(kdir):
        return None
    sys.path.insert(0, REPO)
    from awkward_gb300._signatures import SIGNATURES

    files = sorted({rec["cpu"].split(":")[0].split("/")[-1] for rec in SIGNATURES.values()})
    sources = [os.path.join(kdir, f) for f in files] + [os.path.join(kdir, "kernel-utils.cpp")]
    # the set of compiled files changes when families are added: rebuild then too
    manifest = REF_SO + ".sources"
    listed = open(manifest).read() if os.path.exists(manifest) else ""
    wanted = "\n".join(sources)
    if not (force or _stale(REF_SO, sources) or listed != wanted):
        return REF_SO
    hdr = os.path.join(REF_DIR, "include", "awkward", "kernels.h")
    _write_ref_header(hdr)
    cmd = ["g++", "-O2", "-std=c++17", "-shared", "-fPIC", '-DVERSION_INFO="oracle"',
           "-I", os.path.join(REF_DIR, "include"), "-I", inc, *sources, "-o", REF_SO + ".tmp"]
    subprocess.check_call(cmd)
    os.replace(REF_SO + ".tmp", REF_SO)
    with open(manifest, "w") as f:
        f.write(wanted)
    return REF_SO


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_ref(force="--force" in sys.argv))
