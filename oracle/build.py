"""Build recipe for the oracle's native parts.

- ``liboracle.so`` from ``albatros_oracle.c`` (always; gcc, OpenMP).
- ``_ref/lib_unpacking.so`` and ``_ref/lib_correlations_cpu.so`` from the
  reference's own ``src/correlations/unpacking.c`` and
  ``src/correlations/correlations_cpu.c``, compiled where they lie, only when
  the reference checkout is found: at $ALBATROS_REFERENCE, else in a
  directory ``reference`` beside this repository's checkout.  Outputs go to
  ``oracle/_ref/`` (git-ignored).

TEST INFRASTRUCTURE: the product path never loads these libraries.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.environ.get("ALBATROS_REFERENCE") or os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")
CFLAGS = ["-O3", "-std=c99", "-fPIC", "-shared", "-fopenmp"]


def _cc(srcs, out):
    cmd = ["gcc", *CFLAGS, *srcs, "-o", out, "-lm"]
    subprocess.run(cmd, check=True)
    return out


def build_oracle() -> str:
    return _cc([os.path.join(HERE, "albatros_oracle.c")], os.path.join(HERE, "liboracle.so"))


def build_ref() -> bool:
    src = os.path.join(REF, "albatros_analysis", "src", "correlations")
    files = {"lib_unpacking.so": "unpacking.c", "lib_correlations_cpu.so": "correlations_cpu.c"}
    if not all(os.path.exists(os.path.join(src, f)) for f in files.values()):
        return False
    os.makedirs(os.path.join(HERE, "_ref"), exist_ok=True)
    for out, f in files.items():
        _cc([os.path.join(src, f)], os.path.join(HERE, "_ref", out))
    return True


if __name__ == "__main__":
    print(build_oracle())
    print("reference C built:", build_ref())
    sys.exit(0)
