"""Build recipe for the oracle (test infrastructure only).

``build_oracle()`` compiles the CPU restatement ``oracle/oracle.c`` into
``oracle/liboracle.so`` (gcc, OpenMP, ``-ffp-contract=off``).

``build_ref()`` compiles the reference's own analytic weight functions
(compute_matrix.cu:21-257 of savthe/gpu_determ) for the host into
``oracle/_ref/libref_weights.so``, reading them where they lie in the
reference checkout and streaming them through the compiler's standard input
between ``ref_prelude.h`` and ``ref_epilogue.cpp``; no reference source is
written into the repository.  The checkout is $GD_REFERENCE_DIR, else a
directory ``reference`` beside this repository; the step is skipped (returns
None) when it is absent, e.g. on a machine that has only this repository.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
# the reference checkout: $GD_REFERENCE_DIR, else a directory "reference"
# beside this repository
REF_DIR_DEFAULT = os.path.normpath(os.path.join(HERE, "..", "..", "reference"))
ORACLE_SO = os.path.join(HERE, "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libref_weights.so")

# compute_matrix.cu lines holding f1..f4 and calc_matrix_element
REF_WEIGHT_LINES = (21, 257)


def _stale(target: str, sources: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build_oracle(force: bool = False) -> str:
    src = os.path.join(HERE, "oracle.c")
    hdr = os.path.join(HERE, "oracle.h")
    if force or _stale(ORACLE_SO, [src, hdr]):
        cmd = ["gcc", "-std=c11", "-O3", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
               src, "-o", ORACLE_SO + ".tmp", "-lm"]
        subprocess.run(cmd, check=True)
        os.replace(ORACLE_SO + ".tmp", ORACLE_SO)
    return ORACLE_SO


def build_ref(ref_dir: str | None = None, force: bool = False) -> str | None:
    ref_dir = ref_dir or os.environ.get("GD_REFERENCE_DIR", REF_DIR_DEFAULT)
    src = os.path.join(ref_dir, "compute_matrix.cu")
    if not os.path.exists(src):
        return None
    prelude = os.path.join(HERE, "ref_prelude.h")
    epilogue = os.path.join(HERE, "ref_epilogue.cpp")
    if not (force or _stale(REF_SO, [src, prelude, epilogue])):
        return REF_SO
    os.makedirs(os.path.dirname(REF_SO), exist_ok=True)
    with open(src, "r") as fh:
        lines = fh.read().splitlines()
    lo, hi = REF_WEIGHT_LINES
    body = "\n".join(lines[lo - 1:hi])
    with open(prelude) as fh:
        pre = fh.read()
    with open(epilogue) as fh:
        post = fh.read()
    unit = pre + "\n#line %d \"compute_matrix.cu\"\n" % lo + body + "\n" + post
    cmd = ["g++", "-x", "c++", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-",
           "-o", REF_SO + ".tmp", "-lm"]
    subprocess.run(cmd, input=unit.encode(), check=True)
    os.replace(REF_SO + ".tmp", REF_SO)
    return REF_SO


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_ref(force="--force" in sys.argv))
