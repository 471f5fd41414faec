"""Build recipe for the oracle (TEST INFRASTRUCTURE).

* ``oracle/_build/liboracle.so`` and ``oracle/_build/oracle_cli`` - the CPU
  restatement (sbr_oracle.cpp), built on every machine.
* ``oracle/_ref/ref_harness`` - the reference's own sources compiled against
  the Eigen-subset header (build_ref.sh), only where the reference checkout
  is present.

Compiled with -ffp-contract=off so every FP64 product and sum is rounded
separately, as in the reference.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
CLI = os.path.join(HERE, "_build", "oracle_cli")
REF_HARNESS = os.path.join(HERE, "_ref", "ref_harness")


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed: " + " ".join(cmd) + "\n" + r.stdout)


def _fresh(target, sources):
    return os.path.exists(target) and all(
        os.path.getmtime(s) <= os.path.getmtime(target) for s in sources)


def build_oracle(force: bool = False) -> str:
    src = [os.path.join(HERE, f) for f in ("sbr_oracle.cpp", "sbr_oracle.h", "oracle_cli.cpp")]
    if not force and _fresh(LIB, src) and _fresh(CLI, src):
        return LIB
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    cxx = os.environ.get("CXX", "g++")
    flags = ["-std=c++17", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC"]
    jobs = [[cxx, *flags, "-shared", "-o", LIB + ".tmp", src[0], "-lpthread"],
            [cxx, *flags, "-o", CLI + ".tmp", src[2], "-lpthread"]]
    with ThreadPoolExecutor(2) as ex:
        list(ex.map(_run, jobs))
    os.replace(LIB + ".tmp", LIB)
    os.replace(CLI + ".tmp", CLI)
    return LIB


def build_reference(ref: str | None = None) -> str | None:
    """Compiles the reference's own sources from the checkout `ref` (or
    $SBR_REFERENCE_DIR) into oracle/_ref/ref_harness; None when no checkout
    is given or it holds no sources (as on a machine without the reference)."""
    ref = ref or os.environ.get("SBR_REFERENCE_DIR")
    if not ref or not os.path.exists(os.path.join(ref, "SBRSolver_rev2", "RTSolver.cpp")):
        return None
    _run(["bash", os.path.join(HERE, "build_ref.sh"), ref])
    return REF_HARNESS


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if a != "-f"]
    print(build_oracle(force="-f" in sys.argv), build_reference(args[0] if args else None))
