"""Build recipe for the CPU oracle (test infrastructure only).

Compiles ``mcx_oracle.c`` into ``oracle/_build/liboracle.so`` with plain gcc.
``-ffp-contract=off`` keeps every FP64 expression exactly as written (no fused
multiply-add), which the FP64 decisions of the oracle rely on.

The reference (MonteCarloX.jl) is Julia; no Julia toolchain exists on either
machine, so there is no ``oracle/_ref`` build of the reference itself.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")
SRC = os.path.join(HERE, "mcx_oracle.c")
CFLAGS = ["-O2", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
          "-pthread", "-Wall", "-Wextra", "-Wno-unused-parameter"]


def build(force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(
            os.path.getmtime(SRC), os.path.getmtime(os.path.join(HERE, "mcx_oracle.h"))):
        return LIB
    tmp = LIB + ".tmp.%d" % os.getpid()
    cmd = ["gcc", *CFLAGS, "-o", tmp, SRC, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
