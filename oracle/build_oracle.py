"""Build recipe for the CPU oracle library (test infrastructure only).

Compiles oracle/gsevt_oracle.c into oracle/_build/liboracle.so with gcc.
-ffp-contract=off keeps every multiply and add separately rounded so the FP32
functions follow the operation order written in the source; fmaf() stays fused.
On x86-64 hosts with FMA hardware, -mfma lets gcc inline fmaf() (the result is the
same correctly rounded value either way).
"""
import os
import platform
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")


def _has_x86_fma():
    if platform.machine() not in ("x86_64", "AMD64"):
        return False
    try:
        with open("/proc/cpuinfo") as f:
            return " fma " in f.read()
    except OSError:
        return False


def build(force=False, verbose=False):
    src = os.path.join(HERE, "gsevt_oracle.c")
    inc = os.path.join(HERE, "or_math.inc")
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= max(os.path.getmtime(src), os.path.getmtime(inc))):
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    cmd = ["gcc", "-O2", "-std=c11", "-ffp-contract=off", "-fno-fast-math", "-fopenmp",
           "-fPIC", "-shared", "-o", LIB + ".tmp", src, "-lm"]
    if _has_x86_fma():
        cmd.insert(1, "-mfma")
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
