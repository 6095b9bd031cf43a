"""Build recipe for the oracle (test infrastructure only).

Compiles oracle/pcoracle.c into oracle/_build/libpcoracle.so with
-ffp-contract=off (so every fused multiply-add is an explicit fma() call) and
OpenMP (for the timed CPU baseline).  The reference's own SWE path cannot be
compiled (Peano 3, the TUM SWE sources and scons are absent), so there is no
oracle/_ref build.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libpcoracle.so")


def build(force=False):
    src = os.path.join(HERE, "pcoracle.c")
    hdr = os.path.join(HERE, "pcoracle.h")
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= max(os.path.getmtime(src), os.path.getmtime(hdr))):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    cmd = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off",
           "-fno-fast-math", "-fopenmp", "-Wall", "-o", LIB + ".tmp", src, "-lm"]
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
