"""Build recipe for the oracle (test infrastructure only).

Compiles oracle/pcoracle.c (the FP64 restatement) and oracle/pcoracle_f32.c
(its FP32 twin, a timing baseline at the reference's float precision) into
oracle/_build/libpcoracle.so with -ffp-contract=off (so every fused
multiply-add is an explicit fma() call) and OpenMP (for the timed CPU
baseline).  The reference's own SWE path cannot be
compiled (Peano 3, the TUM SWE sources and scons are absent), so there is no
oracle/_ref build.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libpcoracle.so")


def build(force=False):
    srcs = [os.path.join(HERE, "pcoracle.c"), os.path.join(HERE, "pcoracle_f32.c")]
    hdr = os.path.join(HERE, "pcoracle.h")
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= max(os.path.getmtime(f) for f in srcs + [hdr])):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    cmd = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off",
           "-fno-fast-math", "-fopenmp", "-Wall", "-o", LIB + ".tmp"] + srcs + ["-lm"]
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
