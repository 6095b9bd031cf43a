"""Compiles the GPU Numerics plugin (peanoclaw_gb300/shim/GpuSWEKernel.cpp)
against the stand-in PeanoClaw headers, together with the test driver
tests/shim/drive_numerics.cpp, into a shared library linked to libpcg.so
(test infrastructure: the shim tests load it with ctypes)."""
import os
import subprocess
import tempfile

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SHIM = os.path.join(ROOT, "peanoclaw_gb300", "shim")


def build(out_dir=None, std="c++17"):
    from peanoclaw_gb300 import build as B
    lib = B.build()
    out_dir = out_dir or tempfile.mkdtemp(prefix="pcg_shim_")
    out = os.path.join(out_dir, "libpcg_shim_test.so")
    cmd = ["g++", "-std=" + std, "-O2", "-Wall", "-Wextra", "-Werror", "-Wno-unused-parameter", "-fPIC", "-shared",
           "-I" + os.path.join(SHIM, "standin"), "-I" + SHIM, "-I" + os.path.join(ROOT, "include"),
           os.path.join(SHIM, "GpuSWEKernel.cpp"), os.path.join(ROOT, "tests", "shim", "drive_numerics.cpp"),
           "-L" + os.path.dirname(lib), "-lpcg", "-Wl,-rpath," + os.path.dirname(lib), "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("shim build failed:\n" + r.stdout + r.stderr)
    return out
