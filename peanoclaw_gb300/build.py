"""Builds libpcg.so (the CUDA kernels + C ABI) for sm_103a, in-tree.

The shared library is written to peanoclaw_gb300/_lib/libpcg.so.  Translation
units are compiled in parallel with nvcc; -fmad=false keeps every FP64
operation exactly as written (fused multiply-adds are explicit __fma_rn).
libpcg_pyclaw.so (the pyclaw_peano_* C interface, host C++ only) is linked
against it beside it.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT, "libpcg.so")
PYCLAW_LIB = os.path.join(OUT, "libpcg_pyclaw.so")
PYCLAW_SOURCE = "pcg_pyclaw.cpp"
SOURCES = ["pcg_kernels.cu", "pcg_strips.cu", "pcg_fused.cu", "pcg_pipeline.cu", "pcg_api.cu", "pcg_amr.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-Xcompiler", "-fPIC",
         "-Xptxas", "-warn-spills"]


def _nvcc():
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def _stale():
    if not os.path.exists(LIB) or not os.path.exists(PYCLAW_LIB):
        return True
    t = min(os.path.getmtime(LIB), os.path.getmtime(PYCLAW_LIB))
    inc = os.path.join(os.path.dirname(HERE), "include")
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps += [os.path.join(inc, f) for f in ("pcg.h", "pcg_pyclaw.h")]
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build_pyclaw():
    """libpcg_pyclaw.so: plain g++, linked to libpcg.so through $ORIGIN."""
    tmp = PYCLAW_LIB + ".tmp"
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-fPIC", "-shared",
           os.path.join(CSRC, PYCLAW_SOURCE), "-o", tmp, "-L" + OUT, "-lpcg",
           "-Wl,-rpath,$ORIGIN", "-ldl"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("g++ failed for %s:\n%s%s" % (PYCLAW_SOURCE, r.stdout, r.stderr))
    os.replace(tmp, PYCLAW_LIB)
    return PYCLAW_LIB


def build(force=False, verbose=False):
    if not force and not _stale():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()

    def compile_one(src):
        obj = os.path.join(OUT, os.path.splitext(src)[0] + ".o")
        cmd = [nvcc, *ARCH, *FLAGS, "-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s%s" % (src, r.stdout, r.stderr))
        if verbose and (r.stdout or r.stderr):
            sys.stderr.write(r.stdout + r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB + ".tmp"
    cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    build_pyclaw()
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
