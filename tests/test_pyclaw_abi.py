"""The PyClaw C interface (libpcg_pyclaw.so): the library exports every
pyclaw_peano_* function that include/pcg_pyclaw.h declares, links against
libpcg.so, and the header compiles as C99 and C++11; no GPU needed."""
import os
import re
import subprocess

import pytest

from peanoclaw_gb300 import build as B

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "pcg_pyclaw.h")


def _declared():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"\b(pyclaw_peano_\w+)\s*\(", text)))


def test_library_exports_every_declared_function():
    B.build()
    names = _declared()
    # the reference's six (pyclawBindings.cpp) plus the two additions
    assert set(names) >= {"pyclaw_peano_new", "pyclaw_peano_destroy", "pyclaw_peano_evolveToTime",
                          "pyclaw_peano_gatherSolution", "pyclaw_peano_runTests",
                          "pyclaw_peano_runWorker"}
    syms = subprocess.run(["nm", "-D", "--defined-only", B.PYCLAW_LIB], capture_output=True,
                          text=True, check=True).stdout.split()
    for n in names:
        assert n in syms, n
    needed = subprocess.run(["readelf", "-d", B.PYCLAW_LIB], capture_output=True, text=True,
                            check=True).stdout
    assert "libpcg.so" in needed and "$ORIGIN" in needed


@pytest.mark.parametrize("lang,std", [("c", "c99"), ("c++", "c++11")])
def test_header_compiles(tmp_path, lang, std):
    src = tmp_path / ("t.c" if lang == "c" else "t.cpp")
    src.write_text('#include "pcg_pyclaw.h"\n'
                   "void *(*p_new)(double, double, double, double, double, double, double, int, int, int,\n"
                   "               int, int, int, double, char *, bool, bool, void *, void *, void *, void *,\n"
                   "               void *, void *, void *, void *, bool, int, int *) = pyclaw_peano_new;\n"
                   "void (*p_evolve)(double, void *) = pyclaw_peano_evolveToTime;\n"
                   "void (*p_gather)(void *) = pyclaw_peano_gatherSolution;\n"
                   "void (*p_destroy)(void *) = pyclaw_peano_destroy;\n"
                   "int (*p_worker)(void *) = pyclaw_peano_runWorker;\n")
    cc = "gcc" if lang == "c" else "g++"
    r = subprocess.run([cc, "-std=" + std, "-Wall", "-Werror", "-c", str(src), "-I", os.path.dirname(HEADER),
                        "-o", str(tmp_path / "t.o")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_initialization_callbacks_through_ctypes():
    """pyclaw_peano_new hands every subgrid's q, qbc and aux to the
    initialization callback as writable numpy arrays of the reference's
    shapes, with the subgrid's size and position, before it touches the GPU
    (without one it then fails with the reason)."""
    import pyclaw_ctypes as PC

    lib = PC.load()
    seen = []

    def init(q, qbc, aux, n0, n1, n2, nq, naux, sx, sy, sz, px, py, pz, skip):
        seen.append((q.shape, qbc.shape, aux.shape, n0, n1, n2, nq, naux, sx, sy, px, py, skip))
        q[0] = 1.0 + px
        aux[0] = py
        return sx

    cb = PC.INIT(init)
    h, rank = PC.new(lib, 0.5, 4, 1, 1e-3, cb, None, lower=(-1.0, 2.0), extent=(1.0, 1.5))
    try:
        assert len(seen) == 2 * 3
        pos = sorted((s[10], s[11]) for s in seen)
        assert pos == sorted((-1.0 + 0.5 * i, 2.0 + 0.5 * j) for i in range(2) for j in range(3))
        for s in seen:
            assert s[:3] == ((3, 4, 4), (3, 6, 6), (1, 4, 4))
            assert s[3:10] == (4, 4, 0, 3, 1, 0.5, 0.5) and s[12] is False
        if not h:
            assert b"pcg_create" in lib.pyclaw_peano_lastError()
        else:
            assert rank == 0
    finally:
        if h:
            lib.pyclaw_peano_destroy(h)
    # shapes the GPU kernel does not take are refused before any callback
    seen.clear()
    h, _ = PC.new(lib, 0.5, 4, 2, 1e-3, cb, None)
    assert not h and not seen and b"aux" in lib.pyclaw_peano_lastError()
