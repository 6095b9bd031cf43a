"""The C-ABI library loads and exports every symbol include/pcg.h declares (CPU)."""
import ctypes as C
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "pcg.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(pcg_[a-z0-9_]+)\s*\(", txt)))


def test_header_symbols_exported():
    from peanoclaw_gb300 import pcg
    lib = C.CDLL(pcg.LIB_PATH)
    syms = declared_symbols()
    assert len(syms) >= 30
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing


def test_binding_covers_header():
    from peanoclaw_gb300 import pcg
    assert sorted(pcg.SIGNATURES) == declared_symbols()


def test_vector_size_matches_reference_layout():
    from peanoclaw_gb300 import pcg
    from oracle import oracle as O
    for n, g, nq, pwo, pw in [(16, 1, 3, 0, 1), (27, 1, 3, 0, 1), (2, 2, 1, 0, 0), (5, 2, 4, 1, 2)]:
        d = pcg.PatchDesc(n, n, g, nq, pwo, pw, 0, 1, (C.c_double * 2)(0, 0), (C.c_double * 2)(1, 1))
        p = O.Patch(n, ghost=g, nq=nq, np_wo=pwo, np_w=pw)
        assert pcg.lib().pcg_patch_vector_size(C.byref(d)) == p.u.size == pcg.vector_size(n, g, nq, pwo, pw)


def test_no_gpu_errors_are_reported_not_raised():
    """Without a device, pcg_create fails with an error code and a message."""
    import torch
    if torch.cuda.is_available():
        return
    from peanoclaw_gb300 import pcg
    cfg = pcg.Config()
    cfg.device, cfg.max_patches, cfg.max_groups, cfg.slab_doubles = 0, 4, 1, 1024
    cfg.params = pcg.swe_params()
    h = C.c_void_p()
    rc = pcg.lib().pcg_create(C.byref(cfg), C.byref(h))
    assert rc != 0
    assert len(pcg.lib().pcg_last_error()) > 0


def test_header_compiles_and_links_from_c_and_cpp(tmp_path):
    """include/pcg.h is a plain C99 header (and usable from C++): a caller
    that takes the address of every declared entry point compiles without
    warnings, links against the library and runs (no device call)."""
    import shutil
    import subprocess
    import pytest
    from peanoclaw_gb300 import pcg
    syms = declared_symbols()
    body = "".join('  printf("%%p\\n", (void *)%s);\n' % s for s in syms)
    for compiler, std, ext in (("gcc", "-std=c99", "c"), ("g++", "-std=c++11", "cpp")):
        if shutil.which(compiler) is None:
            pytest.skip(compiler + " not available")
        src = tmp_path / ("caller." + ext)
        src.write_text('#include "pcg.h"\n#include <stdio.h>\nint main(void) {\n' + body + "  return 0;\n}\n")
        exe = tmp_path / ("caller_" + ext)
        subprocess.run([compiler, std, "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
                        str(src), pcg.LIB_PATH, "-o", str(exe)], check=True, capture_output=True)
        out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()
        assert len(out) == len(syms)
