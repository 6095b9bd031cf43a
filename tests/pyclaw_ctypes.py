"""ctypes binding of libpcg_pyclaw.so the way PeanoClaw's Python package
binds libpeano-claw (src/python/peanoclaw/peano.py:44-134): the library
loaded RTLD_GLOBAL, pyclaw_peano_new with its 28 arguments, callbacks as
CFUNCTYPEs whose array arguments arrive as Python objects (py_object)."""
import ctypes as C

from peanoclaw_gb300 import build as B

# PyClawCallbacks.h: InitializationCallback and AddPatchToSolutionCallback
INIT = C.CFUNCTYPE(C.c_double, C.py_object, C.py_object, C.py_object, C.c_int, C.c_int, C.c_int, C.c_int,
                   C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double, C.c_bool)
ADD = C.CFUNCTYPE(None, C.py_object, C.py_object, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
                  C.c_double, C.c_double, C.c_double)

NEW_ARGTYPES = [C.c_double,                                   # initial mesh width
                C.c_double, C.c_double, C.c_double,           # domain offset
                C.c_double, C.c_double, C.c_double,           # domain size
                C.c_int, C.c_int, C.c_int,                    # subdivision factor
                C.c_int, C.c_int, C.c_int,                    # unknowns, aux fields, ghost layer width
                C.c_double,                                   # initial timestep size
                C.c_char_p, C.c_bool, C.c_bool,               # config file, dim. splitting, reduce reductions
                C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,   # init, boundary, solver, refinement
                C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,   # add to solution, interp., restr., flux
                C.c_bool, C.c_int, C.POINTER(C.c_int)]        # logging, fork level increment, rank


def load():
    B.build()
    lib = C.CDLL(B.PYCLAW_LIB, mode=C.RTLD_GLOBAL)
    lib.pyclaw_peano_new.restype = C.c_void_p
    lib.pyclaw_peano_new.argtypes = NEW_ARGTYPES
    lib.pyclaw_peano_destroy.argtypes = [C.c_void_p]
    lib.pyclaw_peano_evolveToTime.argtypes = [C.c_double, C.c_void_p]
    lib.pyclaw_peano_gatherSolution.argtypes = [C.c_void_p]
    lib.pyclaw_peano_runWorker.argtypes = [C.c_void_p]
    lib.pyclaw_peano_lastError.restype = C.c_char_p
    return lib


def new(lib, width, n, naux, dt0, init_cb, add_cb, lower=(0.0, 0.0), extent=(1.0, 1.0)):
    """pyclaw_peano_new on a 2D domain; returns (runner or None, rank)."""
    rank = C.c_int(-1)
    cast = lambda f: C.cast(f, C.c_void_p) if f is not None else None
    h = lib.pyclaw_peano_new(width, lower[0], lower[1], 0.0, extent[0], extent[1], 0.0, n, n, 0, 3, naux, 1,
                             dt0, b"peanoclaw-config.xml", False, False, cast(init_cb), None, None, None,
                             cast(add_cb), None, None, None, False, 0, C.byref(rank))
    return h, rank.value
