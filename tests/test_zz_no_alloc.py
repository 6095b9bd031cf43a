"""The allocation-free single-patch solve against the context-based one.

pcg_solve_timestep_noalloc serves callers that cannot call cudaMalloc (they
work on a patch buffer someone else allocated and must not allocate device
memory themselves, so they cannot create a pcg_context either).  Here the test
plays such a caller: it owns the patch buffer (allocated up front with torch),
calls the entry point through the C ABI twice in a row, and checks state, dt
and estimate bit for bit (the tolerance of every parity test here) against
pcg_solve_timestep on the same input.  This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

from helpers import random_swe_vector

pytestmark = pytest.mark.gpu


def test_noalloc_solve_matches_context_solve_two_calls():
    import torch

    from peanoclaw_gb300 import pcg as P

    prm = P.swe_params(g=9.81, cfl=0.5)
    ctx = P.Context(slab_doubles=2_000_000, max_patches=8, max_groups=1, params=prm)
    try:
        for n, max_dt in ((16, 1e9), (27, 1e-3), (64, 1e9)):
            rng = np.random.default_rng(500 + n)
            vec = random_swe_vector(rng, n)
            size = (0.125, 0.125)
            pid = ctx.alloc(n, pos=(0.0, 0.0), size=size)
            ctx.upload(pid, vec)
            dev = torch.from_numpy(vec.copy()).to("cuda")
            torch.cuda.synchronize()
            sz = (C.c_double * 2)(*size)
            for _ in range(2):
                dt_a, est_a = C.c_double(), C.c_double()
                P.check(P.lib().pcg_solve_timestep(ctx.h, pid, max_dt, C.byref(dt_a), C.byref(est_a)))
                dt_b, est_b = C.c_double(), C.c_double()
                P.check(P.lib().pcg_solve_timestep_noalloc(
                    C.c_void_p(dev.data_ptr()), n, n, sz, C.byref(prm), max_dt,
                    C.byref(dt_b), C.byref(est_b), None))
                torch.cuda.synchronize()
                assert dt_a.value == dt_b.value
                assert est_a.value == est_b.value
                got = dev.cpu().numpy()
                ref = ctx.download(pid, vec.size)
                assert np.array_equal(got, ref)
                assert np.array_equal(np.signbit(got), np.signbit(ref))
            ctx.free(pid)
        # sizes beyond the fixed scratch are rejected, nothing is launched
        big = torch.zeros(P.vector_size(129), dtype=torch.float64, device="cuda")
        rc = P.lib().pcg_solve_timestep_noalloc(C.c_void_p(big.data_ptr()), 129, 129,
                                                (C.c_double * 2)(1.0, 1.0), C.byref(prm), 1.0,
                                                None, None, None)
        assert rc == P.PCG_E_INVALID
        assert b"16384" in P.lib().pcg_last_error()
    finally:
        ctx.close()
