"""The allocation-free single-patch solve against the context-based one and
against the oracle.

pcg_solve_timestep_noalloc serves callers that cannot call cudaMalloc (they
work on a patch buffer someone else allocated and must not allocate device
memory themselves, so they cannot create a pcg_context either).  Here the test
plays such a caller: it owns the patch buffer (allocated up front with torch),
calls the entry point through the C ABI twice in a row, and checks state, dt
and estimate bit for bit (the tolerance of every parity test here) against
pcg_solve_timestep on the same input.  Patches above what the context solve
takes in shared memory (about 90 x 90 cells), up to the fixed scratch's
128 x 128 and non-square shapes within it, are checked against the oracle's
single-patch solve instead.  This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

from helpers import oracle_params, random_swe_vector

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


@pytest.mark.parametrize("nx,ny", [(128, 128), (200, 80), (80, 200)])
def test_noalloc_solve_beyond_context_sizes_matches_oracle(nx, ny):
    """Shapes the context solve cannot take (its net updates live in shared
    memory), up to the scratch limit nx * ny <= 16384, two calls in a row."""
    import torch

    from oracle import oracle as O
    from peanoclaw_gb300 import pcg as P

    prm = P.swe_params(g=9.81, cfl=0.5)
    rng = np.random.default_rng(7000 + nx + ny)
    vec = random_swe_vector(rng, (nx, ny))
    size = (0.5, 0.25)
    dev = torch.from_numpy(vec.copy()).to("cuda")
    torch.cuda.synchronize()
    op = O.Patch((nx, ny), size=size)
    op.u[:] = vec
    sz = (C.c_double * 2)(*size)
    for max_dt in (1e9, 1e-4):
        dt_b, est_b = C.c_double(), C.c_double()
        P.check(P.lib().pcg_solve_timestep_noalloc(C.c_void_p(dev.data_ptr()), nx, ny, sz, C.byref(prm),
                                                   max_dt, C.byref(dt_b), C.byref(est_b), None))
        dt_o, est_o = C.c_double(), C.c_double()
        O.lib().pco_swe_solve_timestep(C.byref(op.s), C.byref(oracle_params(prm)), max_dt,
                                       C.byref(dt_o), C.byref(est_o))
        torch.cuda.synchronize()
        assert dt_b.value == dt_o.value
        assert est_b.value == est_o.value
        got = dev.cpu().numpy()
        assert np.array_equal(got, op.u)
        assert np.array_equal(np.signbit(got), np.signbit(op.u))


def test_noalloc_rejects_host_outputs_under_capture():
    """While the stream is being captured, the read-back of dt_used / est_next
    (a copy and a stream synchronisation) is refused before anything is
    enqueued, so the capture stays valid."""
    import torch

    from peanoclaw_gb300 import pcg as P

    prm = P.swe_params(g=9.81, cfl=0.5)
    n = 16
    vec = random_swe_vector(np.random.default_rng(11), n)
    dev = torch.from_numpy(vec.copy()).to("cuda")
    sz = (C.c_double * 2)(0.125, 0.125)
    # the first call in this context resolves the scratch address outside capture
    P.check(P.lib().pcg_solve_timestep_noalloc(C.c_void_p(dev.data_ptr()), n, n, sz, C.byref(prm), 1e9,
                                               None, None, None))
    torch.cuda.synchronize()
    side = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    dt = C.c_double()
    with torch.cuda.graph(g, stream=side):
        rc = P.lib().pcg_solve_timestep_noalloc(C.c_void_p(dev.data_ptr()), n, n, sz, C.byref(prm), 1e9,
                                                C.byref(dt), None, C.c_void_p(side.cuda_stream))
        dev.add_(0.0)
    assert rc == P.PCG_E_INVALID
    assert b"captured" in P.lib().pcg_last_error()
