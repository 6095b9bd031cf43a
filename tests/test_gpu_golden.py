"""The CUDA path (batched form) against the committed golden first steps of
the three solver configurations (tests/golden/golden_first_steps.json):
same dts and the same state bytes (SHA-256), without running the oracle."""
import numpy as np
import pytest

from helpers import gpu_patchset, slab_for
from peanoclaw_gb300 import pcg as P
from peanoclaw_gb300 import scenarios as S
from test_golden import load_golden

pytestmark = pytest.mark.gpu


def test_gpu_reproduces_the_golden_first_steps():
    mod, gold = load_golden()
    for name, (ps, steps, kind) in mod.cases().items():
        assert mod.input_hash(ps) == gold[name]["input_sha256"], name + ": inputs differ on this platform"
        c = P.Context(slab_doubles=max(slab_for(ps), 4_000_000), max_patches=len(ps) + 8, max_groups=1,
                      params=mod.PRM)
        try:
            if kind == "plain":
                ids = gpu_patchset(c, ps)
            else:
                ids = S.install_amr(c, ps)
                c.restrict_all()
            c.set_group_max_dt(0, 1e9)
            dts = list(c.run(steps, P.PCG_MODE_BATCHED)[:, 0])
            state = c.download_many(ids, int(ps.packed.size))
        finally:
            c.close()
        assert mod.summarize(state, dts) == {k: gold[name][k] for k in ("dts", "sha256", "sum")}, name
