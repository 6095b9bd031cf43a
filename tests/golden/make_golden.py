"""Writes golden_first_steps.json: FP64 golden values of the first steps of
the three solver configurations, computed with the oracle (oracle/pcoracle.c)
on the configurations' generators at fixed seeds:

- radial dam break, 9 x 9 patches of 16^2 (the CPU-runnable configuration),
  10 steps;
- uneven mosaic (sizes {8,16,32,64}^2, sum-of-Gaussians bathymetry, the
  batching configuration's generator) on 6 x 6 slots, 3 steps;
- 3-level adaptive breaking dam (ghost interpolation, flux correction and
  restriction every step), base 3, 9^2 cells per patch, 3 steps.

The generators' bathymetry uses exp(), whose last bit can differ between
platforms' math libraries, so every input value is rounded to a multiple of
2^-24 (then exactly the same everywhere); the SHA-256 of the rounded input
is recorded too.  Per case: the dt of every step as hex floats, the SHA-256
of the final packed state's bytes and the sum of the state.  Regenerate with
`python tests/golden/make_golden.py` after a deliberate change of the
oracle's arithmetic."""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from helpers import oracle_amr_patchset, oracle_amr_step, oracle_params, oracle_patchset, oracle_restrict_all  # noqa: E402
from oracle import oracle as O  # noqa: E402
from peanoclaw_gb300 import pcg as P  # noqa: E402
from peanoclaw_gb300 import scenarios as S  # noqa: E402

PRM = P.swe_params(g=9.81, cfl=0.5)


def quantized(ps):
    ps.packed[:] = np.round(ps.packed * 2.0 ** 24) * 2.0 ** -24
    return ps


def input_hash(ps):
    return hashlib.sha256(np.ascontiguousarray(ps.packed, dtype=np.float64).tobytes()).hexdigest()


def cases():
    return {
        "radial_dam_break_9x9x16": (quantized(S.radial_dam_break(npx=9, n=16)), 10, "plain"),
        "uneven_mosaic_6x6": (quantized(S.uneven_patches(grid=6)), 3, "plain"),
        "breaking_dam_3_levels": (quantized(S.breaking_dam_amr(base=3, n=9, levels=3)), 3, "amr"),
    }


def summarize(state, dts):
    return {"dts": [float(d).hex() for d in dts],
            "sha256": hashlib.sha256(np.ascontiguousarray(state, dtype=np.float64).tobytes()).hexdigest(),
            "sum": float(np.sum(state)).hex()}


def oracle_run(ps, steps, kind):
    prm = oracle_params(PRM)
    if kind == "plain":
        pats = oracle_patchset(ps)
        dts = [O.grid_step(pats, ps.items, ps.wall, prm, 1e9)[0] for _ in range(steps)]
    else:
        pats = oracle_amr_patchset(ps)
        oracle_restrict_all(pats, ps)
        dts = [oracle_amr_step(pats, ps, prm, 1e9) for _ in range(steps)]
    return np.concatenate([p.u for p in pats]), dts


def main():
    out = {}
    for name, (ps, steps, kind) in cases().items():
        state, dts = oracle_run(ps, steps, kind)
        out[name] = dict(summarize(state, dts), steps=steps, kind=kind, input_sha256=input_hash(ps))
    with open(os.path.join(HERE, "golden_first_steps.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
        f.write("\n")


if __name__ == "__main__":
    main()
