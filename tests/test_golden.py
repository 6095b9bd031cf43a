"""Golden first steps (tests/golden/golden_first_steps.json, written by
tests/golden/make_golden.py): the oracle reproduces the committed dts, state
hash and sums of the three solver configurations' first steps."""
import importlib.util
import json
import os

HERE = os.path.dirname(os.path.abspath(__file__))


def load_golden():
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(HERE, "golden", "make_golden.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    with open(os.path.join(HERE, "golden", "golden_first_steps.json")) as f:
        return mod, json.load(f)


def test_oracle_reproduces_the_golden_first_steps():
    mod, gold = load_golden()
    cases = mod.cases()
    assert set(cases) == set(gold)
    for name, (ps, steps, kind) in cases.items():
        assert mod.input_hash(ps) == gold[name]["input_sha256"], name + ": inputs differ on this platform"
        state, dts = mod.oracle_run(ps, steps, kind)
        assert mod.summarize(state, dts) == {k: gold[name][k] for k in ("dts", "sha256", "sum")}, name
