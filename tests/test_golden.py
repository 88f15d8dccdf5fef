"""Golden trajectory fixtures (tests/golden/, made by tests/golden/make_golden.py): the CPU oracle
reproduces every pinned trajectory from the stored tables, and the host table builder still
produces the stored S=1/2 tables."""

import hashlib
import json
import os

import numpy as np
import pytest

from golden_cases import CASES, load_flat

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden():
    with open(os.path.join(GOLDEN, "trajectories.json")) as f:
        return json.load(f)


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def check_walker(ref, L, n, ctr, num_worms, avg_len, ops, state, sums, counts):
    assert (L, n, ctr) == (ref["L"], ref["n"], ref["rng_counter"])
    assert float(num_worms).hex() == ref["num_worms"] and float(avg_len).hex() == ref["avg_worm_length"]
    assert digest(np.asarray(ops, dtype="<u4")) == ref["ops_sha256"]
    assert digest(np.asarray(state, dtype=np.uint8)) == ref["state_sha256"]
    assert [int(x) for x in counts] == ref["obs_counts"]
    want = np.array([float.fromhex(x) for x in ref["obs_sums"]])
    np.testing.assert_allclose(np.asarray(sums, dtype=float), want, rtol=1e-12, atol=0)


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_reproduces_golden(S, O, name):
    g = golden()[name]
    flat = load_flat(S, os.path.join(GOLDEN, f"model_{name}.npz"))
    om = O.OracleModel(flat)
    for ref in g["walkers"]:
        w = O.OracleWalker(om, T=g["T"], seed=g["seed"], stream=ref["stream"], thermalization=g["therm"])
        w.init()
        w.run(g["sweeps"], measure=True)
        s, c, _ = w.obs()
        check_walker(ref, w.w.L, w.w.num_operators, w.w.ctr, w.w.num_worms, w.w.avg_worm_length, w.ops, w.state,
                     s, c)


@pytest.mark.parametrize("name", ["square8_beta2", "square32_beta16"])
def test_table_builder_matches_stored_spin_half_tables(S, name):
    stored = load_flat(S, os.path.join(GOLDEN, f"model_{name}.npz"))
    built = S.flatten_model(CASES[name]["model"](S))
    assert stored.arrays.keys() == built.arrays.keys()
    for k in stored.arrays:
        assert np.array_equal(stored.arrays[k], built.arrays[k]), k
    assert stored.energy_offset == built.energy_offset and stored.est_prefixes == built.est_prefixes
