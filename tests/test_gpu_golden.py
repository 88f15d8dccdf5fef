"""The GPU engine reaches every pinned golden trajectory (tests/golden/) from the stored tables,
without running the oracle."""

import os

import pytest

from golden_cases import load_flat
from test_golden import GOLDEN, check_walker, golden

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng():
    from sse_gb300.engine import Engine

    e = Engine(0)
    yield e
    e.close()


@pytest.mark.parametrize("name", sorted(golden()))
def test_engine_reaches_golden(S, eng, name):
    g = golden()[name]
    flat = load_flat(S, os.path.join(GOLDEN, f"model_{name}.npz"))
    mid = eng.register_model(flat)
    ids = eng.create_walkers(mid, [dict(T=g["T"], seed=g["seed"], stream=r["stream"], thermalization=g["therm"])
                                   for r in g["walkers"]])
    eng.init(ids)
    eng.sweep(ids, g["sweeps"], measure=True)
    for ref, wid in zip(g["walkers"], ids.tolist()):
        ops, st, inf = eng.export(wid)
        s, c, _ = eng.observables([wid])[0]
        check_walker(ref, inf["L"], inf["num_operators"], inf["rng_counter"], inf["num_worms"],
                     inf["avg_worm_length"], ops, st, s, c)
