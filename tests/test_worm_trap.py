"""Worms that never close.

With S=1 Heisenberg tables some worms wander without reaching their tail for far longer
than any opstring length.  The tables satisfy detailed balance move by move, and the
wandering worm keeps taking random scatter steps (it is not a deterministic cycle), so
no early test can prove that it will never close.  The reference's worm_traverse!
(src/sse.jl:262-303) has no length limit and would run on; the oracle and the
engine stop the walker after 64 * (L + 16) steps with status 8 (worm cap).  This file
pins one such walker on the CPU; the GPU test checks the engine stops it identically
while the other walkers of its batch finish normally."""

import numpy as np
import pytest

TRAP = dict(S=1.0, lattice="bilayer", side=6, beta=8.0, seed=99, stream=7, thermalization=100, sweep=1)


def trap_model(S):
    from sse_gb300.serving import model_params

    return S.flatten_model(S.MagnetModel(model_params(TRAP["S"], TRAP["lattice"], TRAP["side"])))


def test_oracle_stops_trapped_worm(S, O):
    flat = trap_model(S)
    om = O.OracleModel(flat)
    w = O.OracleWalker(om, T=1 / TRAP["beta"], seed=TRAP["seed"], stream=TRAP["stream"], thermalization=TRAP["thermalization"])
    w.init()
    with pytest.raises(RuntimeError):
        for _ in range(10):
            w.step(measure=False)
    assert w.w.status == 8 and w.w.sweeps == TRAP["sweep"]


@pytest.mark.gpu
def test_engine_stops_trapped_walker_like_oracle(S, O):
    from sse_gb300.engine import Engine, SSEError

    flat = trap_model(S)
    eng = Engine(0)
    mid = eng.register_model(flat)
    params = [dict(T=1 / TRAP["beta"], seed=TRAP["seed"], stream=s, thermalization=TRAP["thermalization"])
              for s in (TRAP["stream"], 0, 1, 2)]
    ids = eng.create_walkers(mid, params)
    eng.init(ids)
    with pytest.raises(SSEError) as err:
        eng.sweep(ids, 5, measure=False)
    assert err.value.code == 8
    inf = eng.info(int(ids[0]))
    assert inf["status"] == 8 and inf["sweeps"] == TRAP["sweep"]
    # the trapped walker's opstring and counters match the oracle at the cap
    om = O.OracleModel(flat)
    w = O.OracleWalker(om, T=1 / TRAP["beta"], seed=TRAP["seed"], stream=TRAP["stream"], thermalization=TRAP["thermalization"])
    w.init()
    with pytest.raises(RuntimeError):
        w.run(5, measure=False)
    ops, st, inf = eng.export(int(ids[0]))
    assert inf["rng_counter"] == w.w.ctr and np.array_equal(ops, w.ops)
    # the rest of the batch completed all five sweeps
    for i in ids[1:].tolist():
        assert eng.info(i)["sweeps"] == 5 and eng.info(i)["status"] == 0
    # the stopped walker stays stopped
    with pytest.raises(SSEError):
        eng.sweep(ids[:1], 1)
    eng.close()


def test_oracle_smaller_cap_stops_sooner(S, O):
    """A smaller cap factor ends the same trapped worm after fewer steps."""
    flat = trap_model(S)
    om = O.OracleModel(flat)
    steps = {}
    for factor in (64, 4):
        w = O.OracleWalker(om, T=1 / TRAP["beta"], seed=TRAP["seed"], stream=TRAP["stream"],
                           thermalization=TRAP["thermalization"])
        w.w.worm_cap_factor = factor
        w.init()
        with pytest.raises(RuntimeError):
            w.run(5, measure=False)
        assert w.w.status == 8 and w.w.sweeps == TRAP["sweep"]
        steps[factor] = w.w.worm_steps_total
    assert steps[4] < steps[64]


@pytest.mark.gpu
def test_engine_worm_cap_factor_matches_oracle(S, O):
    from sse_gb300.engine import Engine, SSEError

    flat = trap_model(S)
    eng = Engine(0)
    mid = eng.register_model(flat)
    ids = eng.create_walkers(mid, [dict(T=1 / TRAP["beta"], seed=TRAP["seed"], stream=TRAP["stream"],
                                        thermalization=TRAP["thermalization"])])
    eng.set_worm_cap(ids, 4)
    eng.init(ids)
    with pytest.raises(SSEError):
        eng.sweep(ids, 5, measure=False)
    om = O.OracleModel(flat)
    w = O.OracleWalker(om, T=1 / TRAP["beta"], seed=TRAP["seed"], stream=TRAP["stream"],
                       thermalization=TRAP["thermalization"])
    w.w.worm_cap_factor = 4
    w.init()
    with pytest.raises(RuntimeError):
        w.run(5, measure=False)
    ops, st, inf = eng.export(int(ids[0]))
    assert inf["status"] == 8 and inf["rng_counter"] == w.w.ctr and inf["worm_steps"] == w.w.worm_steps_total
    assert np.array_equal(ops, w.ops)
    with pytest.raises(SSEError):
        eng.set_worm_cap(ids, 0)
    eng.close()
