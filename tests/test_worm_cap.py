"""Worms that outrun the length cap.

With S=1 Heisenberg tables the first thermalisation sweeps, while the cutoff L is still
small, can run worms that are orders of magnitude longer than the opstring.  They close
in the end, but the tail is heavy (over 10^9 steps in some chains).  The reference's
worm_traverse! (src/sse.jl:262-303) has no length limit and runs such a worm to its end;
the oracle and the engine stop the walker after 64 * (L + 16) steps with status 8 (worm
cap).  This file pins one such walker on the CPU, checks that the same worm closes under
a larger cap, and on the GPU checks that the engine stops it identically while the other
walkers of its batch finish normally."""

import numpy as np
import pytest

LONG_WORM = dict(S=1.0, lattice="bilayer", side=6, beta=8.0, seed=99, stream=7, thermalization=100, sweep=1)


def long_worm_model(S):
    from sse_gb300.serving import model_params

    return S.flatten_model(S.MagnetModel(model_params(LONG_WORM["S"], LONG_WORM["lattice"], LONG_WORM["side"])))


def test_oracle_stops_long_worm_at_cap(S, O):
    flat = long_worm_model(S)
    om = O.OracleModel(flat)
    w = O.OracleWalker(om, T=1 / LONG_WORM["beta"], seed=LONG_WORM["seed"], stream=LONG_WORM["stream"], thermalization=LONG_WORM["thermalization"])
    w.init()
    with pytest.raises(RuntimeError):
        for _ in range(10):
            w.step(measure=False)
    assert w.w.status == 8 and w.w.sweeps == LONG_WORM["sweep"]


@pytest.mark.gpu
def test_engine_stops_long_worm_walker_like_oracle(S, O):
    from sse_gb300.engine import Engine, SSEError

    flat = long_worm_model(S)
    eng = Engine(0)
    mid = eng.register_model(flat)
    params = [dict(T=1 / LONG_WORM["beta"], seed=LONG_WORM["seed"], stream=s, thermalization=LONG_WORM["thermalization"])
              for s in (LONG_WORM["stream"], 0, 1, 2)]
    ids = eng.create_walkers(mid, params)
    eng.init(ids)
    with pytest.raises(SSEError) as err:
        eng.sweep(ids, 5, measure=False)
    assert err.value.code == 8
    inf = eng.info(int(ids[0]))
    assert inf["status"] == 8 and inf["sweeps"] == LONG_WORM["sweep"]
    # the stopped walker's opstring and counters match the oracle at the cap
    om = O.OracleModel(flat)
    w = O.OracleWalker(om, T=1 / LONG_WORM["beta"], seed=LONG_WORM["seed"], stream=LONG_WORM["stream"], thermalization=LONG_WORM["thermalization"])
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


def test_oracle_stopped_worm_closes_under_larger_cap(S, O):
    """The stopped worm is long, not endless: at 64 * (L + 16) = 139,968 steps it is cut off, and
    with a cap of 1000 * (L + 16) the same trajectory closes it and sweeps on."""
    flat = long_worm_model(S)
    om = O.OracleModel(flat)
    w = O.OracleWalker(om, T=1 / LONG_WORM["beta"], seed=LONG_WORM["seed"], stream=LONG_WORM["stream"],
                       thermalization=LONG_WORM["thermalization"])
    w.w.worm_cap_factor = 1000
    w.init()
    w.run(3, measure=False)
    assert w.w.status == 0 and w.w.sweeps == 3
    assert w.w.worm_steps_total > 64 * (2171 + 16)
    assert w.state.shape == (flat.nsites,)


def test_oracle_smaller_cap_stops_sooner(S, O):
    """A smaller cap factor ends the same long worm after fewer steps."""
    flat = long_worm_model(S)
    om = O.OracleModel(flat)
    steps = {}
    for factor in (64, 4):
        w = O.OracleWalker(om, T=1 / LONG_WORM["beta"], seed=LONG_WORM["seed"], stream=LONG_WORM["stream"],
                           thermalization=LONG_WORM["thermalization"])
        w.w.worm_cap_factor = factor
        w.init()
        with pytest.raises(RuntimeError):
            w.run(5, measure=False)
        assert w.w.status == 8 and w.w.sweeps == LONG_WORM["sweep"]
        steps[factor] = w.w.worm_steps_total
    assert steps[4] < steps[64]


@pytest.mark.gpu
def test_engine_worm_cap_factor_matches_oracle(S, O):
    from sse_gb300.engine import Engine, SSEError

    flat = long_worm_model(S)
    eng = Engine(0)
    mid = eng.register_model(flat)
    ids = eng.create_walkers(mid, [dict(T=1 / LONG_WORM["beta"], seed=LONG_WORM["seed"], stream=LONG_WORM["stream"],
                                        thermalization=LONG_WORM["thermalization"])])
    eng.set_worm_cap(ids, 4)
    eng.init(ids)
    with pytest.raises(SSEError):
        eng.sweep(ids, 5, measure=False)
    om = O.OracleModel(flat)
    w = O.OracleWalker(om, T=1 / LONG_WORM["beta"], seed=LONG_WORM["seed"], stream=LONG_WORM["stream"],
                       thermalization=LONG_WORM["thermalization"])
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
