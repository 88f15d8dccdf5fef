"""Worms that outrun the length cap.

With S=1 Heisenberg tables the first thermalisation sweeps, while the cutoff L is still
small, can run worms that are orders of magnitude longer than the opstring.  They close
in the end, but the tail is heavy (over 10^9 steps in some chains).  The reference's
worm_traverse! (src/sse.jl:262-303) has no length limit and runs such a worm to its end.
The oracle and the engine cap a worm at factor * max(L + 16, 65536) steps (factor 64 by
default, so at least about 4.2 million steps):

* during thermalisation the sweep's worm phase is undone: the opstring returns to its state
  after the diagonal update, the worm-count controller and the spin state stay as they were,
  and the walker goes on (thermalisation sweeps need no detailed balance);
* after thermalisation the walker stops with status 8 (worm cap).

This file pins one such walker on the CPU in both phases, with the cap lowered (factor 2) so that
it cuts the worm; checks that the same worm closes under the default cap and that chains thermalised
with many undone sweeps still sample the ED values; and on the GPU checks that the engine does
exactly what the oracle does."""

import numpy as np
import pytest

# the walker's second sweep (sweeps == 1) runs a worm of 145,785 steps; with the cap factor FACTOR
# the cap is 2 * max(2171 + 16, 65536) = 131,072 steps, so the cap cuts it
LONG_WORM = dict(S=1.0, lattice="bilayer", side=6, beta=8.0, seed=99, stream=7, sweep=1)
FACTOR = 2
CAP = FACTOR * 65536
MEASURED = 0  # thermalization: the long worm falls in a measured sweep and stops the walker
THERMALISING = 100  # thermalization: the long worm's sweep is undone


def long_worm_model(S):
    from sse_gb300.serving import model_params

    return S.flatten_model(S.MagnetModel(model_params(LONG_WORM["S"], LONG_WORM["lattice"], LONG_WORM["side"])))


def oracle_walker(O, om, thermalization, factor=FACTOR):
    w = O.OracleWalker(om, T=1 / LONG_WORM["beta"], seed=LONG_WORM["seed"], stream=LONG_WORM["stream"],
                       thermalization=thermalization)
    if factor is not None:
        w.w.worm_cap_factor = factor
    w.init()
    return w


def test_oracle_stops_long_worm_in_measured_sweep(S, O):
    om = O.OracleModel(long_worm_model(S))
    w = oracle_walker(O, om, MEASURED)
    with pytest.raises(RuntimeError):
        w.run(10, measure=False)
    assert w.w.status == 8 and w.w.sweeps == LONG_WORM["sweep"] and w.w.worm_undos == 0


def test_oracle_undoes_long_worm_in_thermalisation(S, O):
    """The sweep's worm phase is undone: the opstring is again the diagonal update's, and the spin
    state, operator count and worm-count controller are those before the worm phase; the draws
    the worm consumed stay consumed."""
    from test_oracle import isconsistent

    flat = long_worm_model(S)
    om = O.OracleModel(flat)
    w = oracle_walker(O, om, THERMALISING)
    w.run(LONG_WORM["sweep"], measure=False)
    w.diagonal_update(thermalized=False)
    w.make_vertex_list()
    ops, st, before = w.ops, w.state, w.scalars()
    w.worm_update(thermalized=False)
    after = w.scalars()
    assert w.w.worm_undos == 1 and after["status"] == 0
    assert np.array_equal(w.ops, ops) and np.array_equal(w.state, st) and isconsistent(flat, w.ops, w.state)
    for k in ("L", "n", "num_worms", "avg_worm_length"):
        assert after[k] == before[k], k
    assert after["ctr"] > before["ctr"] + CAP
    # the same walker through whole Carlo steps: one undone sweep, then it sweeps on
    w = oracle_walker(O, om, THERMALISING)
    w.run(5, measure=False)
    assert w.w.status == 0 and w.w.sweeps == 5 and w.w.worm_undos == 1
    assert isconsistent(flat, w.ops, w.state)


def test_oracle_long_worm_closes_under_the_default_cap(S, O):
    """The worm is long, not endless: the lowered cap cuts it, and under the default cap
    (64 * 65536 steps here) the same trajectory closes it and sweeps on."""
    flat = long_worm_model(S)
    w = oracle_walker(O, O.OracleModel(flat), MEASURED, factor=64)
    w.run(3, measure=False)
    assert w.w.status == 0 and w.w.sweeps == 3 and w.w.worm_undos == 0
    assert w.w.worm_steps_total > 145_785


def test_oracle_smaller_cap_stops_sooner(S, O):
    """A smaller cap factor ends the same long worm after fewer steps."""
    om = O.OracleModel(long_worm_model(S))
    steps = {}
    for factor in (FACTOR, 1):
        w = oracle_walker(O, om, MEASURED, factor=factor)
        with pytest.raises(RuntimeError):
            w.run(5, measure=False)
        assert w.w.status == 8 and w.w.sweeps == LONG_WORM["sweep"]
        steps[factor] = w.w.worm_steps_total
    assert steps[1] < steps[FACTOR]


def test_oracle_chains_with_undone_sweeps_sample_the_same_distribution(S, O):
    """Chains of the S=1 bilayer thermalised under the lowest cap (factor 1: 65,536 steps), where
    about one chain in five undoes a thermalisation sweep, then measured under the default cap,
    give the same mean operator count (and so energy) as independent chains thermalised under the
    default cap: |difference| <= 4 standard errors."""
    flat = long_worm_model(S)
    om = O.OracleModel(flat)
    therm, sweeps, nchains = 100, 300, 32

    def chain_means(first_stream, factor):
        means, undos = [], 0
        for k in range(nchains):
            w = O.OracleWalker(om, T=1 / LONG_WORM["beta"], seed=7, stream=first_stream + k, thermalization=therm)
            w.w.worm_cap_factor = factor
            w.init()
            w.run(therm, measure=False)
            undos += w.w.worm_undos
            w.w.worm_cap_factor = 64
            w.run(sweeps, measure=True)
            s, c, _ = w.obs()
            means.append(s[1] / c[1])  # OperatorCount
            assert w.w.status == 0
        return np.array(means), undos

    lowered, undos = chain_means(0, 1)
    default, undos_default = chain_means(1000, 64)
    assert undos >= 3 and undos > undos_default  # the longest thermalisation worms pass even the default cap
    diff = lowered.mean() - default.mean()
    err = np.sqrt(lowered.var(ddof=1) / nchains + default.var(ddof=1) / nchains)
    assert abs(diff) <= 4 * err, (diff, err)


@pytest.mark.gpu
def test_engine_stops_long_worm_walker_like_oracle(S, O):
    from sse_gb300.engine import Engine, SSEError

    flat = long_worm_model(S)
    eng = Engine(0)
    mid = eng.register_model(flat)
    params = [dict(T=1 / LONG_WORM["beta"], seed=LONG_WORM["seed"], stream=s, thermalization=MEASURED)
              for s in (LONG_WORM["stream"], 0, 1, 2)]
    ids = eng.create_walkers(mid, params)
    eng.set_worm_cap(ids, FACTOR)
    eng.init(ids)
    with pytest.raises(SSEError) as err:
        eng.sweep(ids, 5, measure=False)
    assert err.value.code == 8
    inf = eng.info(int(ids[0]))
    assert inf["status"] == 8 and inf["sweeps"] == LONG_WORM["sweep"] and inf["worm_undos"] == 0
    # the stopped walker's opstring and counters match the oracle at the cap
    w = oracle_walker(O, O.OracleModel(flat), MEASURED)
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


@pytest.mark.gpu
@pytest.mark.parametrize("staging", [0, 192 * 1024])
def test_engine_undoes_long_worm_like_oracle(S, O, staging):
    """During thermalisation the engine undoes the long worm's sweep exactly as the oracle does
    (records chased in HBM, and staged in shared memory: about 1,700 operators, 55 KB of records,
    in the undone sweep), and the walker sweeps on bit for bit."""
    flat = long_worm_model(S)
    from sse_gb300.engine import Engine

    eng = Engine(0)
    eng.set_staging(staging)
    mid = eng.register_model(flat)
    ids = eng.create_walkers(mid, [dict(T=1 / LONG_WORM["beta"], seed=LONG_WORM["seed"], stream=s,
                                        thermalization=THERMALISING) for s in (LONG_WORM["stream"], 0)])
    eng.set_worm_cap(ids, FACTOR)
    eng.init(ids)
    eng.sweep(ids, 5, measure=False)
    w = oracle_walker(O, O.OracleModel(flat), THERMALISING)
    w.run(5, measure=False)
    ops, st, inf = eng.export(int(ids[0]))
    assert inf["status"] == 0 and inf["sweeps"] == 5 and inf["worm_undos"] == w.w.worm_undos == 1
    assert inf["rng_counter"] == w.w.ctr and inf["worm_steps"] == w.w.worm_steps_total
    assert inf["num_worms"] == w.w.num_worms and inf["avg_worm_length"] == w.w.avg_worm_length
    assert np.array_equal(ops, w.ops) and np.array_equal(st, w.state)
    assert eng.check(ids).tolist() == [0, 0]
    eng.close()


@pytest.mark.gpu
def test_engine_worm_cap_factor_matches_oracle(S, O):
    from sse_gb300.engine import Engine, SSEError

    flat = long_worm_model(S)
    eng = Engine(0)
    mid = eng.register_model(flat)
    ids = eng.create_walkers(mid, [dict(T=1 / LONG_WORM["beta"], seed=LONG_WORM["seed"], stream=LONG_WORM["stream"],
                                        thermalization=MEASURED)])
    eng.set_worm_cap(ids, 1)
    eng.init(ids)
    with pytest.raises(SSEError):
        eng.sweep(ids, 5, measure=False)
    w = oracle_walker(O, O.OracleModel(flat), MEASURED, factor=1)
    with pytest.raises(RuntimeError):
        w.run(5, measure=False)
    ops, st, inf = eng.export(int(ids[0]))
    assert inf["status"] == 8 and inf["rng_counter"] == w.w.ctr and inf["worm_steps"] == w.w.worm_steps_total
    assert np.array_equal(ops, w.ops)
    with pytest.raises(SSEError):
        eng.set_worm_cap(ids, 0)
    eng.close()
