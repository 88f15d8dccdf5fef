"""Parallel tempering in T (src/sse.jl:390-405) on the CPU oracle.

The reference provides the two hooks Carlo.jl's parallel tempering calls:
parallel_tempering_log_weight_ratio(mc, :T, T') = -n log(T'/T) and
parallel_tempering_change_parameter!(mc, :T, T').  Carlo's exchange schedule
and random stream are its own (Carlo.jl is not vendored), so the engine defines
them: neighbouring rungs in T order, alternating parity, one counter-based draw
per proposed pair.  These tests pin that rule on the oracle: the swap weight,
the schedule, the bookkeeping, the stationary distribution of the temperature
permutation, and energies at every temperature of a ladder against exact
diagonalisation.
"""

import itertools
import math

import numpy as np
import pytest

from ed import ed_observables, evaluables, jackknife


def square_2x4(S):
    return S.MagnetModel({"lattice": {"unitcell": S.UnitCells.square, "size": (2, 4)}, "J": 1.23, "hz": -0.2,
                          "measure": S.all_magnetization_estimators(2)})


def test_swap_weight_is_exp_of_log_weight_ratios(O):
    cases = [(0.5, 0.7, 120, 100), (0.5, 0.7, 100, 120), (0.3, 0.31, 4000, 3990), (1.0, 2.0, 7, 7),
             (0.1, 0.4, 0, 3), (0.25, 0.5, 1000, 0)]
    for Ta, Tb, na, nb in cases:
        # Carlo: lwr(a, T_b) + lwr(b, T_a), lwr(mc, T') = -n log(T'/T)  (src/sse.jl:390-396)
        lw = -na * math.log(Tb / Ta) - nb * math.log(Ta / Tb)
        q = O.tempering_weight(Ta, Tb, na, nb)
        if lw < -700:
            assert q < 1e-300
        else:
            assert q == pytest.approx(math.exp(lw), rel=1e-12)


def _ladder(O, S, temps, nl=1, seed=3):
    om = O.OracleModel(S.flatten_model(square_2x4(S)))
    ws = []
    for l in range(nl):
        for k, T in enumerate(temps):
            w = O.OracleWalker(om, T=T, seed=seed, stream=l * len(temps) + k)
            w.init()
            ws.append(w)
    return om, ws


def test_schedule_alternates_parity(S, O):
    temps = [0.3, 0.4, 0.55, 0.8, 1.2]
    _, ws = _ladder(O, S, temps, nl=2)
    for step in range(6):
        acc, rc = O.tempering_exchange(ws, 2, 5, seed=11, step=step)
        assert rc == 0
        for k in range(4):
            proposed = acc[:, k] >= 0
            assert proposed.all() == (k % 2 == step % 2)
            assert (~proposed).all() == (k % 2 != step % 2)


def test_swap_exchanges_temperature_and_accumulators(S, O):
    temps = [0.5, 0.6]
    _, ws = _ladder(O, S, temps)
    for w in ws:
        w.run(30, measure=True)
    # equal operator counts: q = 1, the swap is always accepted
    ws[1].w.num_operators = ws[0].w.num_operators
    before = [w.obs() for w in ws]
    acc, rc = O.tempering_exchange(ws, 1, 2, seed=5, step=0)
    assert rc == 0 and acc[0, 0] == 1
    assert ws[0].w.T == 0.6 and ws[1].w.T == 0.5
    for i in range(3):
        assert np.array_equal(ws[0].obs()[i], before[1][i])
        assert np.array_equal(ws[1].obs()[i], before[0][i])


def test_order_within_a_ladder_does_not_matter(S, O):
    """Walkers are ranked by T, so the order they are listed in changes nothing."""
    temps = [0.35, 0.5, 0.7, 1.0]
    results = []
    for perm in ([0, 1, 2, 3], [2, 0, 3, 1]):
        _, ws = _ladder(O, S, temps)
        for w in ws:
            w.run(20, measure=False)
        for step in range(5):
            acc, rc = O.tempering_exchange([ws[i] for i in perm], 1, 4, seed=9, step=step)
            assert rc == 0
        results.append([w.w.T for w in ws])
    assert results[0] == results[1]


def test_duplicate_temperatures_rejected(S, O):
    _, ws = _ladder(O, S, [0.5, 0.5, 0.7])
    acc, rc = O.tempering_exchange(ws, 1, 3, seed=1, step=0)
    assert rc == 1 and (acc == -1).all()


def test_stopped_walker_pairs_not_proposed(S, O):
    _, ws = _ladder(O, S, [0.4, 0.5, 0.6, 0.7])
    ws[1].w.status = 8  # as if a worm had hit the step cap
    acc, rc = O.tempering_exchange(ws, 1, 4, seed=1, step=0)
    assert rc == 0 and acc[0, 0] == -1 and acc[0, 2] >= 0
    acc, rc = O.tempering_exchange(ws, 1, 4, seed=1, step=1)
    assert acc[0, 1] == -1


def test_permutation_distribution_is_the_product_weight(S, O):
    """With the operator counts held fixed the exchange steps form a Markov chain on the assignment
    sigma of temperatures to configurations, stationary at prod_i T_sigma(i)^(-n_i)."""
    temps = [0.5, 0.65, 0.9]
    _, ws = _ladder(O, S, temps)
    ns = [30, 24, 17]
    for w, n in zip(ws, ns):
        w.w.num_operators = n
    counts = {}
    nsteps = 30000
    for step in range(nsteps):
        O.tempering_exchange(ws, 1, 3, seed=2024, step=step)
        key = tuple(w.w.T for w in ws)
        counts[key] = counts.get(key, 0) + 1
    perms = list(itertools.permutations(temps))
    wts = np.array([math.prod(t ** (-n) for t, n in zip(p, ns)) for p in perms])
    wts /= wts.sum()
    for p, wgt in zip(perms, wts):
        f = counts.get(p, 0) / nsteps
        # autocorrelated samples: allow 5 sigma of an effective sample 1/5 the size
        sig = math.sqrt(wgt * (1 - wgt) / (nsteps / 5))
        assert abs(f - wgt) < 5 * sig + 1e-3, (p, f, wgt)


def test_tempering_ladder_energies_match_ed(S, O):
    """Every temperature of a ladder, sampled with exchanges, against exact diagonalisation (|z| <= 4)."""
    model = square_2x4(S)
    flat = S.flatten_model(model)
    temps = [0.4, 0.6, 0.9, 1.35]
    ed = ed_observables(S, model, temps)
    om = O.OracleModel(flat)
    nl, nr, interval, therm, nbins, bin_blocks = 3, len(temps), 5, 500, 16, 60
    ws = []
    for l in range(nl):
        for k, T in enumerate(temps):
            w = O.OracleWalker(om, T=T, seed=77, stream=l * nr + k, thermalization=therm)
            w.init()
            ws.append(w)
    names = list(O.OBS_BASE_NAMES)
    for p in flat.est_prefixes:
        names += [n.replace("Sign", "Sign" + p, 1) for n in O.OBS_EST_NAMES]
    step = 0

    def block():
        nonlocal step
        for w in ws:
            w.run(interval, measure=True)
        acc, rc = O.tempering_exchange(ws, nl, nr, seed=31, step=step)
        assert rc == 0
        step += 1

    for _ in range(therm // interval):
        block()

    def by_temperature():
        """cumulative (sums, counts) per (ladder, temperature index): the accumulators follow T"""
        out = {}
        for l in range(nl):
            for w in ws[l * nr:(l + 1) * nr]:
                s, c, _ = w.obs()
                out[(l, temps.index(w.w.T))] = (s.copy(), c.copy())
        return out

    prev = by_temperature()
    bins = [{n: [] for n in names} for _ in temps]
    for _ in range(nbins):
        for _ in range(bin_blocks):
            block()
        cur = by_temperature()
        for (l, t), (s, c) in cur.items():
            ds, dc = s - prev[(l, t)][0], c - prev[(l, t)][1]
            for i, n in enumerate(names):
                bins[t][n].append(ds[i] / max(dc[i], 1))
        prev = cur
    funcs = evaluables(flat.est_prefixes, flat.norm_site_count)
    bad = []
    for t, T in enumerate(temps):
        b = {n: np.array(v) for n, v in bins[t].items()}
        for name in ("Energy", "SpecificHeat", "Mag2", "MagChi"):
            mc, err = jackknife(b, funcs[name])
            ref = float(ed[name][t])
            z = abs(mc - ref) / (err if err else 1e-8)
            if z > 4:
                bad.append((T, name, mc, err, ref, z))
    assert not bad, bad


def test_mc_tempering_hooks_follow_reference(S):
    """MC.parallel_tempering_* mirror src/sse.jl:390-405 (host logic; the engine is a stand-in)."""
    from sse_gb300.mc import MC

    class Recorder:
        T = None

        def register_model(self, flat):
            return 0

        def create_walkers(self, model_id, params):
            self.params = params
            return np.array([0], dtype=np.int32)

        def info(self, wid):
            return {"num_operators": 40}

        def set_T(self, wid, T):
            self.T = T

    rec = Recorder()
    params = {"model": S.MagnetModel, "lattice": {"unitcell": S.UnitCells.square, "size": (2, 2)}, "J": 1.0, "T": 0.5}
    mc = MC(params, engine=rec)
    assert mc.parallel_tempering_log_weight_ratio("T", 0.7) == -40 * math.log(0.7 / 0.5)
    with pytest.raises(ValueError, match="unsupported parallel tempering parameter J"):
        mc.parallel_tempering_log_weight_ratio("J", 0.7)
    with pytest.raises(ValueError, match="unsupported parallel tempering parameter J"):
        mc.parallel_tempering_change_parameter("J", 0.7)
    mc.parallel_tempering_change_parameter("T", 0.7)
    assert mc.T == 0.7 and rec.T == 0.7
