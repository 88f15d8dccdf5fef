"""Host logic of the Carlo-style drivers in mc.py (MC, BatchMC, TemperingMC) and of the jackknife
evaluables, against a stand-in engine: no GPU needed."""

import math

import numpy as np
import pytest


class StubEngine:
    """Walkers whose observables are deterministic functions of (walker, sweep): observable i of
    walker w in sweep s is w + s + i / 10.  Temperatures can be swapped like the device exchange."""

    def __init__(self, nobs):
        self.nobs_ = nobs
        self.w = {}
        self.next = 0

    def register_model(self, flat):
        return 0

    def nobs(self, mid):
        return self.nobs_

    def create_walkers(self, mid, params):
        ids = np.arange(self.next, self.next + len(params), dtype=np.int32)
        self.next += len(params)
        for i, p in zip(ids.tolist(), params):
            self.w[i] = dict(p=p, T=p["T"], sweeps=0, sums=np.zeros(self.nobs_), counts=np.zeros(self.nobs_, np.int64))
        return ids

    def init(self, ids):
        pass

    def sweep(self, ids, n, measure=True, plain=False, graph=False):
        for i in np.asarray(ids).tolist():
            w = self.w[i]
            for _ in range(n):
                w["sweeps"] += 1
                if measure and w["sweeps"] > w["p"]["thermalization"]:
                    w["sums"] += i + w["sweeps"] + np.arange(self.nobs_) / 10
                    w["counts"] += 1

    def observables(self, ids, reset=False):
        out = []
        for i in np.asarray(ids).tolist():
            w = self.w[i]
            out.append((w["sums"].copy(), w["counts"].copy(), np.zeros(self.nobs_)))
            if reset:
                w["sums"][:] = 0
                w["counts"][:] = 0
        return out

    def info(self, i):
        return {"T": self.w[int(i)]["T"], "num_operators": 10 * int(i) + 3}

    def set_T(self, i, T):
        self.w[int(i)]["T"] = T

    def sweep_tempering(self, ladders, nblocks, interval, seed, first_step=0, measure=True, graph=False):
        """interval sweeps, then swap the two lowest temperatures of every ladder (with their
        accumulators, as the device exchange does) when the step is even."""
        nl, nr = ladders.shape
        acc = np.zeros((nl, nr - 1), np.int64)
        prop = np.zeros((nl, nr - 1), np.int64)
        for b in range(nblocks):
            self.sweep(ladders.ravel(), interval, measure=measure)
            if (first_step + b) % 2 == 0:
                for l in range(nl):
                    row = sorted(ladders[l].tolist(), key=lambda i: self.w[i]["T"])
                    a, c = self.w[row[0]], self.w[row[1]]
                    a["T"], c["T"] = c["T"], a["T"]
                    for key in ("sums", "counts"):
                        a[key], c[key] = c[key].copy(), a[key].copy()
                    acc[l, 0] += 1
                    prop[l, 0] += 1
        return acc, prop


def params(S, **kw):
    p = {"model": S.MagnetModel, "lattice": {"unitcell": S.UnitCells.square, "size": (2, 2)}, "J": 1.0, "T": 0.5,
         "measure": ["magnetization"], "thermalization": 3, "seed": 9}
    p.update(kw)
    return p


def test_mc_forwards_one_value_per_step(S):
    from sse_gb300.mc import MC, MCContext

    p = params(S)
    eng = StubEngine(nobs=11)
    mc = MC(p, engine=eng)
    ctx = MCContext(p)
    mc.init(ctx)
    for _ in range(6):
        mc.sweep(ctx)
        if ctx.is_thermalized():
            mc.measure(ctx)
    # Carlo's rule: is_thermalized = sweeps > thermalization, so sweeps 4..6 measured
    assert ctx.sweeps == 6
    assert ctx.observables["Sign"] == [0 + 4 + 0.0, 0 + 5 + 0.0, 0 + 6 + 0.0]
    assert ctx.observables["OperatorCount"] == pytest.approx([4.1, 5.1, 6.1])


def test_batchmc_bins_and_jackknife(S):
    from sse_gb300.mc import BatchMC

    p = params(S, thermalization=4)
    eng = StubEngine(nobs=11)
    mc = BatchMC(p, nwalkers=3, engine=eng)
    mc.run(sweeps=20, binsize=5)
    # 4 bins per walker, each the mean of 5 measured sweeps
    assert len(mc.bins) == 3 * 4
    assert mc.bins[0]["Sign"] == pytest.approx(np.mean([0 + s for s in range(5, 10)]))
    res = mc.results()
    assert set(res) >= {"Energy", "SpecificHeat", "Mag", "Mag2", "BinderRatio", "Sign"}
    # jackknife of a ratio against a direct leave-one-out computation
    sign = np.array([b["Sign"] for b in mc.bins])
    se = np.array([b["SignEnergy"] for b in mc.bins])
    full = se.mean() / sign.mean()
    loo = np.array([(se.sum() - se[i]) / (sign.sum() - sign[i]) for i in range(len(sign))])
    err = math.sqrt((len(sign) - 1) / len(sign) * ((loo - loo.mean()) ** 2).sum())
    assert res["Energy"][0] == pytest.approx(full, rel=1e-12)
    assert res["Energy"][1] == pytest.approx(err, rel=1e-9)


def test_tempering_mc_bins_follow_the_temperature(S):
    """The accumulators move with the temperature, so every bin lands at the temperature its
    measurements were taken at, whichever walker holds it at the end."""
    from sse_gb300.mc import TemperingMC

    p = params(S, thermalization=0)
    eng = StubEngine(nobs=11)
    temps = [0.3, 0.5, 0.8]
    pt = TemperingMC(p, temps, nladders=2, interval=2, engine=eng)
    assert pt.ladders.shape == (2, 3)
    assert [eng.w[int(i)]["T"] for i in pt.ladders[0]] == temps
    pt.init()
    pt.sweep(1)  # step 0: even, the two lowest temperatures swap
    assert [eng.w[int(i)]["T"] for i in pt.ladders[0]] == [0.5, 0.3, 0.8]
    assert (pt.temperature_of()[0] == [1, 0, 2]).all()
    pt.collect_bin()
    # the bin at T=0.3 holds walker 0's two sweeps (its accumulators moved to walker 1)
    w0 = int(pt.ladders[0][0])
    assert pt.bins[0][0]["Sign"] == pytest.approx(np.mean([w0 + 1, w0 + 2]))
    assert pt.acceptance()[0] == 1.0 and np.isnan(pt.acceptance()[1])
    with pytest.raises(ValueError):
        TemperingMC(p, [0.5, 0.5], engine=eng)


def test_jackknife_skips_empty_bins_and_single_bin(S):
    """A bin in which a walker measured nothing (NaN means) is left out instead of counting as zero;
    one bin gives means with NaN errors instead of a division by zero."""
    from sse_gb300.mc import jackknife_results, observable_names

    flat = S.flatten_model(S.MagnetModel({"lattice": {"unitcell": S.UnitCells.square, "size": (2, 2)}, "J": 1.0,
                                          "measure": ["magnetization"]}))
    names = observable_names(flat.est_prefixes)
    rng = np.random.default_rng(4)
    full = [{n: float(v) for n, v in zip(names, rng.uniform(0.5, 1.5, len(names)))} for _ in range(6)]
    empty = {n: float("nan") for n in names}
    with_empty = jackknife_results(full[:3] + [empty] + full[3:], names, flat)
    without = jackknife_results(full, names, flat)
    for k, (m, e) in without.items():
        assert with_empty[k][0] == pytest.approx(m, rel=1e-12) and with_empty[k][1] == pytest.approx(e, rel=1e-12)
    one = jackknife_results(full[:1], names, flat)
    assert one["Energy"][0] == pytest.approx(full[0]["SignEnergy"] / full[0]["Sign"]) and math.isnan(one["Energy"][1])
    assert jackknife_results([empty], names, flat) == {}
