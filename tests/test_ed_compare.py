"""Statistical check of the oracle against exact diagonalisation
(test/test_ed_compare.jl with the jobs of test/test_jobs.jl:4-67).

The reference runs 40000 sweeps after 5000 thermalisation sweeps and
requires |z| <= 4 for every observable.  The CPU suite runs shorter chains
(several independent walkers, binned) with the same |z| <= 4 criterion.
"""

import numpy as np
import pytest

from ed import ed_observables, evaluables, jackknife

OBS_BASE = ["Sign", "OperatorCount", "SignOperatorCount", "SignOperatorCount2", "SignEnergy", "WormLengthFraction"]
OBS_EST = ["SignMag", "SignAbsMag", "SignMag2", "SignMag4", "SignMagChi"]


def obs_names(prefixes):
    names = list(OBS_BASE)
    for p in prefixes:
        names += [n.replace("Sign", "Sign" + p, 1) for n in OBS_EST]
    return names


def run_binned(O, flat, T, seed, nbins, binsize, therm, nwalkers=4):
    om = O.OracleModel(flat)
    names = obs_names(flat.est_prefixes)
    bins = {n: [] for n in names}
    walkers = [O.OracleWalker(om, T=T, seed=seed, stream=k, thermalization=therm) for k in range(nwalkers)]
    for w in walkers:
        w.init()
        w.run(therm, measure=True)
    prev = [w.obs()[0].copy() for w in walkers]
    prevc = [w.obs()[1].copy() for w in walkers]
    for _ in range(nbins):
        for k, w in enumerate(walkers):
            w.run(binsize, measure=True)
            s, c, _ = w.obs()
            ds, dc = s - prev[k], c - prevc[k]
            prev[k], prevc[k] = s.copy(), c.copy()
            for i, n in enumerate(names):
                bins[n].append(ds[i] / max(dc[i], 1))
    return {n: np.array(v) for n, v in bins.items()}


JOBS = {
    "magnet_square": dict(
        lattice=("square", (2, 4)), J=1.23, hz=-0.2,
    ),
    "honeycomb": dict(
        lattice=("honeycomb", (2, 2)), parameter_map={"S": ["Sa", "Sb"], "J": ["J1", "J2", "J3"]},
        J1=1.0, J2=0.5, J3=1.0, d=0.2, Dz=0.2, Dx=0.5, Sa=0.5, Sb=1.0,
    ),
}


_ED_CACHE = {}


def make_model(S, job):
    p = dict(job)
    uc, size = p.pop("lattice")
    p["lattice"] = {"unitcell": getattr(S.UnitCells, uc), "size": size}
    p["measure"] = S.all_magnetization_estimators(2)
    return S.MagnetModel(p)


@pytest.mark.parametrize("job", list(JOBS))
@pytest.mark.parametrize("T", [0.04, 0.70, 2.02, 4.0])
def test_oracle_vs_ed(S, O, job, T):
    model = make_model(S, JOBS[job])
    flat = S.flatten_model(model)
    key = (job, T)
    if key not in _ED_CACHE:
        _ED_CACHE[key] = ed_observables(S, model, [T])
    ed = _ED_CACHE[key]
    bins = run_binned(O, flat, T, seed=124535, nbins=16, binsize=400, therm=1000)
    funcs = evaluables(flat.est_prefixes, flat.norm_site_count)
    bad = []
    for name, f in funcs.items():
        mc, err = jackknife(bins, f)
        ref = float(ed[name][0])
        z = abs(mc - ref) / (err if err != 0 else 1e-8)
        if z > 4:
            bad.append((name, mc, err, ref, z))
    assert not bad, bad


@pytest.mark.parametrize("spin,size,T", [(1.5, (2, 3), 0.5), (2.0, (2, 2), 2.0)])
def test_oracle_vs_ed_higher_spin(S, O, spin, size, T):
    """Spins above 1 (site dimensions 4 and 5, with a field): the oracle's chains against exact
    diagonalisation, |z| <= 4 on every observable."""
    model = S.MagnetModel({"lattice": {"unitcell": S.UnitCells.square, "size": size}, "S": spin, "J": 1.0,
                           "hz": 0.1, "measure": S.all_magnetization_estimators(2)})
    flat = S.flatten_model(model)
    assert flat.maxdim == int(2 * spin + 1)
    ed = ed_observables(S, model, [T])
    bins = run_binned(O, flat, T, seed=11, nbins=16, binsize=400, therm=1000)
    bad = []
    for name, f in evaluables(flat.est_prefixes, flat.norm_site_count).items():
        mc, err = jackknife(bins, f)
        ref = float(ed[name][0])
        z = abs(mc - ref) / (err if err != 0 else 1e-8)
        if z > 4:
            bad.append((name, mc, err, ref, z))
    assert not bad, bad


def test_oracle_vs_ed_frustrated_triangle(S, O):
    """The antiferromagnetic XXZ magnet on the triangular lattice (3x3, Jz = 1.4 J): negative vertex
    weights (average sign about 0.22 at T = 1), so every observable is a ratio of signed means; the
    oracle against exact diagonalisation, |z| <= 4."""
    model = S.MagnetModel({"lattice": {"unitcell": S.UnitCells.triangle, "size": (3, 3)}, "J": 1.0, "d": 0.4,
                           "measure": S.all_magnetization_estimators(2)})
    flat = S.flatten_model(model)
    assert (flat.arrays["sign"] < 0).any()
    T = 1.0
    ed = ed_observables(S, model, [T])
    bins = run_binned(O, flat, T, seed=11, nbins=16, binsize=400, therm=1000)
    bad = []
    for name, f in evaluables(flat.est_prefixes, flat.norm_site_count).items():
        mc, err = jackknife(bins, f)
        ref = float(ed[name][0])
        z = abs(mc - ref) / (err if err != 0 else 1e-8)
        if z > 4:
            bad.append((name, mc, err, ref, z))
    assert not bad, bad
