"""Seeded trajectory cases pinned by tests/golden/trajectories.json (made by tests/golden/make_golden.py)."""


def _square8(S):
    return S.MagnetModel({"lattice": {"unitcell": S.UnitCells.square, "size": (8, 8)}, "J": 1.0,
                          "measure": ["magnetization", "staggered_magnetization"]})


def _honeycomb_mixed(S):
    return S.MagnetModel({"lattice": {"unitcell": S.UnitCells.honeycomb, "size": (4, 4)}, "J": 1.4,
                          "parameter_map": {"S": ("S1", "S2")}, "S1": 0.5, "S2": 1.0,
                          "measure": S.all_magnetization_estimators(2)})


def _bilayer_s1(S):
    return S.MagnetModel({"lattice": {"unitcell": S.UnitCells.square_bilayer, "size": (4, 4)}, "S": 1.0, "J": 1.0,
                          "Jp": 0.5, "parameter_map": {"J": ["Jp", "J", "J", "J", "J"]}, "Dz": 0.3, "hz": 0.2,
                          "measure": ["magnetization"]})


def _cluster(S):
    return S.ClusterModel({
        "inner_model": S.MagnetModel,
        "lattice": {"unitcell": S.UnitCells.fully_frust_square_bilayer, "size": (3, 2)},
        "parameter_map": {"S": ["Sa", "Sb"], "J": ["JD", "JxP", "JxP", "JyP", "JyP", "JxX", "JxX", "JyX", "JyX"]},
        "cluster_bases": (S.ClusterBases.dimer,), "measure_quantum_numbers": [{"name": "", "quantum_number": 2}],
        "JD": 1, "JxP": 0.55, "JyP": 0.6, "JxX": 0.7, "JyX": 0.3, "d": -0.2, "Dz": 0.2, "Dx": 0.5,
        "Sa": 0.5, "Sb": 0.5})


def _square32(S):
    return S.MagnetModel({"lattice": {"unitcell": S.UnitCells.square, "size": (32, 32)}, "J": 1.0,
                          "measure": ["magnetization", "staggered_magnetization"]})


CASES = {
    "square8_beta2": dict(model=_square8, T=0.5, seed=101, therm=10, sweeps=40, streams=[0, 7]),
    "honeycomb_mixed_T0.1": dict(model=_honeycomb_mixed, T=0.1, seed=202, therm=10, sweeps=30, streams=[1, 2]),
    "bilayer_s1_T0.25": dict(model=_bilayer_s1, T=0.25, seed=303, therm=10, sweeps=25, streams=[0, 3]),
    "cluster_dimer_T0.3": dict(model=_cluster, T=0.3, seed=404, therm=10, sweeps=25, streams=[0, 5]),
    "square32_beta16": dict(model=_square32, T=1 / 16, seed=505, therm=4, sweeps=8, streams=[11]),
}


def save_flat(flat, path):
    """A FlatModel as an .npz: its arrays plus the scalar fields."""
    import numpy as np

    np.savez_compressed(path, **{f"a_{k}": v for k, v in flat.arrays.items()},
                        scalars=np.array([flat.nsites, flat.nbonds, flat.ntypes, flat.maxdim, flat.nest]),
                        floats=np.array([flat.energy_offset, flat.norm_site_count]),
                        prefixes=np.array(flat.est_prefixes, dtype=str))


def load_flat(S, path):
    import numpy as np

    z = np.load(path)
    nsites, nbonds, ntypes, maxdim, nest = (int(x) for x in z["scalars"])
    arrays = {k[2:]: np.ascontiguousarray(z[k]) for k in z.files if k.startswith("a_")}
    return S.FlatModel(nsites=nsites, nbonds=nbonds, ntypes=ntypes, maxdim=maxdim, nest=nest,
                       energy_offset=float(z["floats"][0]), norm_site_count=float(z["floats"][1]),
                       arrays=arrays, est_prefixes=[str(p) for p in z["prefixes"]])
