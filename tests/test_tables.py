"""The flattened model tables of every model family satisfy what sse_model_register checks (and
what the sweep kernel relies on when it indexes them), plus the structure of the scatter rows: the
host builder's output is caught here, on the CPU, before a GPU ever sees it."""

import numpy as np
import pytest

from golden_cases import CASES


def families(S):
    out = {name: c["model"] for name, c in CASES.items()}
    out["square_s1_field"] = lambda S: S.MagnetModel({
        "lattice": {"unitcell": S.UnitCells.square, "size": (3, 3)}, "S": 1.0, "J": 1.0, "hz": 0.3, "Dz": -0.2,
        "measure": ["magnetization"]})
    out["triangle_xxz"] = lambda S: S.MagnetModel({
        "lattice": {"unitcell": S.UnitCells.triangle, "size": (3, 3)}, "J": 1.0, "d": 0.4,
        "measure": ["magnetization"]})
    return out


@pytest.fixture(scope="module", params=["square8_beta2", "honeycomb_mixed_T0.1", "bilayer_s1_T0.25",
                                        "cluster_dimer_T0.3", "square_s1_field", "triangle_xxz"])
def flat(S, request):
    return S.flatten_model(families(S)[request.param](S))


def test_bonds_and_sites(flat):
    a = flat.arrays
    bs = a["bond_sites"].reshape(-1, 2)
    assert ((bs >= 0) & (bs < flat.nsites)).all() and (bs[:, 0] != bs[:, 1]).all()
    bt = a["bond_type"]
    assert ((bt >= 0) & (bt < flat.ntypes)).all()
    td = a["type_dims"].reshape(-1, 2)
    assert np.array_equal(a["site_dims"][bs[:, 0]], td[bt, 0]) and np.array_equal(a["site_dims"][bs[:, 1]], td[bt, 1])
    assert flat.maxdim == a["site_dims"].max() and 2 <= flat.maxdim <= 255


def test_vertices_and_diagonal_table(flat):
    a = flat.arrays
    td = a["type_dims"].reshape(-1, 2)
    for t in range(flat.ntypes):
        nv, vo = int(a["type_nverts"][t]), int(a["type_vert_off"][t])
        assert 1 <= nv <= 512
        ls = a["leg_state"][4 * vo: 4 * (vo + nv)].reshape(nv, 4)
        assert (ls[:, [0, 2]] < td[t, 0]).all() and (ls[:, [1, 3]] < td[t, 1]).all()
        assert (a["weight"][vo: vo + nv] > 0).all()
        assert set(np.unique(a["sign"][vo: vo + nv])) <= {-1, 1}
        do = int(a["type_diag_off"][t])
        for st in range(td[t, 0] * td[t, 1]):
            vc = int(a["diag_vertex"][do + st])
            if vc < 0:
                continue
            v = vc >> 1
            assert vc & 1 and v < nv
            # the diagonal vertex of compound state s0 + d0*s1 has those states on its legs, unchanged
            s0, s1 = st % td[t, 0], st // td[t, 0]
            assert list(ls[v]) == [s0, s1, s0, s1]


def test_scatter_rows(flat):
    a = flat.arrays
    nout = len(a["out_cum"])
    for t in range(flat.ntypes):
        nv, mw, to = int(a["type_nverts"][t]), int(a["type_maxworm"][t]), int(a["type_trans_off"][t])
        for r in range(to, to + nv * 4 * mw):
            st, cnt = int(a["trans_start"][r]), int(a["trans_count"][r])
            if st < 0:
                assert cnt == 0
                continue
            assert 1 <= cnt <= 256 and st + cnt <= nout
            cum = a["out_cum"][st: st + cnt]
            assert (np.diff(cum) >= 0).all() and cum[0] > 0
            assert cum[-1] == pytest.approx(1.0, abs=1e-9)
            assert ((a["out_leg"][st: st + cnt] >= 0) & (a["out_leg"][st: st + cnt] <= 3)).all()
            assert ((a["out_worm"][st: st + cnt] >= 1) & (a["out_worm"][st: st + cnt] <= mw)).all()
            tgt = a["out_target"][st: st + cnt]
            assert ((tgt >= 0) & ((tgt >> 1) < nv)).all()


def test_estimator_coefficients(flat):
    a = flat.arrays
    coef = a["est_coef"].reshape(flat.nest, flat.nsites, flat.maxdim) if flat.nest else np.zeros((0,))
    if flat.nest:
        assert np.isfinite(coef).all()
        # entries beyond a site's dimension are never read and stay zero
        for site in range(flat.nsites):
            assert not coef[:, site, a["site_dims"][site]:].any()
        # every coefficient is a multiple of 1/2, so the engine can measure in exact integers
        assert np.array_equal(2 * coef, np.rint(2 * coef))
