"""Ports of test/test_lattice.jl, test/models/test_magnet.jl, test/test_sse_data.jl
and test/test_common_operators.jl."""

from math import comb

import numpy as np
import pytest


def test_unitcell_signs_coordinations(S):
    uc = S.UnitCells.square
    assert uc.sites[0].sublattice_sign == 1 and uc.sites[0].coordination == 4
    uc = S.UnitCells.columnar_dimer
    assert [s.sublattice_sign for s in uc.sites] == [1, -1]
    assert [s.coordination for s in uc.sites] == [4, 4]
    uc = S.UnitCells.honeycomb
    assert [s.sublattice_sign for s in uc.sites] == [1, -1]
    assert [s.coordination for s in uc.sites] == [3, 3]


def _adj(lat):
    n = lat.site_count()
    A = np.zeros((n, n), dtype=np.int64)
    for b in lat.bonds:
        A[b.i - 1, b.j - 1] = 1
        A[b.j - 1, b.i - 1] = 1
    return A


def _sq(n):
    return comb(n, n // 2) ** 2 if n % 2 == 0 else 0


def _hc(n):
    return sum(comb(n // 2, k) ** 2 * comb(2 * k, k) for k in range(n // 2 + 1)) if n % 2 == 0 else 0


def _tri(n):
    return sum((-2) ** (n - k) * comb(n, k) * sum(comb(k, j) ** 3 for j in range(k + 1)) for k in range(n + 1))


@pytest.mark.parametrize("Ls", [(3, 4), (8, 4), (5, 5), (8, 8)])
def test_lattice_walks(S, Ls):
    # test/test_lattice.jl:41-77
    ucs = [S.UnitCells.square, S.UnitCells.columnar_dimer, S.UnitCells.honeycomb, S.UnitCells.triangle]
    walks = [_sq, _sq, _hc, _tri]
    for uc, nw in zip(ucs, walks):
        lat = S.Lattice.make(uc, Ls)
        A = _adj(lat)
        assert np.trace(A @ A) // 2 == len(lat.bonds)
        for n in range(2, 7):
            if any(L <= n for L in Ls):
                continue
            assert np.trace(np.linalg.matrix_power(A, n)) // lat.site_count() == nw(n)


def test_neel_vector(S):
    # test/test_lattice.jl:79-84
    assert S.neel_vector(S.UnitCells.square) == ((True, True), False)
    assert S.neel_vector(S.UnitCells.columnar_dimer) == ((True, False), True)
    assert S.neel_vector(S.UnitCells.honeycomb) == ((False, False), True)
    assert S.neel_vector(S.UnitCells.triangle) is None


def test_magnet_params(S):
    # test/models/test_magnet.jl
    L, hz = 5, 0.3
    m = S.MagnetModel({"lattice": {"unitcell": S.UnitCells.square, "size": (L, L)}, "J": 1.2, "hz": hz, "Dz": 0.32, "Dx": 0.06})
    assert len(m.site_spin_states) == L * L
    assert len(m.bond_params) == 2 * L * L
    assert m.bond_params[0].hz == pytest.approx((hz / 4, hz / 4))
    m = S.MagnetModel({"lattice": {"unitcell": S.UnitCells.square, "size": (L, 2 * L)}, "J": 1.0, "hz": hz})
    assert len(m.site_spin_states) == 2 * L * L and len(m.bond_params) == 4 * L * L
    m = S.MagnetModel({"lattice": {"unitcell": S.UnitCells.square, "size": (L, 2 * L)}, "parameter_map": {"J": ("Jx", "Jy")},
                       "hz": hz, "Jx": 1.0, "Jy": 2.0})
    assert m.bond_params[0].J == pytest.approx(1.0) and m.bond_params[1].J == pytest.approx(2.0)
    with pytest.raises(KeyError):
        S.MagnetModel({"lattice": {"unitcell": S.UnitCells.square, "size": (L, 2 * L)},
                       "parameter_map": {"J": ("Jx", "nonexistent")}, "hz": hz, "Jx": 1.0, "Jy": 2.0})


def test_sse_data_inconsistent_dims(S):
    # test/test_sse_data.jl
    vd32 = S.make_vertex_data((3, 2), np.eye(6))
    vd23 = S.make_vertex_data((2, 3), np.eye(6))
    vds = [vd32, vd23]
    ok = [S.SSEBond(1, (1, 2)), S.SSEBond(2, (2, 3))]
    sites = S.generate_sites_from_bonds(vds, ok)
    assert [s.dim for s in sites] == [3, 2, 3]
    with pytest.raises(ValueError):
        S.generate_sites_from_bonds(vds, [S.SSEBond(1, (1, 2)), S.SSEBond(1, (2, 3))])
    with pytest.raises(ValueError):
        S.generate_sites_from_bonds(vds, [S.SSEBond(1, (1, 2)), S.SSEBond(2, (3, 2))])


def test_common_operators(S):
    sp, sz = S.spin_operators(2)
    assert np.allclose(sp, [[0, 1], [0, 0]]) and np.allclose(sz, [[0.5, 0], [0, -0.5]])
    for d in np.random.default_rng(5).integers(2, 100, 10):
        sp, sz = S.spin_operators(int(d))
        s = (d - 1) / 2
        assert np.allclose(sz @ sz + 0.5 * (sp.T @ sp + sp @ sp.T), np.eye(d) * s * (s + 1))
        a = S.bosonic_a_operator(int(d))
        assert np.allclose(a.T @ a, np.diag(np.arange(d)))
