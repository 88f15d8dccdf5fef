"""ClusterModel (src/models/cluster/cluster.jl): ports of test/models/test_cluster.jl, and the
oracle against exact diagonalisation on the reference's cluster ED job (test/test_jobs.jl:69-110)."""

import numpy as np
import pytest

from ed import ed_observables, evaluables, jackknife
from test_ed_compare import run_binned


def dimer_magnet_params(S):
    """test/models/test_cluster.jl:17-37."""
    return {
        "inner_model": S.MagnetModel,
        "lattice": {"unitcell": S.UnitCells.fully_frust_square_bilayer, "size": (2, 2)},
        "parameter_map": {"J": ["J1", "J2", "J3", "J4", "J5", "J6", "J7", "J8", "J9"], "Dz": ["Dz1", "Dz2"]},
        "cluster_bases": (S.ClusterBases.dimer,),
        "measure_quantum_numbers": [],
        "J1": 1, "J2": 1.1, "J3": 1.2, "J4": 1.3, "J5": 1.4, "J6": 1.5, "J7": 1.6, "J8": 1.7, "J9": 1.8,
    }


def cluster_job_params(S):
    """The cluster ED job, test/test_jobs.jl:69-110."""
    return {
        "inner_model": S.MagnetModel,
        "lattice": {"unitcell": S.UnitCells.fully_frust_square_bilayer, "size": (2, 2)},
        "parameter_map": {"S": ["Sa", "Sb"], "J": ["JD", "JxP", "JxP", "JyP", "JyP", "JxX", "JxX", "JyX", "JyX"]},
        "cluster_bases": (S.ClusterBases.dimer,),
        "measure_quantum_numbers": [{"name": "", "quantum_number": 2}],
        "JD": 1, "JxP": 0.55, "JyP": 0.6, "JxX": 0.7, "JyX": 0.3, "d": -0.2, "Dz": 0.2, "Dx": 0.5,
        "Sa": 0.5, "Sb": 0.5,
    }


def test_lift_twobody_operator(S):
    """test/models/test_cluster.jl:3-15 (matrices filled column-major, as reshape(1:n, k, k))."""
    A = np.arange(1, 17, dtype=float).reshape(4, 4).T
    B = np.arange(1, 10, dtype=float).reshape(3, 3).T
    C = np.arange(1, 5, dtype=float).reshape(2, 2).T
    kron = np.kron
    assert np.array_equal(S.lift_twobody_operator(kron(A, B), (4, 3, 2), (1, 2)), kron(kron(A, B), np.eye(2)))
    L = S.lift_twobody_operator(kron(A, B), (3, 2, 4), (3, 1))
    assert np.array_equal(L @ kron(kron(np.eye(3), C), np.eye(4)), kron(kron(B, C), A))
    assert np.array_equal(L @ kron(kron(B, C), np.eye(4)), kron(kron(B @ B, C), A))


def test_dimer_basis_is_orthogonal(S):
    U = S.ClusterBases.dimer.transformation
    np.testing.assert_allclose(U.T @ U, np.eye(4), atol=1e-15)


def test_dimer_magnet_hamiltonians(S):
    """test/models/test_cluster.jl:39-80."""
    model = S.ClusterModel(dimer_magnet_params(S))
    intra, inter = S.build_cluster_hamiltonians(model.uc_cluster_ids, model.lattice.uc.bonds,
                                                model.inner_model.bond_params, model.inner_model.site_spin_states)
    U = model.basis[0].transformation
    np.testing.assert_allclose(U.T @ intra[0] @ U, np.diag([-0.75, 0.25, 0.25, 0.25]), atol=1e-12)
    assert set(inter) == {(1, 1, (1, 0)), (1, 1, (0, 1))}
    expected = np.array([
        [1, 0, 0, 0, 0, 0, 0, 0, 0],
        [0, 0, 0, 1, 0, 0, 0, 0, 0],
        [0, 0, -1, 0, 1, 0, 0, 0, 0],
        [0, 1, 0, 0, 0, 0, 0, 0, 0],
        [0, 0, 1, 0, 0, 0, 1, 0, 0],
        [0, 0, 0, 0, 0, 0, 0, 1, 0],
        [0, 0, 0, 0, 1, 0, -1, 0, 0],
        [0, 0, 0, 0, 0, 1, 0, 0, 0],
        [0, 0, 0, 0, 0, 0, 0, 0, 1],
    ], dtype=float)
    UU = np.kron(U, U)
    for Hb in inter.values():
        H = (UU.T @ Hb @ UU).reshape(4, 4, 4, 4)  # [out_i, out_j, in_i, in_j]
        H[np.abs(H) < 1e-10] = 0
        trip = H[1:, 1:, 1:, 1:].reshape(9, 9)
        np.testing.assert_allclose(trip / trip[0, 0], expected, atol=1e-12)
        # singlets do not hop and only see the diagonal part
        assert not H[0, :, 0, :].any()
        assert not H[:, 0, :, 0].any()
        m = H[0, :, :, 0]
        assert np.array_equal(m, np.diag(np.diag(m)))
        m = H[:, 0, 0, :]
        assert np.array_equal(m, np.diag(np.diag(m)))
    sse = model.generate_sse_data()
    assert len(sse.bonds) == 8


def test_cluster_basis_count_checked(S):
    p = dimer_magnet_params(S)
    p["cluster_bases"] = (S.ClusterBases.dimer, S.ClusterBases.dimer)
    with pytest.raises(ValueError, match="does not match number of distinct"):
        S.ClusterModel(p)


def test_cluster_quantum_number_estimator_coefficients(S):
    """magnetization_state of a cluster model is the chosen quantum number of the basis state
    (cluster.jl:66-73); with the dimer's m the estimator measures the total S^z."""
    model = S.ClusterModel(cluster_job_params(S))
    flat = S.flatten_model(model)
    assert flat.est_prefixes == [""] and flat.maxdim == 4
    coef = flat.arrays["est_coef"].reshape(flat.nsites, 4)
    assert np.array_equal(coef, np.tile([0.0, 1.0, 0.0, -1.0], (flat.nsites, 1)))
    assert flat.norm_site_count == 8


@pytest.mark.parametrize("T", [0.04, 0.70, 2.02, 4.0])
def test_cluster_oracle_vs_ed(S, O, T):
    """The cluster job against ED of the inner magnet (the same Hamiltonian in another basis); the
    quantum-number-2 estimator is the uniform magnetisation of the inner model."""
    model = S.ClusterModel(cluster_job_params(S))
    flat = S.flatten_model(model)
    inner = S.MagnetModel(dict(cluster_job_params(S), measure=["magnetization"]))
    ed = ed_observables(S, inner, [T])
    bins = run_binned(O, flat, T, seed=124535, nbins=16, binsize=400, therm=1000)
    funcs = evaluables(flat.est_prefixes, flat.norm_site_count)
    bad = []
    for name in ("Energy", "SpecificHeat", "Mag", "AbsMag", "Mag2", "Mag4", "MagChi"):
        mc, err = jackknife(bins, funcs[name])
        ref = float(ed[name][0])
        z = abs(mc - ref) / (err if err != 0 else 1e-8)
        if z > 4:
            bad.append((name, mc, err, ref, z))
    assert not bad, bad
