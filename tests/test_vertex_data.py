"""Port of test/test_vertex_data.jl (detailed balance, S=1/2 known answers,
random Hamiltonians) plus the same checks on the flat device tables."""

import numpy as np
import pytest


def check_detailed_balance(S, vd):
    """test/test_vertex_data.jl:1-57."""
    import sse_gb300.util as U

    nsites = len(vd.dims)
    for v in range(1, vd.vertex_count() + 1):
        weight = vd.weights[v - 1]
        for (leg_in, worm_in, vv), t in vd.transitions.items():
            if vv != v or t.isinvalid():
                continue
            cum = vd.transition_cumprobs[t.offset - 1 : t.offset + t.length]
            probs = np.diff(np.concatenate([[0.0], cum]))
            targets = vd.transition_targets[t.offset - 1 : t.offset + t.length]
            outs = vd.transition_step_outs[t.offset - 1 : t.offset + t.length]
            for prob, target, (leg_out, worm_out) in zip(probs, targets, outs):
                t_inv = vd.get_transition(
                    leg_out,
                    S.worm_inverse(worm_out, vd.dims[S.site_of_leg(leg_out, nsites) - 1]),
                    U.ref_vertex_idx(target),
                )
                inv_targets = [U.ref_vertex_idx(x) for x in vd.transition_targets[t_inv.offset - 1 : t_inv.offset + t_inv.length]]
                assert v in inv_targets
                i_inv = inv_targets.index(v)
                probs_back = np.diff(np.concatenate([[0.0], vd.transition_cumprobs[t_inv.offset - 1 : t_inv.offset + t_inv.length]]))
                assert prob * weight == pytest.approx(probs_back[i_inv] * vd.get_vertex_weight(target), rel=1e-7, abs=1e-9)


def heisenberg_bond(S):
    sp, sz = S.spin_operators(2)
    return np.kron(sz, sz) + 0.5 * (np.kron(sp, sp.T) + np.kron(sp.T, sp))


def test_vertex_apply_change_inverse(S):
    # test/test_vertex_data.jl:63-79
    from sse_gb300.vertex_data import vertex_apply_change
    import itertools

    dim, nsites = 4, 2
    legs = np.array(list(itertools.product(range(1, dim + 1), repeat=2 * nsites)), dtype=np.uint8)[:, ::-1].T
    rng = np.random.default_rng(3)
    for leg in range(1, 2 * nsites + 1):
        for worm in range(1, S.worm_count(dim) + 1):
            v = int(rng.integers(1, dim ** (2 * nsites) + 1))
            assert vertex_apply_change(legs, (dim,) * 2, v, (leg, worm), (leg, S.worm_inverse(worm, dim))) == v


def test_s12_heisenberg_known_answers(S):
    # test/test_vertex_data.jl:81-100
    import sse_gb300.util as U

    vd = S.make_vertex_data((2, 2), heisenberg_bond(S), energy_offset_factor=0.0)
    check_detailed_balance(S, vd)
    assert vd.energy_offset == pytest.approx(-0.25)
    assert sum(U.ref_vertex_isinvalid(c) for c in vd.diagonal_vertices) == 2
    assert np.allclose(vd.weights, 0.5)
    assert np.allclose(vd.transition_cumprobs, np.ones(16))
    for vertex in range(1, vd.vertex_count() + 1):
        for leg in range(1, 5):
            t = vd.get_transition(leg, 1, vertex)
            assert vd.transition_step_outs[t.offset - 1][0] == ((leg - 1) ^ 1) + 1


@pytest.mark.parametrize("dims", [(4, 4), (2, 4)])
def test_random_hamiltonian(S, dims):
    # test/test_vertex_data.jl:102-135
    rng = np.random.default_rng(11)
    H = rng.random((int(np.prod(dims)), int(np.prod(dims))))
    vd = S.make_vertex_data(dims, H)
    check_detailed_balance(S, vd)
    for v in range(vd.vertex_count()):
        assert all(vd.leg_states[:, v] <= np.array(dims + dims))
    for state in range(1, int(np.prod(dims)) + 1):
        split = S.split_idx(dims, state)
        diag = vd.get_leg_state(vd.diagonal_vertices[state - 1])
        assert list(diag) == list(split) + list(split)
    for (leg, worm, v), t in vd.transitions.items():
        if worm > S.worm_count(dims[S.site_of_leg(leg, 2) - 1]):
            assert t.isinvalid()
        assert t.isinvalid() or vd.transition_cumprobs[t.offset + t.length - 1] == pytest.approx(1.0)


def test_magnet_s12_tables_factor_quarter(S):
    """MagnetModel always builds factor-0.25 tables (see magnet.generate_bond_hamiltonian)."""
    m = S.MagnetModel({"lattice": {"unitcell": S.UnitCells.square, "size": (4, 4)}, "J": 1.0})
    vd = m.generate_sse_data().vertex_data[0]
    assert vd.energy_offset == pytest.approx(-0.375)
    assert sorted(vd.weights) == pytest.approx([0.125, 0.125, 0.5, 0.5, 0.625, 0.625])
    check_detailed_balance(S, vd)


def test_s1_bilayer_tables_valid(S):
    p = {"lattice": {"unitcell": S.UnitCells.square_bilayer, "size": (3, 3)}, "S": 1, "J1": 0.5, "J2": 1.0,
         "parameter_map": {"J": ["J1", "J2", "J2", "J2", "J2"]}, "Dz": 0.3, "hz": 0.2}
    p["J"] = 1.0
    m = S.MagnetModel(p)
    sd = m.generate_sse_data()
    assert len(sd.vertex_data) == 5
    for vd in sd.vertex_data:
        check_detailed_balance(S, vd)
    flat = S.flatten_model(m)
    # every valid transition row of the flat table is normalised
    a = flat.arrays
    for start, cnt in zip(a["trans_start"], a["trans_count"]):
        if start >= 0 and cnt > 0:
            assert a["out_cum"][start + cnt - 1] == pytest.approx(1.0, abs=1e-6)
