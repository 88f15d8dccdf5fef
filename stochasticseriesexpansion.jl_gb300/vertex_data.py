"""Abstract-loop vertex tables (restatement of src/vertex_data.jl).

``VertexData(dims, H, energy_offset_factor=...)`` enumerates the vertices of a
bond Hamiltonian (vertex_data.jl:137-169) and solves one linear programme per
vertex-equivalence class for the worm scattering probabilities
(vertex_data.jl:213-416).  The reference solves the LP with HiGHS through
MathOptInterface; here it is ``scipy.optimize.linprog(method="highs")``.

All indices in this module follow the reference (1-based vertices, legs,
worms and states) so that the tables can be compared entry by entry with the
reference's own tests; :mod:`tables` converts them to the flat 0-based device
layout.  Where an LP optimum is not unique (S >= 1), the chosen optimal vertex
may differ from the reference's warm-started HiGHS run: such tables are valid
(detailed balance, normalisation) but their values are not pinned to the
reference.  The S=1/2 Heisenberg tables are unique and pinned by the known
answers in test/test_vertex_data.jl:111-130.
"""

from __future__ import annotations

import warnings
from dataclasses import dataclass

import numpy as np
from scipy.optimize import linprog

from .util import (
    join_idx,
    ref_vertex_code,
    ref_vertex_idx,
    ref_vertex_isinvalid,
    REF_INVALID_VERTEX,
    site_of_leg,
    split_idx,
    worm_action,
    worm_count,
    worm_inverse,
)


@dataclass
class Transition:
    """vertex_data.jl:6-11 -- ``offset`` is 1-based, ``length`` is count-1."""

    offset: int = -1
    length: int = 0

    def isinvalid(self) -> bool:
        return self.offset < 0


@dataclass
class VertexData:
    """vertex_data.jl:13-28.

    ``transitions`` is a dict ``(leg_in, worm_in, vertex) -> Transition`` with
    every missing key invalid (the reference's dense array of ``Transition()``).
    """

    energy_offset: float
    dims: tuple
    diagonal_vertices: list  # reference vertex codes, REF_INVALID_VERTEX if absent
    signs: list
    weights: list
    transitions: dict
    max_worm_count: int
    transition_cumprobs: list
    transition_targets: list
    transition_step_outs: list
    leg_states: np.ndarray  # [2*NSites, nverts], 1-based states

    @property
    def nsites(self) -> int:
        return len(self.dims)

    def vertex_count(self) -> int:
        return len(self.weights)

    def get_transition(self, leg_in: int, worm_in: int, vertex: int) -> Transition:
        return self.transitions.get((leg_in, worm_in, vertex), Transition())

    def get_vertex_weight(self, vcode: int) -> float:
        """vertex_data.jl:94-95."""
        return 0.0 if ref_vertex_isinvalid(vcode) else self.weights[ref_vertex_idx(vcode) - 1]

    def get_leg_state(self, vcode: int) -> np.ndarray:
        return self.leg_states[:, ref_vertex_idx(vcode) - 1]

    def scatter(self, vcode: int, leg_in: int, worm_in: int, random: float):
        """vertex_data.jl:106-125 (linear search over the cumulative table)."""
        t = self.get_transition(leg_in, worm_in, ref_vertex_idx(vcode))
        for out in range(t.offset, t.offset + t.length + 1):
            if random < self.transition_cumprobs[out - 1]:
                leg_out, worm_out = self.transition_step_outs[out - 1]
                return leg_out, worm_out, self.transition_targets[out - 1]
        return -1, -1, REF_INVALID_VERTEX


def calc_energy_offset(H: np.ndarray, energy_offset_factor: float) -> float:
    """vertex_data.jl:129-135."""
    d = np.diag(H)
    hmin = d.min()
    hmax = d.max()
    epsilon = (hmax - hmin) * energy_offset_factor
    return -(hmax + epsilon)


def _reversed_split(dims, i):
    return tuple(reversed(split_idx(tuple(reversed(dims)), i)))


def construct_vertices(dims, H, energy_offset, tolerance):
    """vertex_data.jl:137-169 -- column-major walk over the matrix elements."""
    D = H.shape[0]
    diagonal_vertices = [REF_INVALID_VERTEX] * D
    weights = []
    leg_states = []
    signs = []
    for j in range(1, D + 1):  # CartesianIndices: row index fastest
        for i in range(1, D + 1):
            w = -H[i - 1, j - 1]
            if i == j:
                w -= energy_offset
            if abs(w) > tolerance:
                if i == j:
                    # reversed because of the join_idx convention
                    reversed_i = join_idx(dims, _reversed_split(dims, i))
                    diagonal_vertices[reversed_i - 1] = ref_vertex_code(True, len(weights) + 1)
                leg_states.append(list(_reversed_split(dims, i)) + list(_reversed_split(dims, j)))
                weights.append(abs(w))
                signs.append(1 if w >= 0 else -1)
    ls = np.array(leg_states, dtype=np.uint8).T.reshape(2 * len(dims), len(weights))
    return diagonal_vertices, weights, ls, signs


def wrap_vertex_idx(leg_states: np.ndarray, vertex_idx):
    """vertex_data.jl:171-187."""
    if vertex_idx is None:
        return REF_INVALID_VERTEX
    leg_count = leg_states.shape[0]
    ls = leg_states[:, vertex_idx - 1]
    diagonal = True
    for s in range(leg_count // 2):
        diagonal &= bool(ls[s] == ls[leg_count // 2 + s])
    return ref_vertex_code(diagonal, vertex_idx)


def vertex_apply_change(leg_states, dims, vertex, step_in, step_out):
    """vertex_data.jl:192-211 -- returns a 1-based vertex index or ``None``."""
    nsites = len(dims)
    new = leg_states[:, vertex - 1].astype(np.int64).copy()
    leg_in, worm_in = step_in
    leg_out, worm_out = step_out
    dim_in = dims[site_of_leg(leg_in, nsites) - 1]
    dim_out = dims[site_of_leg(leg_out, nsites) - 1]
    new[leg_in - 1] = worm_action(worm_in, int(new[leg_in - 1]), dim_in)
    new[leg_out - 1] = worm_action(worm_out, int(new[leg_out - 1]), dim_out)
    match = np.nonzero(np.all(leg_states.astype(np.int64) == new[:, None], axis=0))[0]
    return int(match[0]) + 1 if len(match) else None


def _solve_lp(cost, A, b, lp_tolerance, lp_point):
    """The transition LP (vertex_data.jl:267-350): min bounces s.t. A x = b, x >= 0.

    lp_point = "vertex": a basic optimal solution (HiGHS simplex, like the reference's solver).
    lp_point = "central": a point inside the optimal face (HiGHS interior point without
    crossover), polished onto A x = b on its support.  The optimum is not unique for S >= 1;
    vertex solutions put probability 1 on many single outcomes.  A central optimum keeps every
    transition that some optimal solution allows, with the same (minimal) bounce weight.  With
    central tables no walker ran a worm past the step cap in sampled dimer-basis and S=1
    square-lattice runs; S=1 bilayer walkers still did, and mixed-spin honeycomb walkers began to.
    """
    import warnings as _w

    def vertex():
        res = linprog(cost, A_eq=A, b_eq=b, bounds=(0, None), method="highs",
                      options={"primal_feasibility_tolerance": lp_tolerance, "dual_feasibility_tolerance": lp_tolerance})
        if res.status != 0:
            raise RuntimeError(f"transition probability optimization failed: {res.message}")
        return res.x

    if lp_point == "vertex":
        return vertex()
    x0 = vertex()
    with _w.catch_warnings():
        _w.simplefilter("ignore")
        res = linprog(cost, A_eq=A, b_eq=b, bounds=(0, None), method="highs-ipm",
                      options={"run_crossover": "off", "presolve": False, "ipm_optimality_tolerance": 1e-12,
                               "primal_feasibility_tolerance": lp_tolerance, "dual_feasibility_tolerance": lp_tolerance})
    if res.status != 0 or res.x is None:
        return x0
    x = np.where(res.x > 1e-9 * max(1.0, float(np.abs(b).max())), res.x, 0.0)
    support = x > 0
    if not support.any():
        return x0
    As = A[:, support]
    for _ in range(3):  # least-squares projection onto A x = b on the support
        r = b - A @ x
        dx, *_ = np.linalg.lstsq(As, r, rcond=None)
        x[support] += dx
    if (x < 0).any() or np.abs(A @ x - b).max() > 1e-13 * max(1.0, float(np.abs(b).max())):
        return x0
    if float(cost @ x) > float(cost @ x0) + 1e-9:
        return x0
    return x


def construct_transitions(weights, leg_states, max_worm_count, dims, tolerance, lp_tolerance, lp_point="vertex"):
    """vertex_data.jl:213-416."""
    nsites = len(dims)
    leg_count = 2 * nsites
    nverts = len(weights)
    used_inaccurate_truncations = False

    transitions: dict = {}
    cumprobs: list = []
    targets_out: list = []
    step_outs: list = []

    steps = []
    inv_steps = {}
    step_idx = {}
    for worm in range(1, max_worm_count + 1):
        for leg in range(1, leg_count + 1):
            dim = dims[site_of_leg(leg, nsites) - 1]
            if worm <= worm_count(dim):
                steps.append((leg, worm))
                step_idx[(leg, worm)] = len(steps)
                inv_steps[(leg, worm)] = (leg, worm_inverse(worm, dim))

    def inverse(vc):
        return (inv_steps[vc[1]], inv_steps[vc[0]])

    variables = []
    var_set = set()
    for s_in in steps:
        for s_out in steps:
            vc = (s_in, s_out)
            if inverse(vc) not in var_set:
                variables.append(vc)
                var_set.add(vc)
    var_lookup = {}
    for vi, vc in enumerate(variables):
        var_lookup.setdefault(vc, vi)
        var_lookup.setdefault(inverse(vc), vi)

    cost = np.array([1.0 if vc == inverse(vc) else 0.0 for vc in variables])

    # one equality row per step: variables whose step_in (or inverse's step_in) is the step
    A = np.zeros((len(steps), len(variables)))
    for si, step in enumerate(steps):
        for xi, vc in enumerate(variables):
            if vc[0] == step or inverse(vc)[0] == step:
                A[si, xi] = 1.0

    def is_invalid(step, v):
        return (step[0], step[1], v) not in transitions

    while True:
        v = None
        step_in = None
        for empty_v in range(1, nverts + 1):
            found = next((s for s in steps if is_invalid(s, empty_v)), None)
            if found is not None:
                v = empty_v
                step_in = inv_steps[found]
                break
        if v is None:
            break

        targets = {}
        constraints = np.zeros(len(steps))
        for step_out in steps:
            target = vertex_apply_change(leg_states, dims, v, step_in, step_out)
            targets[step_out] = target
            constraints[step_idx[step_out] - 1] = weights[target - 1] if target is not None else 0.0

        solution = _solve_lp(cost, A, constraints, lp_tolerance, lp_point)

        for s_in in steps:
            if targets[s_in] is None:
                continue
            c = constraints[step_idx[s_in] - 1]
            norm = 1.0 if c == 0 else c
            offset = len(cumprobs) + 1
            length = -1
            for out in steps:
                var = var_lookup[(s_in, out)]
                assert solution[var] >= -lp_tolerance
                prob = solution[var] / norm
                if prob < 0.0:
                    used_inaccurate_truncations = prob < -tolerance
                    prob = 0.0
                assert solution[var] <= norm + lp_tolerance
                if prob > 1.0:
                    used_inaccurate_truncations = prob > 1 + tolerance
                    prob = 1.0
                if prob > tolerance / len(steps):
                    cumprobs.append(prob)
                    vc = variables[var]
                    in_inv = inverse(vc)[0] if vc[0] == s_in else vc[0]
                    targets_out.append(wrap_vertex_idx(leg_states, targets[in_inv]))
                    step_outs.append(out)
                    assert not ref_vertex_isinvalid(targets_out[-1])
                    length += 1
            transitions[(s_in[0], s_in[1], targets[s_in])] = Transition(offset, length)
            if length >= 0:
                seg = np.cumsum(cumprobs[offset - 1 : offset + length])
                if lp_point == "central" and abs(seg[-1] - 1) <= tolerance:
                    seg[-1] = 1.0  # polished solutions are normalised to ~1e-13; make the row exact
                cumprobs[offset - 1 : offset + length] = seg.tolist()
                if abs(seg[-1] - 1) > tolerance:
                    warnings.warn(f"normalization error: {seg[-1]} != 1")

    if used_inaccurate_truncations:
        warnings.warn("had to truncate some probabilities in a possibly inaccurate way!")
    return transitions, cumprobs, targets_out, step_outs


def make_vertex_data(dims, H, energy_offset_factor=0.25, tolerance=1e-7, lp_tolerance=1e-10,
                     lp_point=None) -> VertexData:
    """``VertexData(dims, bond_hamiltonian; ...)`` (vertex_data.jl:48-88).

    ``lp_point`` selects which optimal LP solution becomes the table (see ``_solve_lp``).  The
    default, "vertex", is a basic solution from the simplex method, the kind the reference's HiGHS
    run returns; "central" is an opt-in alternative.
    """
    if lp_point is None:
        lp_point = "vertex"
    dims = tuple(int(d) for d in dims)
    H = np.asarray(H, dtype=float)
    energy_offset = calc_energy_offset(H, energy_offset_factor)
    total_dim = int(np.prod(dims))
    max_worm_count = max(worm_count(d) for d in dims)
    diag, weights, leg_states, signs = construct_vertices(dims, H, energy_offset, tolerance)
    assert len(dims) >= 1
    assert total_dim == H.shape[0] == H.shape[1]
    assert leg_states.shape == (2 * len(dims), len(weights))
    transitions, cum, tgt, souts = construct_transitions(
        weights, leg_states, max_worm_count, dims, tolerance, lp_tolerance, lp_point
    )
    return VertexData(
        energy_offset=energy_offset,
        dims=dims,
        diagonal_vertices=diag,
        signs=signs,
        weights=weights,
        transitions=transitions,
        max_worm_count=max_worm_count,
        transition_cumprobs=cum,
        transition_targets=tgt,
        transition_step_outs=souts,
        leg_states=leg_states,
    )
