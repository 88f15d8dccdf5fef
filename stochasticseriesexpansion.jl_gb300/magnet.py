"""Quantum magnet model (restatement of src/models/magnet/magnet.jl) and the
magnetisation estimators (src/models/common/magnetization_estimator.jl).

Parameters are a plain ``dict`` with the reference's symbol names as string
keys (``"J"``, ``"d"``, ``"hz"``, ``"Dz"``, ``"Dx"``, ``"S"``, ``"lattice"``,
``"parameter_map"``, ``"measure"``).  Spins are given as ``fractions.Fraction``
or floats (``S=0.5`` and ``Fraction(1, 2)`` are the same).
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .abstract_model import AbstractModel
from .lattice import Lattice, neel_vector
from .operators import spin_operators
from .sse_data import SSEBond, SSEData
from .vertex_data import make_vertex_data


@dataclass(frozen=True)
class MagnetBondParams:
    """magnet.jl:1-19."""

    J: float
    d: float
    Dx: tuple
    Dz: tuple
    hz: tuple


@dataclass(frozen=True)
class MagnetizationEstimatorSpec:
    """Type parameters of ``MagnetizationEstimator{OrderingVector,StaggerUC,Model,Prefix,Tag}``
    (magnetization_estimator.jl:32-48)."""

    ordering_vector: tuple
    stagger_uc: bool
    prefix: str
    tag: int | None = None  # quantum-number index for cluster models (cluster.jl:222-240)


def magnetization_estimator_standard_prefix(q, stagger_uc: bool) -> str:
    """magnetization_estimator.jl:172-180."""
    if not any(q) and not stagger_uc:
        return ""

    def direction_name(i):  # mod('X' - 'A' + i - 1, 26) + 'A'
        return chr((ord("X") - ord("A") + i - 1) % 26 + ord("A"))

    return "Stag" + "".join(direction_name(i + 1) for i, x in enumerate(q) if x) + ("uc" if stagger_uc else "")


def all_magnetization_estimators(dimension: int):
    """magnetization_estimator.jl:55-70 -- stagger_uc outer... (Julia comprehension: first
    generator varies fastest, i.e. stagger_uc fastest, then q with its first component fastest)."""
    import itertools

    out = []
    for q_rev in itertools.product((False, True), repeat=dimension):
        q = tuple(reversed(q_rev))
        for stagger_uc in (False, True):
            out.append(MagnetizationEstimatorSpec(q, stagger_uc, magnetization_estimator_standard_prefix(q, stagger_uc)))
    return out


def magnetization_estimator_obs_names(prefix: str):
    """magnetization_estimator.jl:192-202: observable names and their sign-weighted twins."""
    names = ["Mag", "AbsMag", "Mag2", "Mag4", "MagChi", "BinderRatio"]
    return [prefix + n for n in names], ["Sign" + prefix + n for n in names]


def _get_parameter(parameter_map, name: str, index: int) -> str:
    """magnet.jl:68-79 (1-based index into the map entry)."""
    if parameter_map is None:
        return name
    if name not in parameter_map:
        return name
    entry = parameter_map[name]
    if not (1 <= index <= len(entry)):
        return name
    return entry[index - 1]


class MagnetModel(AbstractModel):
    """magnet.jl:54-120."""

    LEG_COUNT = 4

    def __init__(self, params: dict):
        self.params = params
        lattice = params["lattice"]
        if not isinstance(lattice, Lattice):
            lattice = Lattice.from_params(lattice)
        self.lattice = lattice
        assert len(lattice.bonds) > 0
        pmap = params.get("parameter_map")

        def pm(name, index):
            return _get_parameter(pmap, name, index)

        def split_site(param, bond, default):
            iuc, _ = lattice.split_idx(bond.i)
            juc, _ = lattice.split_idx(bond.j)
            first = params.get(pm(param, iuc), default) / lattice.uc.sites[iuc - 1].coordination
            second = params.get(pm(param, juc), default) / lattice.uc.sites[juc - 1].coordination
            return (first, second)

        self.bond_params = [
            MagnetBondParams(
                float(params[pm("J", b.type)]),
                float(params.get(pm("d", b.type), 0.0)),
                split_site("Dx", b, 0.0),
                split_site("Dz", b, 0.0),
                split_site("hz", b, 0.0),
            )
            for b in lattice.bonds
        ]
        uc_spin_states = [int(round(float(params.get(pm("S", i), 0.5)) * 2 + 1)) for i in range(1, len(lattice.uc.sites) + 1)]
        self.site_spin_states = uc_spin_states * int(np.prod(lattice.Ls))
        self.opstring_estimators = gen_opstring_estimators(lattice, params)

    # ---- AbstractModel interface (src/abstract_model.jl) ----
    @classmethod
    def leg_count(cls) -> int:
        return cls.LEG_COUNT

    def normalization_site_count(self) -> int:
        return self.lattice.site_count()

    def get_opstring_estimators(self):
        return self.opstring_estimators

    def magnetization_state(self, site_idx: int, state_idx: int) -> float:
        """magnet.jl:122-129 (1-based site and state)."""
        return (self.site_spin_states[site_idx - 1] - 1) * 0.5 - state_idx + 1

    def generate_sse_data(self) -> SSEData:
        """magnet.jl:169-184: one VertexData per unit-cell bond, built from the first cell's bond parameters."""
        uc = self.lattice.uc
        vds = []
        for uc_bond, bp in zip(uc.bonds, self.bond_params):
            dims, H, factor = generate_bond_hamiltonian(
                bp, (self.site_spin_states[uc_bond.iuc - 1], self.site_spin_states[uc_bond.juc - 1])
            )
            vds.append(make_vertex_data(dims, H, energy_offset_factor=factor, lp_point=self.params.get("lp_point")))
        bonds = [SSEBond(b.type, (b.i, b.j)) for b in self.lattice.bonds]
        return SSEData.make(vds, bonds)


def generate_bond_hamiltonian(bond: MagnetBondParams, spin_states):
    """magnet.jl:133-165.

    The reference picks ``energy_offset_factor = 0`` only when
    ``bond.hz == 0 && bond.Dz == 0 && bond.Dx == 0``.  Those fields are
    2-tuples, and a tuple never equals the integer 0 in Julia, so that branch
    is never taken and every MagnetModel bond uses 0.25.  The restatement keeps
    that behaviour so that tables (and therefore trajectories) match.
    """
    dimi, dimj = spin_states
    splusi, szi = spin_operators(dimi)
    splusj, szj = spin_operators(dimj)
    idi = np.eye(dimi)
    idj = np.eye(dimj)
    kron = np.kron
    H = (
        bond.J * (0.5 * (kron(splusi.T, splusj) + kron(splusi, splusj.T)) + (1 + bond.d) * kron(szi, szj))
        + bond.hz[0] * kron(idi, szj)
        + bond.hz[1] * kron(szi, idj)
        + bond.Dx[0] / 4 * kron(np.linalg.matrix_power(splusi + splusi.T, 2), idj)
        + bond.Dx[1] / 4 * kron(idi, np.linalg.matrix_power(splusj + splusj.T, 2))
        + bond.Dz[0] * kron(szi @ szi, idj)
        + bond.Dz[1] * kron(idi, szj @ szj)
    )
    energy_offset_factor = 0.25
    # tuple == 0 is false in the reference: the deterministic S=1/2 branch is dead code there
    return (dimi, dimj), H, energy_offset_factor


def gen_opstring_estimators(lattice: Lattice, params: dict):
    """magnet.jl:186-209."""
    ests = []
    for est in params.get("measure", []):
        if est == "magnetization":
            ests.append(MagnetizationEstimatorSpec(tuple([False] * lattice.dimension), False, ""))
        elif est == "staggered_magnetization":
            neel = neel_vector(lattice.uc)
            if neel is None:
                raise ValueError("selected :staggered_magnetization measurement, but lattice does not have a Neel vector.")
            q, stagger_uc = neel
            ests.append(MagnetizationEstimatorSpec(q, stagger_uc, "Stag"))
        elif isinstance(est, MagnetizationEstimatorSpec):
            ests.append(est)
        else:
            raise ValueError(f"Unrecognized measure option '{est}'")
    return ests
