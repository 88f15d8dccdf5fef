"""Unit cells and periodic lattices (restatement of src/models/common/lattice.jl).

Site and bond enumeration order follows lattice.jl:223-243 exactly (unit-cell
index fastest, then the first lattice direction), because bond indices end up
inside the operator codes and site indices inside the spin state.
"""

from __future__ import annotations

import itertools
from dataclasses import dataclass, field

import numpy as np

from .util import join_idx, split_idx


@dataclass(frozen=True)
class UCBond:
    """lattice.jl:14-18 -- bond from unit-cell site ``iuc`` to ``juc`` in the cell offset by ``jd``."""

    iuc: int
    jd: tuple
    juc: int


@dataclass
class UCSite:
    """lattice.jl:34-40."""

    pos: tuple
    sublattice_sign: int = 0
    coordination: int = 0


def calculate_uc_signs(bonds, num_sites):
    """lattice.jl:74-102.

    The reference loop never ends for a unit cell whose sites are not all
    reached by intra-cell bonds; the iteration cap below only changes that
    non-terminating case (all signs then fall back to +1, as the reference's
    post-loop fallback does).
    """
    signs = [0] * num_sites
    signs[0] = 1
    tries = 0
    guard = 0
    while any(s == 0 for s in signs) or tries > len(bonds) ** 2:
        guard += 1
        if guard > 4 * (len(bonds) + 1) ** 2 + 16:
            break
        for b in bonds:
            if any(x != 0 for x in b.jd):
                continue
            i, j = b.iuc - 1, b.juc - 1
            if signs[i] != 0 and signs[j] == 0:
                signs[j] = -signs[i]
            elif signs[j] != 0 and signs[i] == 0:
                signs[i] = -signs[j]
            elif signs[i] == signs[j]:
                signs = [1] * num_sites  # lattice not bipartite
                break
            tries += 1
    if any(s == 0 for s in signs):
        signs = [1] * num_sites
    return signs


def calculate_uc_coordinations(bonds, num_sites):
    """lattice.jl:104-113."""
    c = [0] * num_sites
    for b in bonds:
        c[b.iuc - 1] += 1
        c[b.juc - 1] += 1
    return c


@dataclass
class UnitCell:
    """lattice.jl:67-132."""

    lattice_vectors: np.ndarray
    sites: list
    bonds: list

    @staticmethod
    def make(lattice_vectors, sites, bonds) -> "UnitCell":
        signs = calculate_uc_signs(bonds, len(sites))
        coords = calculate_uc_coordinations(bonds, len(sites))
        return UnitCell(
            np.asarray(lattice_vectors, dtype=float),
            [UCSite(s.pos, sg, c) for s, sg, c in zip(sites, signs, coords)],
            list(bonds),
        )

    @property
    def dimension(self) -> int:
        return len(self.sites[0].pos)


def neel_vector(uc: UnitCell):
    """lattice.jl:134-150 -- ``(q, stagger_uc)`` or ``None``; q iterates first component fastest."""
    D = uc.dimension
    for stagger_uc in (False, True):
        for q_rev in itertools.product((False, True), repeat=D):
            q = tuple(reversed(q_rev))  # Iterators.product: first component fastest
            ok = True
            for b in uc.bonds:
                signi = uc.sites[b.iuc - 1].sublattice_sign ** int(stagger_uc)
                signj = uc.sites[b.juc - 1].sublattice_sign ** int(stagger_uc) * (
                    (-1) ** sum(int(x) * int(y) for x, y in zip(b.jd, q))
                )
                if signi == signj:
                    ok = False
                    break
            if ok:
                return q, stagger_uc
    return None


@dataclass(frozen=True)
class LatticeBond:
    """lattice.jl:165-169 (1-based type and sites)."""

    type: int
    i: int
    j: int


@dataclass(frozen=True)
class LatticeSite:
    iuc: int
    ix: tuple


@dataclass
class Lattice:
    """lattice.jl:210-243."""

    uc: UnitCell
    Ls: tuple
    bonds: list = field(default_factory=list)
    sites: list = field(default_factory=list)

    @staticmethod
    def make(uc: UnitCell, Ls) -> "Lattice":
        Ls = tuple(int(x) for x in Ls)
        dims = (len(uc.sites),) + Ls
        bonds = []
        sites = []
        # Iterators.product(1:L1, 1:L2, ...) -- first component fastest
        for r_rev in itertools.product(*[range(1, L + 1) for L in reversed(Ls)]):
            r = tuple(reversed(r_rev))
            for bond_type, b in enumerate(uc.bonds, start=1):
                assert 1 <= b.iuc <= len(uc.sites)
                assert 1 <= b.juc <= len(uc.sites)
                i = join_idx(dims, (b.iuc,) + r)
                jr = tuple((x + d - 1) % L + 1 for x, d, L in zip(r, b.jd, Ls))
                j = join_idx(dims, (b.juc,) + jr)
                bonds.append(LatticeBond(bond_type, i, j))
            for iuc in range(1, len(uc.sites) + 1):
                sites.append(LatticeSite(iuc, r))
        return Lattice(uc, Ls, bonds, sites)

    @staticmethod
    def from_params(p) -> "Lattice":
        """``Lattice(params[:lattice])`` with ``unitcell`` and ``size`` keys (lattice.jl:221)."""
        if isinstance(p, dict):
            return Lattice.make(p["unitcell"], p["size"])
        return Lattice.make(p.unitcell, p.size)

    @property
    def dimension(self) -> int:
        return len(self.Ls)

    def site_count(self) -> int:
        return len(self.uc.sites) * int(np.prod(self.Ls))

    def split_idx(self, site_idx: int):
        r = split_idx((len(self.uc.sites),) + self.Ls, site_idx)
        return r[0], r[1:]

    def staggered_sign(self, ordering_vector, stagger_uc: bool, site_idx: int) -> int:
        """lattice.jl:257-267 (1-based site)."""
        s = self.sites[site_idx - 1]
        sign = self.uc.sites[s.iuc - 1].sublattice_sign if stagger_uc else 1
        parity = sum(int(q) * x for q, x in zip(ordering_vector, s.ix)) % 2
        return sign * (1 - 2 * parity)


class UnitCells:
    """Predefined unit cells (lattice.jl:280-331) plus the square bilayer used
    by the S=1 benchmark workload, which the reference does not predefine."""

    square = UnitCell.make(
        [[1.0, 0.0], [0.0, 1.0]],
        [UCSite((0.0, 0.0))],
        [UCBond(1, (0, 1), 1), UCBond(1, (1, 0), 1)],
    )
    columnar_dimer = UnitCell.make(
        [[1.0, 0.0], [0.0, 2.0]],
        [UCSite((0.0, 0.0)), UCSite((0.0, 0.5))],
        [UCBond(1, (0, 0), 2), UCBond(1, (1, 0), 1), UCBond(2, (1, 0), 2), UCBond(2, (0, 1), 1)],
    )
    honeycomb = UnitCell.make(
        [[np.sqrt(3) / 2, np.sqrt(3 / 2)], [-0.5, 0.5]],
        [UCSite((0.0, 0.0)), UCSite((1 / 3, 1 / 3))],
        [UCBond(1, (0, 0), 2), UCBond(2, (0, 1), 1), UCBond(2, (1, 0), 1)],
    )
    triangle = UnitCell.make(
        [[1.0, -0.5], [0.0, np.sqrt(3 / 2)]],
        [UCSite((0.0, 0.0))],
        [UCBond(1, (0, 1), 1), UCBond(1, (1, 0), 1), UCBond(1, (1, 1), 1)],
    )
    fully_frust_square_bilayer = UnitCell.make(
        [[1.0, 0.0], [0.0, 1.0]],
        [UCSite((0.0, 0.0)), UCSite((0.0, 0.0))],
        [
            UCBond(1, (0, 0), 2),
            UCBond(1, (0, 1), 1),
            UCBond(2, (0, 1), 2),
            UCBond(1, (1, 0), 1),
            UCBond(2, (1, 0), 2),
            UCBond(1, (0, 1), 2),
            UCBond(2, (0, 1), 1),
            UCBond(1, (1, 0), 2),
            UCBond(2, (1, 0), 1),
        ],
    )
    # Two-site square bilayer: bond 1 is the interlayer rung, bonds 2-5 the
    # intralayer nearest neighbours of each layer.  Used with
    # parameter_map J = [J_perp, J, J, J, J].
    square_bilayer = UnitCell.make(
        [[1.0, 0.0], [0.0, 1.0]],
        [UCSite((0.0, 0.0)), UCSite((0.0, 0.0))],
        [
            UCBond(1, (0, 0), 2),
            UCBond(1, (1, 0), 1),
            UCBond(1, (0, 1), 1),
            UCBond(2, (1, 0), 2),
            UCBond(2, (0, 1), 2),
        ],
    )
