"""Cluster-basis models (restatement of src/models/cluster/cluster.jl).

``ClusterModel`` rewrites an inner model -- here a :class:`MagnetModel` -- in
the basis of local clusters of its unit-cell sites, e.g. the singlet/triplet
basis of dimers, which removes the sign problem of some frustrated magnets.
Each cluster becomes one SSE site of dimension prod(site dims); the bonds
between clusters carry the inter-cluster Hamiltonian with the intra-cluster
terms absorbed into them, rotated into the cluster basis, and go through the
same vertex/LP table builder as every other model.  The GPU engine needs
nothing model-specific: it consumes the flattened tables.

Parameters (src/models/cluster/cluster.jl:14-25):

* ``inner_model``             the inner model class (``MagnetModel``)
* ``cluster_bases``           tuple of :class:`ClusterBasis`, one per cluster id
* ``cluster_id`` / ``parameter_map["cluster_id"]``  cluster id of each unit-cell site (default 1)
* ``measure_quantum_numbers`` list of ``{"name": str, "quantum_number": int}``: magnetisation
  estimators over a quantum number of the cluster basis
"""

from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from .abstract_model import AbstractModel
from .magnet import MagnetizationEstimatorSpec, MagnetModel, _get_parameter, generate_bond_hamiltonian
from .sse_data import SSEBond, SSEData
from .vertex_data import make_vertex_data


@dataclass(frozen=True)
class ClusterBasis:
    """cluster.jl:1-11: quantum numbers of every basis state, and the unitary whose columns are the
    basis states written in the product basis of the cluster's sites (first site slowest, as kron)."""

    quantum_numbers: tuple
    transformation: np.ndarray

    def __post_init__(self):
        T = np.asarray(self.transformation, dtype=float)
        if T.shape[0] != T.shape[1] or T.shape[1] != len(self.quantum_numbers):
            raise ValueError("a cluster basis needs one quantum-number tuple per column of a square transformation")
        object.__setattr__(self, "transformation", T)


def _dimer_basis() -> ClusterBasis:
    """Two spin-1/2 sites: singlet, then the triplet m = +1, 0, -1 (quantum numbers (S, m)).
    Product states are ordered (up,up), (up,down), (down,up), (down,down)."""
    r = 1 / math.sqrt(2)
    singlet = [0.0, r, -r, 0.0]
    t_plus = [1.0, 0.0, 0.0, 0.0]
    t_zero = [0.0, r, r, 0.0]
    t_minus = [0.0, 0.0, 0.0, 1.0]
    return ClusterBasis(((0.0, 0.0), (1.0, 1.0), (1.0, 0.0), (1.0, -1.0)),
                        np.array([singlet, t_plus, t_zero, t_minus]).T)


class ClusterBases:
    """Predefined cluster bases (cluster.jl:308-323)."""

    dimer = _dimer_basis()


def lift_twobody_operator(op, site_dims, sites) -> np.ndarray:
    """Embed a two-site operator ``op`` (on the kron product of sites[0], sites[1], in that order) into
    the product space of ``site_dims`` (first factor slowest, as kron), acting as the identity on the
    other factors (cluster.jl:79-126).  ``sites`` are 1-based."""
    site_dims = tuple(int(d) for d in site_dims)
    a, b = sites[0] - 1, sites[1] - 1
    if a == b:
        raise ValueError("the two sites of a two-body operator must differ")
    n = len(site_dims)
    op4 = np.asarray(op).reshape(site_dims[a], site_dims[b], site_dims[a], site_dims[b])
    # res[out..., in...] with factor k at axis k (out) and n + k (in)
    res = np.zeros(site_dims + site_dims, dtype=np.result_type(op4, float))
    others = [k for k in range(n) if k not in (a, b)]
    eye = np.ones(())
    for k in others:
        eye = np.multiply.outer(eye, np.eye(site_dims[k]))
    # eye axes: (o_k0, i_k0, o_k1, i_k1, ...); op4 axes: (o_a, o_b, i_a, i_b)
    full = np.multiply.outer(op4, eye)
    src = ["oa", "ob", "ia", "ib"] + [f"{io}{k}" for k in others for io in ("o", "i")]
    want = [f"o{k}" if k not in (a, b) else ("oa" if k == a else "ob") for k in range(n)]
    want += [f"i{k}" if k not in (a, b) else ("ia" if k == a else "ib") for k in range(n)]
    res = np.transpose(full, [src.index(w) for w in want])
    d = int(np.prod(site_dims))
    return res.reshape(d, d)


def build_cluster_hamiltonians(cluster_ids, uc_bonds, bond_params, site_spin_states):
    """cluster.jl:128-196.  ``cluster_ids``: 1-based id of each unit-cell site; ``bond_params``: the
    first cell's bond parameters in unit-cell bond order.  Returns the intra-cluster Hamiltonian of
    every cluster id and a dict (iuc, juc, jd) -> inter-cluster bond Hamiltonian, in first-appearance
    order of the unit-cell bonds."""
    ids = list(cluster_ids)
    order = list(dict.fromkeys(ids))
    if sorted(order) != list(range(1, len(order) + 1)):
        raise ValueError("cluster ids must be 1..number of clusters")
    clusters = {c: [i for i, x in enumerate(ids) if x == c] for c in order}
    cluster_dims = {c: tuple(int(site_spin_states[i]) for i in clusters[c]) for c in order}
    position = [0] * len(ids)
    for c in order:
        for k, i in enumerate(clusters[c]):
            position[i] = k + 1
    intra = {c: np.zeros((int(np.prod(cluster_dims[c])),) * 2) for c in order}
    inter = {}
    for ub, bp in zip(uc_bonds, bond_params):
        (di, dj), H, _ = generate_bond_hamiltonian(bp, (site_spin_states[ub.iuc - 1], site_spin_states[ub.juc - 1]))
        ci, cj = ids[ub.iuc - 1], ids[ub.juc - 1]
        if ci == cj and not any(ub.jd):
            if ub.iuc == ub.juc:
                raise ValueError("found bond in Magnet connecting site to itself... not supported by ClusterModel")
            intra[ci] = intra[ci] + lift_twobody_operator(H, cluster_dims[ci],
                                                          (position[ub.iuc - 1], position[ub.juc - 1]))
        else:
            key = (ci, cj, tuple(ub.jd))
            dims = cluster_dims[ci] + cluster_dims[cj]
            d = int(np.prod(dims))
            Hij = inter.setdefault(key, np.zeros((d, d)))
            inter[key] = Hij + lift_twobody_operator(
                H, dims, (position[ub.iuc - 1], len(cluster_dims[ci]) + position[ub.juc - 1]))
    return [intra[c] for c in range(1, len(order) + 1)], inter


def absorb_intracluster_hamiltonians(intra, inter):
    """cluster.jl:198-220: every inter-cluster bond type takes 1/coordination of the intra-cluster
    Hamiltonian of each of its two clusters (coordination counted over bond types)."""
    coord = [sum((k[0] == c) + (k[1] == c) for k in inter) for c in range(1, len(intra) + 1)]
    out = {}
    for k, H in inter.items():
        hi, hj = intra[k[0] - 1], intra[k[1] - 1]
        out[k] = (H + np.kron(hi, np.eye(hj.shape[0]) / coord[k[0] - 1])
                  + np.kron(np.eye(hi.shape[0]) / coord[k[1] - 1], hj))
    return out


class ClusterModel(AbstractModel):
    """cluster.jl:26-62."""

    def __init__(self, params: dict):
        inner = params["inner_model"](params)
        if not isinstance(inner, MagnetModel):
            raise TypeError("ClusterModel supports MagnetModel as the inner model")
        self.params = params
        self.inner_model = inner
        self.basis = tuple(params["cluster_bases"])
        pmap = params.get("parameter_map")
        nuc = len(inner.lattice.uc.sites)
        uc_ids = [int(params.get(_get_parameter(pmap, "cluster_id", i), 1)) for i in range(1, nuc + 1)]
        ncl = len(set(uc_ids))
        if ncl != len(self.basis):
            raise ValueError(f"Number of cluster bases ({len(self.basis)}) does not match number of distinct "
                             f"cluster ids ({ncl}).")
        self.uc_cluster_ids = uc_ids
        self.cluster_ids = uc_ids * int(np.prod(inner.lattice.Ls))
        for c, b in enumerate(self.basis, start=1):
            need = int(np.prod([inner.site_spin_states[i] for i in range(nuc) if uc_ids[i] == c]))
            if b.transformation.shape[0] != need:
                raise ValueError(f"cluster basis {c} has dimension {b.transformation.shape[0]}, the cluster {need}")
        self.opstring_estimators = [
            MagnetizationEstimatorSpec(tuple([False] * inner.lattice.dimension), False, str(m["name"]),
                                       int(m["quantum_number"]))
            for m in params.get("measure_quantum_numbers", [])
        ]

    @property
    def lattice(self):
        return self.inner_model.lattice

    @classmethod
    def leg_count(cls) -> int:
        return MagnetModel.leg_count()

    def normalization_site_count(self) -> int:
        return self.inner_model.normalization_site_count()

    def get_opstring_estimators(self):
        return self.opstring_estimators

    def magnetization_state(self, site_idx: int, state_idx: int, quantum_number: int = 1) -> float:
        """cluster.jl:66-73: quantum number ``quantum_number`` (1-based) of basis state ``state_idx`` of
        the cluster at SSE site ``site_idx``."""
        nuc_clusters = len(self.basis)
        cid = (site_idx - 1) % nuc_clusters + 1
        return float(self.basis[cid - 1].quantum_numbers[state_idx - 1][quantum_number - 1])

    def staggered_sign(self, spec, site_idx: int) -> int:
        """cluster.jl:75."""
        return 1

    def generate_sse_data(self) -> SSEData:
        """cluster.jl:242-306: the inter-cluster bonds of the lattice, duplicates merged, with one
        vertex table per bond type from U' H U, U = kron of the two cluster transformations."""
        mag = self.inner_model
        lat = mag.lattice
        nuc = len(lat.uc.sites)
        ncl = len(self.basis)
        intra, inter = build_cluster_hamiltonians(self.uc_cluster_ids, lat.uc.bonds, mag.bond_params[:len(lat.uc.bonds)],
                                                  mag.site_spin_states[:nuc])
        keys = list(inter)
        bonds = []
        seen = set()
        for b in lat.bonds:
            ub = lat.uc.bonds[b.type - 1]
            ci, cj = self.uc_cluster_ids[ub.iuc - 1], self.uc_cluster_ids[ub.juc - 1]
            if ci == cj and not any(ub.jd):
                continue
            i = ncl * ((b.i - 1) // nuc) + ci
            j = ncl * ((b.j - 1) // nuc) + cj
            sb = SSEBond(keys.index((ci, cj, tuple(ub.jd))) + 1, (i, j))
            if sb not in seen:
                seen.add(sb)
                bonds.append(sb)
        absorbed = absorb_intracluster_hamiltonians(intra, inter)
        vds = []
        for k in keys:
            U = np.kron(self.basis[k[0] - 1].transformation, self.basis[k[1] - 1].transformation)
            vds.append(make_vertex_data((intra[k[0] - 1].shape[0], intra[k[1] - 1].shape[0]), U.T @ absorbed[k] @ U,
                                        energy_offset_factor=0.25, lp_point=self.params.get("lp_point")))
        return SSEData.make(vds, bonds)
