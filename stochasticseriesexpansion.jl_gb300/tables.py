"""Flatten :class:`SSEData` and the estimator list into the device table layout.

The engine (and the CPU oracle) consume a model as a handful of flat arrays,
uploaded once.  Everything is 0-based except worm indices, which keep the
reference's 1-based numbering (src/worms.jl) so that ``worm_inverse`` reads
the same.

=================  ==========  ==================================================
array              dtype       meaning
=================  ==========  ==================================================
site_dims          int32[N]    local Hilbert space dimension per site
bond_type          int32[Nb]   vertex-table index of each bond
bond_sites         int32[2Nb]  the two sites of each bond
type_dims          int32[2T]   site dims of each bond type
type_nverts        int32[T]    vertex count per type
type_maxworm       int32[T]    max worm count per type
type_diag_off      int32[T]    offset into ``diag_vertex`` (d0*d1 entries per type)
type_vert_off      int32[T]    offset into ``weight``/``sign`` (and 4x into ``leg_state``)
type_trans_off     int32[T]    offset into ``trans_start``/``trans_count``
diag_vertex        int32       device vertex code of the diagonal vertex for the
                               compound state ``s0 + d0*s1`` (reference join_idx
                               convention, sse.jl:155-158), or -1
weight             float64     vertex weights
sign               int8        vertex signs
leg_state          uint8       leg states [v*4 + leg], 0-based
trans_start        int32       first outcome of (v, leg_in, worm_in) at
                               ``(v*4 + leg)*maxworm + worm-1``, -1 if invalid
trans_count        int32       number of outcomes (reference ``length + 1``)
out_cum            float64     cumulative probabilities
out_target         int32       device vertex code after the step
out_leg            int8        outgoing leg (0-based)
out_worm           int8        outgoing worm (1-based)
est_coef           float64     staggered_sign * magnetization_state per
                               (estimator, site, state): [e*N*maxdim + site*maxdim + s]
=================  ==========  ==================================================
"""

from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .util import DEV_MAX_BONDS, DEV_MAX_VERTICES, dev_vertex_code, ref_vertex_idx, ref_vertex_isinvalid


@dataclass
class FlatModel:
    nsites: int
    nbonds: int
    ntypes: int
    maxdim: int
    nest: int
    energy_offset: float
    norm_site_count: float
    arrays: dict = field(default_factory=dict)
    est_prefixes: list = field(default_factory=list)

    def __getitem__(self, k):
        return self.arrays[k]


def _dev_vcode_from_ref(code: int) -> int:
    if ref_vertex_isinvalid(code):
        return -1
    return dev_vertex_code(code & 1, ref_vertex_idx(code) - 1)


def flatten_sse_data(sse_data, estimators=(), model=None, norm_site_count=None) -> FlatModel:
    """Build the flat arrays for ``sse_data`` (src/sse_data.jl) and the magnetisation estimators.

    ``model`` supplies ``magnetization_state`` and ``lattice.staggered_sign``
    for the estimators (magnetization_estimator.jl:86-123).
    """
    for b in sse_data.bonds:
        if len(b.sites) != 2:
            raise ValueError("only two-site bonds (leg count 4) are supported")
        if b.sites[0] == b.sites[1]:
            raise ValueError(f"bond {b} connects a site to itself")
    N = len(sse_data.sites)
    Nb = len(sse_data.bonds)
    if Nb >= DEV_MAX_BONDS:
        raise ValueError(f"too many bonds for 32-bit operator codes ({Nb} >= {DEV_MAX_BONDS})")
    site_dims = np.array([s.dim for s in sse_data.sites], dtype=np.int32)
    if (site_dims <= 0).any():
        raise ValueError("every site must belong to at least one bond")
    bond_type = np.array([b.type - 1 for b in sse_data.bonds], dtype=np.int32)
    bond_sites = np.array([[b.sites[0] - 1, b.sites[1] - 1] for b in sse_data.bonds], dtype=np.int32).reshape(-1)

    T = len(sse_data.vertex_data)
    type_dims, type_nverts, type_maxworm = [], [], []
    type_diag_off, type_vert_off, type_trans_off = [], [], []
    diag_vertex, weight, sign, leg_state = [], [], [], []
    trans_start, trans_count = [], []
    out_cum, out_target, out_leg, out_worm = [], [], [], []

    for vd in sse_data.vertex_data:
        if len(vd.dims) != 2:
            raise ValueError("only two-site vertex tables are supported")
        nv = vd.vertex_count()
        if nv > DEV_MAX_VERTICES:
            raise ValueError(f"too many vertices per bond type ({nv} > {DEV_MAX_VERTICES})")
        mw = vd.max_worm_count
        type_dims += list(vd.dims)
        type_nverts.append(nv)
        type_maxworm.append(mw)
        type_diag_off.append(len(diag_vertex))
        type_vert_off.append(len(weight))
        type_trans_off.append(len(trans_start))
        diag_vertex += [_dev_vcode_from_ref(c) for c in vd.diagonal_vertices]
        weight += list(vd.weights)
        sign += list(vd.signs)
        for v in range(nv):
            leg_state += [int(x) - 1 for x in vd.leg_states[:, v]]
        out_base = len(out_cum)
        out_cum += list(vd.transition_cumprobs)
        out_target += [_dev_vcode_from_ref(c) for c in vd.transition_targets]
        out_leg += [lo - 1 for lo, _ in vd.transition_step_outs]
        out_worm += [wo for _, wo in vd.transition_step_outs]
        for v in range(1, nv + 1):
            for leg in range(1, 5):
                for worm in range(1, mw + 1):
                    t = vd.get_transition(leg, worm, v)
                    if t.isinvalid():
                        trans_start.append(-1)
                        trans_count.append(0)
                    else:
                        trans_start.append(out_base + t.offset - 1)
                        trans_count.append(t.length + 1)

    maxdim = int(site_dims.max())
    ests = list(estimators)
    est_coef = np.zeros(len(ests) * N * maxdim, dtype=np.float64)
    for e, spec in enumerate(ests):
        for site in range(1, N + 1):
            if hasattr(model, "staggered_sign"):
                sg = model.staggered_sign(spec, site)
            else:
                sg = model.lattice.staggered_sign(spec.ordering_vector, spec.stagger_uc, site)
            for s in range(site_dims[site - 1]):
                if spec.tag is None:
                    m = model.magnetization_state(site, s + 1)
                else:
                    m = model.magnetization_state(site, s + 1, spec.tag)
                est_coef[(e * N + site - 1) * maxdim + s] = sg * m

    if norm_site_count is None:
        norm_site_count = model.normalization_site_count() if model is not None else N

    arrays = dict(
        site_dims=site_dims,
        bond_type=bond_type,
        bond_sites=bond_sites,
        type_dims=np.array(type_dims, dtype=np.int32),
        type_nverts=np.array(type_nverts, dtype=np.int32),
        type_maxworm=np.array(type_maxworm, dtype=np.int32),
        type_diag_off=np.array(type_diag_off, dtype=np.int32),
        type_vert_off=np.array(type_vert_off, dtype=np.int32),
        type_trans_off=np.array(type_trans_off, dtype=np.int32),
        diag_vertex=np.array(diag_vertex, dtype=np.int32),
        weight=np.array(weight, dtype=np.float64),
        sign=np.array(sign, dtype=np.int8),
        leg_state=np.array(leg_state, dtype=np.uint8),
        trans_start=np.array(trans_start, dtype=np.int32),
        trans_count=np.array(trans_count, dtype=np.int32),
        out_cum=np.array(out_cum, dtype=np.float64),
        out_target=np.array(out_target, dtype=np.int32),
        out_leg=np.array(out_leg, dtype=np.int8),
        out_worm=np.array(out_worm, dtype=np.int8),
        est_coef=est_coef,
    )
    for k, a in arrays.items():
        arrays[k] = np.ascontiguousarray(a)
    return FlatModel(
        nsites=N,
        nbonds=Nb,
        ntypes=T,
        maxdim=maxdim,
        nest=len(ests),
        energy_offset=float(sse_data.energy_offset),
        norm_site_count=float(norm_site_count),
        arrays=arrays,
        est_prefixes=[s.prefix for s in ests],
    )


def flatten_model(model) -> FlatModel:
    """``generate_sse_data(model)`` plus its opstring estimators, flattened."""
    sd = model.generate_sse_data()
    return flatten_sse_data(sd, model.get_opstring_estimators(), model=model)
