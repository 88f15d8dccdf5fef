"""Bond graph plus vertex tables (restatement of src/sse_data.jl)."""

from __future__ import annotations

from dataclasses import dataclass


@dataclass(frozen=True)
class SSESite:
    """sse_data.jl:1-3."""

    dim: int


@dataclass(frozen=True)
class SSEBond:
    """sse_data.jl:10-13 -- ``type`` is a 1-based index into ``vertex_data``; sites are 1-based."""

    type: int
    sites: tuple


@dataclass
class SSEData:
    """sse_data.jl:15-22."""

    vertex_data: list
    sites: list
    bonds: list
    energy_offset: float

    @staticmethod
    def make(vertex_data, bonds) -> "SSEData":
        """sse_data.jl:34-42: the energy offset is the sum over bonds of their type's offset."""
        energy_offset = 0.0
        for b in bonds:  # Julia sum() -- pairwise for long arrays; see tables.total_energy_offset
            energy_offset += vertex_data[b.type - 1].energy_offset
        sites = generate_sites_from_bonds(vertex_data, bonds)
        return SSEData(list(vertex_data), sites, list(bonds), energy_offset)

    def get_vertex_data(self, bond_idx: int):
        """sse_data.jl:70-71 (1-based bond)."""
        return self.vertex_data[self.bonds[bond_idx - 1].type - 1]


def generate_sites_from_bonds(vertex_data, bonds):
    """sse_data.jl:44-62 -- site dimensions implied by the bonds; inconsistent dims raise."""
    max_site = max(max(b.sites) for b in bonds)
    sites = [SSESite(0)] * max_site
    for b in bonds:
        for i_s, s in enumerate(b.sites):
            new_dim = vertex_data[b.type - 1].dims[i_s]
            if sites[s - 1].dim == 0:
                sites[s - 1] = SSESite(new_dim)
            elif sites[s - 1].dim != new_dim:
                raise ValueError(
                    f"SSEData: site dimensions set by VertexData are inconsistent!\n"
                    f"Site {s}: {sites[s - 1].dim}, Bond {b.type}: {new_dim}"
                )
    return sites
