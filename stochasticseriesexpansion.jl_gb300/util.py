"""Index helpers, worm functions and operator codes.

Mirrors the reference's small building blocks:

* ``split_idx`` / ``join_idx``   -- src/util.jl:3-23 (mixed radix, first index fastest)
* ``worm_action`` & co.          -- src/worms.jl:1-7
* ``VertexCode`` / ``OperCode``  -- src/opercode.jl:1-71 (reference UInt64 layout)

The GPU engine stores operators as 32-bit codes.  Only the *mapping*
(bond, vertex index, diagonal flag) has to be preserved, not the bits, so the
device layout is

    bit 0        1 for a non-identity operator (identity = 0)
    bit 1        diagonal flag
    bits 2..10   vertex index, 0-based (at most 512 vertices per bond type)
    bits 11..31  bond index, 0-based (at most 2**21 bonds)

``ref_to_dev`` / ``dev_to_ref`` convert between the two so that opstrings can
round-trip through the reference's checkpoint format (src/sse.jl:89-107).
"""

from __future__ import annotations

import numpy as np

# --------------------------------------------------------------------------
# src/util.jl
# --------------------------------------------------------------------------


def split_idx(dims, idx: int) -> tuple:
    """1-based mixed-radix split, first dimension fastest (src/util.jl:3-13)."""
    idx -= 1
    r = []
    for d in dims:
        r.append(idx % d + 1)
        idx //= d
    return tuple(r)


def join_idx(dims, idxs) -> int:
    """Inverse of :func:`split_idx` (src/util.jl:15-23)."""
    r = 0
    for idx, d in zip(reversed(tuple(idxs)), reversed(tuple(dims))):
        r *= d
        r += idx - 1
    return r + 1


# --------------------------------------------------------------------------
# src/worms.jl
# --------------------------------------------------------------------------


def worm_action(worm: int, state: int, basis_size: int) -> int:
    """src/worms.jl:4 -- 1-based worm acting on a 1-based state."""
    return (state + worm - 1) % basis_size + 1


def worm_inverse(worm: int, basis_size: int) -> int:
    """src/worms.jl:6."""
    return basis_size - worm


def worm_count(basis_size: int) -> int:
    """src/worms.jl:7."""
    return basis_size - 1


def site_of_leg(leg: int, num_sites: int) -> int:
    """src/vertex_data.jl:190 (1-based legs and sites)."""
    return leg - num_sites if leg > num_sites else leg


# --------------------------------------------------------------------------
# src/opercode.jl  (reference 64-bit layout)
# --------------------------------------------------------------------------

VERTEX_CODE_MAXBITS = 8 * 3 + 1  # src/opercode.jl:2
REF_INVALID_VERTEX = (1 << VERTEX_CODE_MAXBITS) + 1  # VertexCode(nothing)


def ref_vertex_code(diagonal: bool, vertex_idx: int) -> int:
    """VertexCode(diagonal, vertex_idx) with a 1-based index (src/opercode.jl:16-19)."""
    return int(bool(diagonal)) | (int(vertex_idx) << 1)


def ref_vertex_isinvalid(code: int) -> bool:
    return code >= (1 << VERTEX_CODE_MAXBITS)


def ref_vertex_isdiagonal(code: int) -> bool:
    return bool(code & 1)


def ref_vertex_idx(code: int) -> int:
    return code >> 1


def ref_opercode(bond: int, vertex_code: int) -> int:
    """OperCode(bond, vertex) with a 1-based bond (src/opercode.jl:43-47)."""
    return 1 | (vertex_code << 1) | (bond << (1 + VERTEX_CODE_MAXBITS))


def ref_get_bond(op: int) -> int:
    return op >> (1 + VERTEX_CODE_MAXBITS)


def ref_get_vertex(op: int) -> int:
    return (op & ((1 << VERTEX_CODE_MAXBITS) - 1)) >> 1


# --------------------------------------------------------------------------
# device 32-bit layout
# --------------------------------------------------------------------------

DEV_VERTEX_BITS = 9
DEV_BOND_SHIFT = 11
DEV_MAX_VERTICES = 1 << DEV_VERTEX_BITS
DEV_MAX_BONDS = 1 << (32 - DEV_BOND_SHIFT)
DEV_INVALID_VERTEX = -1


def dev_vertex_code(diagonal: bool, vertex_idx0: int) -> int:
    """Device vertex code: diagonal flag in bit 0, 0-based index above it."""
    return int(bool(diagonal)) | (int(vertex_idx0) << 1)


def dev_opercode(bond0: int, vcode: int) -> int:
    return (1 | (vcode << 1) | (bond0 << DEV_BOND_SHIFT)) & 0xFFFFFFFF


def dev_get_bond(op: int) -> int:
    return (op & 0xFFFFFFFF) >> DEV_BOND_SHIFT


def dev_get_vcode(op: int) -> int:
    return (op >> 1) & ((1 << (DEV_VERTEX_BITS + 1)) - 1)


def dev_isdiagonal(op: int) -> bool:
    return bool((op >> 1) & 1)


def ref_to_dev(ops_ref) -> np.ndarray:
    """Reference UInt64 opcodes -> device uint32 opcodes."""
    ops_ref = np.asarray(ops_ref, dtype=np.uint64)
    out = np.zeros(len(ops_ref), dtype=np.uint32)
    for i, op in enumerate(ops_ref.tolist()):
        if op == 0:
            continue
        v = ref_get_vertex(op)
        out[i] = dev_opercode(ref_get_bond(op) - 1, dev_vertex_code(v & 1, (v >> 1) - 1))
    return out


def dev_to_ref(ops_dev) -> np.ndarray:
    """Device uint32 opcodes -> reference UInt64 opcodes."""
    ops_dev = np.asarray(ops_dev, dtype=np.uint32)
    out = np.zeros(len(ops_dev), dtype=np.uint64)
    for i, op in enumerate(ops_dev.tolist()):
        if op == 0:
            continue
        vc = dev_get_vcode(op)
        out[i] = ref_opercode(dev_get_bond(op) + 1, ref_vertex_code(vc & 1, (vc >> 1) + 1))
    return out
