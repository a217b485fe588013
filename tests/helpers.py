"""Shared helpers of the parity tests."""

import numpy as np
import scipy.sparse as sp

from easyfea_gb300.mesh import ElemType, GroupElem, Mesh


def boundary_groups(g):
    """[(element type, connect)] of a fixture's boundary groups: belem /
    bconnect, and belem2 / bconnect2 where the mesh has a second face type
    (the prisms' quadrangles and triangles)."""
    out = [(str(g["belem"]), g["bconnect"])]
    if "belem2" in g:
        out.append((str(g["belem2"]), g["bconnect2"]))
    return out


def mesh_from_golden(g) -> Mesh:
    coord = np.asarray(g["coord"], dtype=float)
    groups = {ElemType(e): GroupElem(ElemType(e), c, coord) for e, c in boundary_groups(g)}
    groups[ElemType(str(g["elem"]))] = GroupElem(ElemType(str(g["elem"])), g["connect"], coord)
    return Mesh(groups)


def csr(g, p, n):
    return sp.csr_matrix((g[p + "_data"], g[p + "_indices"], g[p + "_indptr"]), shape=(n, n))


def row_scaled_err(A, B):
    """max_ij |A_ij - B_ij| / max_j |B_ij| (the K parity metric)."""
    D = (A - B).tocsr()
    D.eliminate_zeros()
    if D.nnz == 0:
        return 0.0
    rmax = abs(B).tocsr().max(axis=1).toarray().ravel()
    dmax = abs(D).max(axis=1).toarray().ravel()
    rmax[rmax == 0] = 1
    return float(np.max(dmax / rmax))


def same_pattern(A, B):
    return np.array_equal(np.asarray(A.indptr, np.int64), np.asarray(B.indptr, np.int64)) and \
        np.array_equal(np.asarray(A.indices, np.int64), np.asarray(B.indices, np.int64))


def field_loads(dim, coord, right):
    """Loads that vary over the boundary (the "el_*_field_load" fixtures):
    [(nodes, values, unknowns)] of add_surfLoad -- a function of position on
    the x = L face / edge and, in 2D, an array of one value per node."""
    if dim == 2:
        ramp = lambda x, y, z: -800 / 13**2 * (1.0 + y / 13.0)  # noqa: E731
        per_node = 5.0 * (1.0 + np.arange(right.size, dtype=float) / right.size)
        return [(right, [ramp], ["y"]), (right, [per_node], ["x"])]
    ramp3 = lambda x, y, z: -1.0 * (1.0 + y / 10.0 + 0.5 * z / 10.0)  # noqa: E731
    return [(right, [ramp3], ["z"])]
