"""Shared helpers of the parity tests."""

import numpy as np
import scipy.sparse as sp

from easyfea_gb300.mesh import ElemType, GroupElem, Mesh


def mesh_from_golden(g) -> Mesh:
    coord = np.asarray(g["coord"], dtype=float)
    groups = {
        ElemType(str(g["belem"])): GroupElem(ElemType(str(g["belem"])), g["bconnect"], coord),
        ElemType(str(g["elem"])): GroupElem(ElemType(str(g["elem"])), g["connect"], coord),
    }
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
