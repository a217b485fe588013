"""Mesh containers and structured mesh generators.

The reference builds meshes through gmsh (``EasyFEA/FEM/_mesher.py``) and stores
them as ``Mesh`` objects holding one ``_GroupElem`` per element type
(``EasyFEA/FEM/_mesh.py:46-91``, ``EasyFEA/FEM/_group_elem.py:2225-2355``).  gmsh
is not part of this library: meshes are given as ``coord`` / ``connect`` arrays,
or produced by the organised (structured) generators below, which reproduce the
node and element orderings of the reference's organised meshes:

* QUAD4 / QUAD9 / TRI3 rectangles: node id ``j*(nx+1)+i``; counter-clockwise
  elements; SEG2 boundary groups on the four edges.
* HEXA8 boxes: node id ``(k*(ny+1)+j)*(nx+1)+i``; local node order of
  ``EasyFEA/FEM/Elems/_hexa.py:14-60``; QUAD4 boundary faces on the six faces.
* TETRA4 boxes (six tetrahedra per cell), the quadratic TRI6 / QUAD8 /
  TETRA10 meshes (mid-edge nodes added to the linear ones), HEXA20 / HEXA27
  and PRISM15 / PRISM18 boxes on the half-spacing node grid, PRISM6 boxes and
  TRI10 / TRI15 rectangles; every element in the local node order of
  ``EasyFEA/FEM/Elems``.  ``Mesh_Rect`` / ``Mesh_Box`` pick the generator of
  an element type.

Everything here is host-side numpy (set-up work done once per mesh); device
copies are made by the simulations that use the mesh.
"""

from __future__ import annotations

from enum import Enum
from typing import Callable, Optional

import numpy as np


class ElemType(str, Enum):
    """Element types handled by the GPU path (names of ``EasyFEA/FEM/_utils.py:9-34``)."""

    SEG2 = "SEG2"
    TRI3 = "TRI3"
    QUAD4 = "QUAD4"
    QUAD9 = "QUAD9"
    HEXA8 = "HEXA8"
    TETRA4 = "TETRA4"
    SEG3 = "SEG3"
    TRI6 = "TRI6"
    QUAD8 = "QUAD8"
    TETRA10 = "TETRA10"
    HEXA20 = "HEXA20"
    HEXA27 = "HEXA27"
    PRISM6 = "PRISM6"
    PRISM15 = "PRISM15"
    PRISM18 = "PRISM18"
    TRI10 = "TRI10"
    TRI15 = "TRI15"
    SEG4 = "SEG4"
    SEG5 = "SEG5"


class MatrixType(str, Enum):
    """Quadrature families (``EasyFEA/FEM/_utils.py:79-88``)."""

    rigi = "rigi"
    mass = "mass"


# (nPe, topological dim, C-ABI element code)
ELEM_INFO = {
    ElemType.SEG2: (2, 1, 0),
    ElemType.TRI3: (3, 2, 1),
    ElemType.QUAD4: (4, 2, 2),
    ElemType.QUAD9: (9, 2, 3),
    ElemType.HEXA8: (8, 3, 4),
    ElemType.TETRA4: (4, 3, 5),
    ElemType.TRI6: (6, 2, 6),
    ElemType.QUAD8: (8, 2, 7),
    ElemType.TETRA10: (10, 3, 8),
    ElemType.SEG3: (3, 1, 9),
    ElemType.HEXA20: (20, 3, 10),
    ElemType.HEXA27: (27, 3, 11),
    ElemType.PRISM6: (6, 3, 12),
    ElemType.PRISM15: (15, 3, 13),
    ElemType.PRISM18: (18, 3, 14),
    ElemType.TRI10: (10, 2, 15),
    ElemType.TRI15: (15, 2, 16),
    ElemType.SEG4: (4, 1, 17),
    ElemType.SEG5: (5, 1, 18),
}

# Gauss points per (element, matrixType), as chosen by
# EasyFEA/FEM/_gauss.py:364-480 (TRI3 rigi 1 / mass 3, QUAD4 4, QUAD9 9,
# HEXA8 8, SEG2 rigi 1 / mass 2).
NPG = {
    (ElemType.SEG2, MatrixType.rigi): 1,
    (ElemType.SEG2, MatrixType.mass): 2,
    (ElemType.TRI3, MatrixType.rigi): 1,
    (ElemType.TRI3, MatrixType.mass): 3,
    (ElemType.QUAD4, MatrixType.rigi): 4,
    (ElemType.QUAD4, MatrixType.mass): 4,
    (ElemType.QUAD9, MatrixType.rigi): 9,
    (ElemType.QUAD9, MatrixType.mass): 9,
    (ElemType.HEXA8, MatrixType.rigi): 8,
    (ElemType.HEXA8, MatrixType.mass): 8,
    (ElemType.TETRA4, MatrixType.rigi): 1,
    (ElemType.TETRA4, MatrixType.mass): 4,
    (ElemType.SEG3, MatrixType.rigi): 1,
    (ElemType.SEG3, MatrixType.mass): 3,
    (ElemType.TRI6, MatrixType.rigi): 3,
    (ElemType.TRI6, MatrixType.mass): 6,
    (ElemType.QUAD8, MatrixType.rigi): 4,
    (ElemType.QUAD8, MatrixType.mass): 9,
    (ElemType.TETRA10, MatrixType.rigi): 4,
    (ElemType.TETRA10, MatrixType.mass): 4,
    (ElemType.HEXA20, MatrixType.rigi): 27,
    (ElemType.HEXA20, MatrixType.mass): 27,
    (ElemType.HEXA27, MatrixType.rigi): 27,
    (ElemType.HEXA27, MatrixType.mass): 27,
    (ElemType.PRISM6, MatrixType.rigi): 6,
    (ElemType.PRISM6, MatrixType.mass): 6,
    (ElemType.PRISM15, MatrixType.rigi): 6,
    (ElemType.PRISM15, MatrixType.mass): 6,
    (ElemType.PRISM18, MatrixType.rigi): 21,
    (ElemType.PRISM18, MatrixType.mass): 21,
    (ElemType.TRI10, MatrixType.rigi): 6,
    (ElemType.TRI10, MatrixType.mass): 6,
    (ElemType.TRI15, MatrixType.rigi): 12,
    (ElemType.TRI15, MatrixType.mass): 12,
    (ElemType.SEG4, MatrixType.rigi): 2,
    (ElemType.SEG4, MatrixType.mass): 4,
    (ElemType.SEG5, MatrixType.rigi): 4,
    (ElemType.SEG5, MatrixType.mass): 5,
}


class GroupElem:
    """One element group: ``connect`` (Ne, nPe) into the shared ``coord`` (Nn, 3).

    Mirrors the data half of ``_GroupElem`` (``EasyFEA/FEM/_group_elem.py``);
    the Gauss-point arithmetic lives in the CUDA kernels.
    """

    def __init__(self, elemType: ElemType, connect: np.ndarray, coord: np.ndarray):
        elemType = ElemType(elemType)
        nPe, dim, code = ELEM_INFO[elemType]
        connect = np.ascontiguousarray(connect, dtype=np.int64)
        assert connect.ndim == 2 and connect.shape[1] == nPe, (
            f"{elemType} connect must be (Ne, {nPe})"
        )
        self.elemType = elemType
        self.nPe = nPe
        self.dim = dim
        self.code = code
        self.__connect = connect
        self.__connect.setflags(write=False)
        self.__coord = coord

    @property
    def connect(self) -> np.ndarray:
        return self.__connect

    @property
    def coord(self) -> np.ndarray:
        return self.__coord

    @property
    def Ne(self) -> int:
        return self.__connect.shape[0]

    @property
    def nodes(self) -> np.ndarray:
        return np.unique(self.__connect)

    def Get_assembly_e(self, dof_n: int) -> np.ndarray:
        """Element DOF map ``node*dof_n + d`` (``EasyFEA/FEM/_group_elem.py:346-380``)."""
        Ne, nPe = self.__connect.shape
        assembly = np.empty((Ne, nPe * dof_n), dtype=np.int64)
        for d in range(dof_n):
            assembly[:, d::dof_n] = self.__connect * dof_n + d
        return assembly

    def Get_Elements_Nodes(self, nodes: np.ndarray, exclusively: bool = True) -> np.ndarray:
        """Elements using the given nodes (``EasyFEA/FEM/_group_elem.py:1500-1537``).

        With ``exclusively`` only elements whose every node is in ``nodes``.
        """
        mark = np.zeros(self.__coord.shape[0], dtype=bool)
        nodes = np.asarray(nodes, dtype=np.int64)
        mark[nodes[nodes < mark.size]] = True
        hit = mark[self.__connect]
        sel = hit.all(axis=1) if exclusively else hit.any(axis=1)
        return np.nonzero(sel)[0]


class Mesh:
    """A set of element groups sharing one coordinate array (``EasyFEA/FEM/_mesh.py:46-191``)."""

    def __init__(self, dict_groupElem: dict):
        assert len(dict_groupElem) > 0, "dict_groupElem is empty."
        coords = {id(g.coord) for g in dict_groupElem.values()}
        assert len(coords) == 1, "All element groups must share the same coordinates."
        self.__dict = dict(dict_groupElem)
        first = next(iter(self.__dict.values()))
        self.__coord = first.coord
        self.__dim = max(g.dim for g in self.__dict.values())
        used = np.zeros(self.Nn, dtype=bool)
        for g in self.__dict.values():
            used[g.connect.ravel()] = True
        self.__orphanNodes = np.nonzero(~used)[0]
        self.__version = 0

    @property
    def dict_groupElem(self) -> dict:
        return self.__dict

    @property
    def coord(self) -> np.ndarray:
        return self.__coord

    @property
    def coordGlob(self) -> np.ndarray:
        return self.__coord

    @property
    def Nn(self) -> int:
        return self.__coord.shape[0]

    @property
    def dim(self) -> int:
        return self.__dim

    @property
    def inDim(self) -> int:
        """Embedding dimension deduced from the coordinates (``EasyFEA/FEM/_group_elem.py:155-175``)."""
        if self.__dim == 3:
            return 3
        _, y, z = np.abs(self.__coord.T)
        if z.size and np.max(z) > 0:
            return 3
        if y.size and np.max(y) > 0:
            return 2
        return 1

    @property
    def orphanNodes(self) -> np.ndarray:
        return self.__orphanNodes

    @property
    def groupElem(self) -> GroupElem:
        """The main-dimension element group."""
        return self.Get_list_groupElem(self.__dim)[0]

    @property
    def elemType(self) -> ElemType:
        return self.groupElem.elemType

    @property
    def Ne(self) -> int:
        return self.groupElem.Ne

    @property
    def connect(self) -> np.ndarray:
        return self.groupElem.connect

    def Get_list_groupElem(self, dim: Optional[int] = None) -> list:
        if dim is None:
            dim = self.__dim
        out = [g for g in self.__dict.values() if g.dim == dim]
        out.reverse()
        return out

    def Nodes_Conditions(self, func: Callable) -> np.ndarray:
        """Nodes of the main group whose coordinates satisfy ``func(x, y, z)``
        (``EasyFEA/FEM/_mesh.py:619-644``)."""
        nodes = self.groupElem.nodes
        x, y, z = self.__coord[nodes].T
        return nodes[np.asarray(func(x, y, z), dtype=bool)]

    def __str__(self) -> str:
        return f"elemType: {self.elemType.value}\nNe: {self.Ne}\nNn: {self.Nn}"


# ---------------------------------------------------------------------------
# organised mesh generators
# ---------------------------------------------------------------------------


def _grid2d(L: float, h: float, nx: int, ny: int, x0: float = 0.0, y0: float = 0.0):
    xs = x0 + np.linspace(0.0, L, nx + 1)
    ys = y0 + np.linspace(0.0, h, ny + 1)
    X, Y = np.meshgrid(xs, ys)  # (ny+1, nx+1), node id j*(nx+1)+i
    coord = np.zeros(((nx + 1) * (ny + 1), 3))
    coord[:, 0] = X.ravel()
    coord[:, 1] = Y.ravel()
    return coord


def _edges2d(nx: int, ny: int, stride: int = 1):
    """SEG2 edges of an (nx*stride)x(ny*stride) node grid boundary, counter-clockwise."""
    NX = nx * stride
    nid = lambda i, j: j * (NX + 1) + i  # noqa: E731
    segs = []
    for i in range(NX):
        segs.append((nid(i, 0), nid(i + 1, 0)))
    for j in range(ny * stride):
        segs.append((nid(NX, j), nid(NX, j + 1)))
    for i in range(NX, 0, -1):
        segs.append((nid(i, ny * stride), nid(i - 1, ny * stride)))
    for j in range(ny * stride, 0, -1):
        segs.append((nid(0, j), nid(0, j - 1)))
    return np.asarray(segs, dtype=np.int64)


def Mesh_Quad4_Rect(L: float, h: float, nx: int, ny: int) -> Mesh:
    """Organised QUAD4 mesh of [0,L]x[0,h] with SEG2 boundary edges."""
    coord = _grid2d(L, h, nx, ny)
    i, j = np.meshgrid(np.arange(nx), np.arange(ny))
    i = i.ravel()
    j = j.ravel()
    n0 = j * (nx + 1) + i
    connect = np.stack([n0, n0 + 1, n0 + nx + 2, n0 + nx + 1], axis=1)
    groups = {
        ElemType.SEG2: GroupElem(ElemType.SEG2, _edges2d(nx, ny), coord),
        ElemType.QUAD4: GroupElem(ElemType.QUAD4, connect, coord),
    }
    return Mesh(groups)


def Mesh_Tri3_Rect(L: float, h: float, nx: int, ny: int) -> Mesh:
    """Organised TRI3 mesh: each square split along its (i,j)-(i+1,j+1) diagonal."""
    coord = _grid2d(L, h, nx, ny)
    i, j = np.meshgrid(np.arange(nx), np.arange(ny))
    n00 = (j * (nx + 1) + i).ravel()
    n10 = n00 + 1
    n11 = n00 + nx + 2
    n01 = n00 + nx + 1
    t1 = np.stack([n00, n10, n11], axis=1)
    t2 = np.stack([n00, n11, n01], axis=1)
    connect = np.stack([t1, t2], axis=1).reshape(-1, 3)
    groups = {
        ElemType.SEG2: GroupElem(ElemType.SEG2, _edges2d(nx, ny), coord),
        ElemType.TRI3: GroupElem(ElemType.TRI3, connect, coord),
    }
    return Mesh(groups)


def Mesh_Quad9_Rect(L: float, h: float, nx: int, ny: int) -> Mesh:
    """Organised QUAD9 mesh (corner, mid-edge, centre nodes) on a (2nx+1)x(2ny+1) grid."""
    NX, NY = 2 * nx, 2 * ny
    coord = _grid2d(L, h, NX, NY)
    nid = lambda i, j: j * (NX + 1) + i  # noqa: E731
    I, J = np.meshgrid(np.arange(nx), np.arange(ny))
    I = 2 * I.ravel()
    J = 2 * J.ravel()
    connect = np.stack(
        [
            nid(I, J), nid(I + 2, J), nid(I + 2, J + 2), nid(I, J + 2),
            nid(I + 1, J), nid(I + 2, J + 1), nid(I + 1, J + 2), nid(I, J + 1),
            nid(I + 1, J + 1),
        ],
        axis=1,
    )
    # boundary: SEG2 pieces between consecutive boundary nodes
    groups = {
        ElemType.SEG2: GroupElem(ElemType.SEG2, _edges2d(NX, NY), coord),
        ElemType.QUAD9: GroupElem(ElemType.QUAD9, connect, coord),
    }
    return Mesh(groups)


def Mesh_Hexa8_Box(Lx: float, Ly: float, Lz: float, nx: int, ny: int, nz: int) -> Mesh:
    """Organised HEXA8 mesh of [0,Lx]x[0,Ly]x[0,Lz] with QUAD4 boundary faces."""
    xs = np.linspace(0.0, Lx, nx + 1)
    ys = np.linspace(0.0, Ly, ny + 1)
    zs = np.linspace(0.0, Lz, nz + 1)
    Z, Y, X = np.meshgrid(zs, ys, xs, indexing="ij")
    coord = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)
    nid = lambda i, j, k: (k * (ny + 1) + j) * (nx + 1) + i  # noqa: E731
    K, J, I = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    I, J, K = I.ravel(), J.ravel(), K.ravel()
    connect = np.stack(
        [
            nid(I, J, K), nid(I + 1, J, K), nid(I + 1, J + 1, K), nid(I, J + 1, K),
            nid(I, J, K + 1), nid(I + 1, J, K + 1), nid(I + 1, J + 1, K + 1), nid(I, J + 1, K + 1),
        ],
        axis=1,
    )
    faces = []
    # x = 0 and x = Lx
    b, a = np.meshgrid(np.arange(nz), np.arange(ny), indexing="ij")
    a, b = a.ravel(), b.ravel()
    for i in (0, nx):
        faces.append(np.stack([nid(i, a, b), nid(i, a + 1, b), nid(i, a + 1, b + 1), nid(i, a, b + 1)], 1))
    # y = 0 and y = Ly
    b, a = np.meshgrid(np.arange(nz), np.arange(nx), indexing="ij")
    a, b = a.ravel(), b.ravel()
    for j in (0, ny):
        faces.append(np.stack([nid(a, j, b), nid(a + 1, j, b), nid(a + 1, j, b + 1), nid(a, j, b + 1)], 1))
    # z = 0 and z = Lz
    b, a = np.meshgrid(np.arange(ny), np.arange(nx), indexing="ij")
    a, b = a.ravel(), b.ravel()
    for k in (0, nz):
        faces.append(np.stack([nid(a, b, k), nid(a + 1, b, k), nid(a + 1, b + 1, k), nid(a, b + 1, k)], 1))
    faces = np.concatenate(faces, 0)
    groups = {
        ElemType.QUAD4: GroupElem(ElemType.QUAD4, faces, coord),
        ElemType.HEXA8: GroupElem(ElemType.HEXA8, connect, coord),
    }
    return Mesh(groups)


def Mesh_Tetra4_Box(Lx: float, Ly: float, Lz: float, nx: int, ny: int, nz: int) -> Mesh:
    """Organised TETRA4 mesh of [0,Lx]x[0,Ly]x[0,Lz]: every cell of the
    HEXA8 grid (same node numbering) split into the six tetrahedra of its
    main diagonal (conforming: each cell face is cut along its diagonal from
    the corner of lowest to highest coordinates); the TRI3 boundary faces
    are the tetrahedra's faces that belong to one tetrahedron only."""
    xs = np.linspace(0.0, Lx, nx + 1)
    ys = np.linspace(0.0, Ly, ny + 1)
    zs = np.linspace(0.0, Lz, nz + 1)
    Z, Y, X = np.meshgrid(zs, ys, xs, indexing="ij")
    coord = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)
    nid = lambda i, j, k: (k * (ny + 1) + j) * (nx + 1) + i  # noqa: E731
    K, J, I = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    I, J, K = I.ravel(), J.ravel(), K.ravel()
    corner = lambda a, b, c: nid(I + a, J + b, K + c)  # noqa: E731
    tets = []
    # a path 000 -> 111 through the cell's corners for each order of the axes
    for order in ((0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0)):
        p = [0, 0, 0]
        path = [corner(*p)]
        for ax in order:
            p[ax] = 1
            path.append(corner(*p))
        tets.append(np.stack(path, axis=1))
    connect = np.concatenate(tets, 0)
    faces = np.concatenate([connect[:, [0, 2, 1]], connect[:, [0, 3, 2]], connect[:, [0, 1, 3]],
                            connect[:, [1, 2, 3]]], 0)
    key = np.sort(faces, axis=1)
    _, inv, counts = np.unique(key, axis=0, return_inverse=True, return_counts=True)
    boundary = faces[counts[inv.ravel()] == 1]
    groups = {
        ElemType.TRI3: GroupElem(ElemType.TRI3, boundary, coord),
        ElemType.TETRA4: GroupElem(ElemType.TETRA4, connect, coord),
    }
    return Mesh(groups)


def _quadratic(m: Mesh, elem: ElemType, edges, belem: ElemType, bedges) -> Mesh:
    """The quadratic version of a linear mesh: one node at the middle of
    every edge, appended after the vertices; ``edges`` / ``bedges`` list the
    local vertex pairs whose middle nodes follow the vertices, in the
    reference's node order (EasyFEA/FEM/Elems: TRI6 01 12 20; QUAD8 01 12 23
    30; TETRA10 01 12 20 03 23 13; SEG3 01; boundary TRI6 as TRI6)."""
    coord = m.coord
    lin = m.groupElem.connect
    blin = m.Get_list_groupElem(m.dim - 1)[0].connect
    pairs = np.concatenate([np.sort(lin[:, list(e)], axis=1) for e in edges] +
                           [np.sort(blin[:, list(e)], axis=1) for e in bedges])
    uniq, inv = np.unique(pairs, axis=0, return_inverse=True)
    inv = inv.ravel()
    Nn = len(coord)
    mids = (coord[uniq[:, 0]] + coord[uniq[:, 1]]) / 2
    coord2 = np.concatenate([coord, mids])
    n_e = len(lin) * len(edges)
    emid = (Nn + inv[:n_e]).reshape(len(edges), -1).T
    bmid = (Nn + inv[n_e:]).reshape(len(bedges), -1).T
    groups = {
        belem: GroupElem(belem, np.concatenate([blin, bmid], axis=1), coord2),
        elem: GroupElem(elem, np.concatenate([lin, emid], axis=1), coord2),
    }
    return Mesh(groups)


def Mesh_Tri6_Rect(L: float, h: float, nx: int, ny: int) -> Mesh:
    """Organised TRI6 mesh (the TRI3 mesh with mid-edge nodes) with SEG3 boundary edges."""
    return _quadratic(Mesh_Tri3_Rect(L, h, nx, ny), ElemType.TRI6, [(0, 1), (1, 2), (2, 0)], ElemType.SEG3, [(0, 1)])


def Mesh_Quad8_Rect(L: float, h: float, nx: int, ny: int) -> Mesh:
    """Organised QUAD8 mesh (the QUAD4 mesh with mid-edge nodes) with SEG3 boundary edges."""
    return _quadratic(Mesh_Quad4_Rect(L, h, nx, ny), ElemType.QUAD8, [(0, 1), (1, 2), (2, 3), (3, 0)], ElemType.SEG3,
                      [(0, 1)])


def Mesh_Tetra10_Box(Lx: float, Ly: float, Lz: float, nx: int, ny: int, nz: int) -> Mesh:
    """Organised TETRA10 mesh (the TETRA4 mesh with mid-edge nodes) with TRI6 boundary faces."""
    return _quadratic(Mesh_Tetra4_Box(Lx, Ly, Lz, nx, ny, nz), ElemType.TETRA10,
                      [(0, 1), (1, 2), (2, 0), (0, 3), (2, 3), (1, 3)], ElemType.TRI6, [(0, 1), (1, 2), (2, 0)])


# local coordinates of the HEXA27 nodes in the reference's order (corners,
# edge middles, face centres, centre; EasyFEA/FEM/Elems/_hexa.py); HEXA20
# takes the first 20
_HEXA_LOCAL = np.array([
    [-1, -1, -1], [1, -1, -1], [1, 1, -1], [-1, 1, -1], [-1, -1, 1], [1, -1, 1], [1, 1, 1], [-1, 1, 1],
    [0, -1, -1], [-1, 0, -1], [-1, -1, 0], [1, 0, -1], [1, -1, 0], [0, 1, -1], [1, 1, 0], [-1, 1, 0],
    [0, -1, 1], [-1, 0, 1], [1, 0, 1], [0, 1, 1], [0, 0, -1], [0, -1, 0], [-1, 0, 0], [1, 0, 0],
    [0, 1, 0], [0, 0, 1], [0, 0, 0]])


def _hexa_quadratic_box(Lx, Ly, Lz, nx, ny, nz, nPe: int) -> Mesh:
    """HEXA20 / HEXA27 box on the half-spacing node grid: element nodes at
    their local coordinates, faces as QUAD8 / QUAD9 (corners around the face,
    edge middles, centre), grid nodes no element uses dropped."""
    NX, NY, NZ = 2 * nx, 2 * ny, 2 * nz
    xs, ys, zs = np.linspace(0.0, Lx, NX + 1), np.linspace(0.0, Ly, NY + 1), np.linspace(0.0, Lz, NZ + 1)
    Z, Y, X = np.meshgrid(zs, ys, xs, indexing="ij")
    coord = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)
    nid = lambda i, j, k: (k * (NY + 1) + j) * (NX + 1) + i  # noqa: E731
    K, J, I = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    I, J, K = 2 * I.ravel() + 1, 2 * J.ravel() + 1, 2 * K.ravel() + 1  # cell centres on the grid
    loc = _HEXA_LOCAL[:nPe]
    connect = np.stack([nid(I + a, J + b, K + c) for a, b, c in loc], axis=1)
    # faces: on each side of the box, the face-local (u, v) grid of the cells there
    ring = [(-1, -1), (1, -1), (1, 1), (-1, 1)]
    mids = [(0, -1), (1, 0), (0, 1), (-1, 0)]
    uv = ring + mids + ([(0, 0)] if nPe == 27 else [])
    faces = []
    for axis, side, n_cells in ((0, -1, None), (0, 1, None), (1, -1, None), (1, 1, None), (2, -1, None), (2, 1, None)):
        sel = [(I, J, K)[axis] == (1 if side < 0 else (NX, NY, NZ)[axis] - 1)][0]
        cols = []
        for u, v in uv:
            off = [0, 0, 0]
            others = [a for a in range(3) if a != axis]
            off[axis] = side
            off[others[0]] = u
            off[others[1]] = v
            cols.append(nid(I[sel] + off[0], J[sel] + off[1], K[sel] + off[2]))
        faces.append(np.stack(cols, axis=1))
    faces = np.concatenate(faces)
    used = np.unique(np.concatenate([connect.ravel(), faces.ravel()]))
    new = -np.ones(len(coord), dtype=np.int64)
    new[used] = np.arange(len(used))
    belem = ElemType.QUAD9 if nPe == 27 else ElemType.QUAD8
    elem = ElemType.HEXA27 if nPe == 27 else ElemType.HEXA20
    c = coord[used]
    return Mesh({belem: GroupElem(belem, new[faces], c), elem: GroupElem(elem, new[connect], c)})


def Mesh_Hexa20_Box(Lx: float, Ly: float, Lz: float, nx: int, ny: int, nz: int) -> Mesh:
    """Organised HEXA20 mesh of [0,Lx]x[0,Ly]x[0,Lz] with QUAD8 boundary faces."""
    return _hexa_quadratic_box(Lx, Ly, Lz, nx, ny, nz, 20)


def Mesh_Hexa27_Box(Lx: float, Ly: float, Lz: float, nx: int, ny: int, nz: int) -> Mesh:
    """Organised HEXA27 mesh of [0,Lx]x[0,Ly]x[0,Lz] with QUAD9 boundary faces."""
    return _hexa_quadratic_box(Lx, Ly, Lz, nx, ny, nz, 27)


# (i1, i2) = p (r, s) of the TRI10 / TRI15 nodes in the reference's order
# (EasyFEA/FEM/Elems/_tri.py Get_Local_Coords: corners, p - 1 nodes along
# each edge 01, 12, 20 in that direction, inner nodes)
_TRI_LAGRANGE = {
    3: [(0, 0), (3, 0), (0, 3), (1, 0), (2, 0), (2, 1), (1, 2), (0, 2), (0, 1), (1, 1)],
    4: [(0, 0), (4, 0), (0, 4), (1, 0), (2, 0), (3, 0), (3, 1), (2, 2), (1, 3), (0, 3), (0, 2), (0, 1),
        (1, 1), (2, 1), (1, 2)],
}


def _boundary_cells2d(nx: int, ny: int):
    """The rectangle's boundary cell edges, counter-clockwise, as pairs of
    coarse grid points ((i, j), (i', j'))."""
    e = [((i, 0), (i + 1, 0)) for i in range(nx)]
    e += [((nx, j), (nx, j + 1)) for j in range(ny)]
    e += [((i, ny), (i - 1, ny)) for i in range(nx, 0, -1)]
    e += [((0, j), (0, j - 1)) for j in range(ny, 0, -1)]
    return e


def _tri_lagrange_rect(L: float, h: float, nx: int, ny: int, p: int) -> Mesh:
    """TRI10 (p = 3) / TRI15 (p = 4) rectangle: the cells of Mesh_Tri3_Rect
    (split along their (i,j)-(i+1,j+1) diagonal) on a node grid of spacing
    1/p of a cell, node id J*(p nx+1)+I; boundary edges SEG4 / SEG5 (the two
    ends, then the inner nodes from the first end, counter-clockwise)."""
    NX, NY = p * nx, p * ny
    coord = _grid2d(L, h, NX, NY)
    nid = lambda i, j: j * (NX + 1) + i  # noqa: E731
    J, I = np.meshgrid(np.arange(ny), np.arange(nx), indexing="ij")
    I, J = p * I.ravel(), p * J.ravel()
    tris = []
    for P0, P1, P2 in (((0, 0), (1, 0), (1, 1)), ((0, 0), (1, 1), (0, 1))):
        cols = []
        for i1, i2 in _TRI_LAGRANGE[p]:
            dx = p * P0[0] + i1 * (P1[0] - P0[0]) + i2 * (P2[0] - P0[0])
            dy = p * P0[1] + i1 * (P1[1] - P0[1]) + i2 * (P2[1] - P0[1])
            cols.append(nid(I + dx, J + dy))
        tris.append(np.stack(cols, axis=1))
    connect = np.stack(tris, axis=1).reshape(-1, len(_TRI_LAGRANGE[p]))
    segs = []
    for (a, b) in _boundary_cells2d(nx, ny):
        ia, ja, ib, jb = p * a[0], p * a[1], p * b[0], p * b[1]
        di, dj = (ib - ia) // p, (jb - ja) // p
        segs.append([nid(ia, ja), nid(ib, jb)] + [nid(ia + k * di, ja + k * dj) for k in range(1, p)])
    belem = ElemType.SEG4 if p == 3 else ElemType.SEG5
    elem = ElemType.TRI10 if p == 3 else ElemType.TRI15
    return Mesh({belem: GroupElem(belem, np.asarray(segs, dtype=np.int64), coord),
                 elem: GroupElem(elem, connect, coord)})


def Mesh_Tri10_Rect(L: float, h: float, nx: int, ny: int) -> Mesh:
    """Organised TRI10 mesh (cubic triangles) with SEG4 boundary edges."""
    return _tri_lagrange_rect(L, h, nx, ny, 3)


def Mesh_Tri15_Rect(L: float, h: float, nx: int, ny: int) -> Mesh:
    """Organised TRI15 mesh (quartic triangles) with SEG5 boundary edges."""
    return _tri_lagrange_rect(L, h, nx, ny, 4)


# local coordinates (2 r, 2 s, t) of the PRISM18 nodes in the reference's order
# (EasyFEA/FEM/Elems/_prism.py Get_Local_Coords: the corners of the t = -1
# and t = 1 triangles, the edge middles, the quadrangular faces' centres);
# PRISM6 takes the first 6, PRISM15 the first 15
_PRISM_LOCAL = np.array([
    [0, 0, -1], [2, 0, -1], [0, 2, -1], [0, 0, 1], [2, 0, 1], [0, 2, 1],
    [1, 0, -1], [0, 1, -1], [0, 0, 0], [1, 1, -1], [2, 0, 0], [0, 2, 0],
    [1, 0, 1], [0, 1, 1], [1, 1, 1], [1, 0, 0], [0, 1, 0], [1, 1, 0]])


def _prism_box(Lx, Ly, Lz, nx, ny, nz, nPe: int) -> Mesh:
    """Prisms of [0,Lx]x[0,Ly]x[0,Lz]: the triangles of Mesh_Tri3_Rect's
    cells in x-y extruded over nz layers along z.  The quadratic prisms use
    the half-spacing node grid (grid nodes no element uses are dropped).
    Boundary faces: the triangles at z = 0 and z = Lz (TRI3 / TRI6: corners,
    then the middles of edges 01, 12, 20) and the quadrangles of the four
    sides (QUAD4 / QUAD8 / QUAD9: corners around the face, edge middles,
    centre)."""
    q = 1 if nPe == 6 else 2
    NX, NY, NZ = q * nx, q * ny, q * nz
    xs, ys, zs = np.linspace(0.0, Lx, NX + 1), np.linspace(0.0, Ly, NY + 1), np.linspace(0.0, Lz, NZ + 1)
    Z, Y, X = np.meshgrid(zs, ys, xs, indexing="ij")
    coord = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)
    nid = lambda i, j, k: (k * (NY + 1) + j) * (NX + 1) + i  # noqa: E731
    K, J, I = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    K, J, I = K.ravel(), J.ravel(), I.ravel()
    loc = _PRISM_LOCAL[:nPe]
    prisms = []
    for P0, P1, P2 in (((0, 0), (1, 0), (1, 1)), ((0, 0), (1, 1), (0, 1))):
        cols = []
        for r2, s2, t in loc:
            # fine-grid offsets: q P0 + (q r) (P1 - P0) + (q s) (P2 - P0), layer q k + q (t + 1) / 2
            di = q * P0[0] + (q * r2 // 2) * (P1[0] - P0[0]) + (q * s2 // 2) * (P2[0] - P0[0])
            dj = q * P0[1] + (q * r2 // 2) * (P1[1] - P0[1]) + (q * s2 // 2) * (P2[1] - P0[1])
            cols.append(nid(q * I + di, q * J + dj, q * K + q * (t + 1) // 2))
        prisms.append(np.stack(cols, axis=1))
    connect = np.stack(prisms, axis=1).reshape(-1, nPe)
    # triangular faces: the bottom triangles of the first layer, the top ones of the last
    tri_bot = [0, 1, 2] if q == 1 else [0, 1, 2, 6, 9, 7]
    tri_top = [3, 4, 5] if q == 1 else [3, 4, 5, 12, 14, 13]
    first = np.repeat(K == 0, 2)
    last = np.repeat(K == nz - 1, 2)
    tris = np.concatenate([connect[first][:, tri_bot], connect[last][:, tri_top]])
    # quadrangular faces on the four sides, layer by layer
    quads = []
    for (a, b) in _boundary_cells2d(nx, ny):
        for k in range(nz):
            ia, ja, ib, jb = q * a[0], q * a[1], q * b[0], q * b[1]
            k0, k1 = q * k, q * (k + 1)
            row = [nid(ia, ja, k0), nid(ib, jb, k0), nid(ib, jb, k1), nid(ia, ja, k1)]
            if q == 2:
                im, jm, km = (ia + ib) // 2, (ja + jb) // 2, k0 + 1
                row += [nid(im, jm, k0), nid(ib, jb, km), nid(im, jm, k1), nid(ia, ja, km)]
                if nPe == 18:
                    row.append(nid(im, jm, km))
            quads.append(row)
    quads = np.asarray(quads, dtype=np.int64)
    used = np.unique(np.concatenate([connect.ravel(), tris.ravel(), quads.ravel()]))
    new = -np.ones(len(coord), dtype=np.int64)
    new[used] = np.arange(len(used))
    c = coord[used]
    elem = {6: ElemType.PRISM6, 15: ElemType.PRISM15, 18: ElemType.PRISM18}[nPe]
    qelem = {6: ElemType.QUAD4, 15: ElemType.QUAD8, 18: ElemType.QUAD9}[nPe]
    telem = ElemType.TRI3 if q == 1 else ElemType.TRI6
    return Mesh({qelem: GroupElem(qelem, new[quads], c), telem: GroupElem(telem, new[tris], c),
                 elem: GroupElem(elem, new[connect], c)})


def Mesh_Prism6_Box(Lx: float, Ly: float, Lz: float, nx: int, ny: int, nz: int) -> Mesh:
    """Organised PRISM6 mesh (triangles in x-y extruded along z) with QUAD4
    side faces and TRI3 end faces."""
    return _prism_box(Lx, Ly, Lz, nx, ny, nz, 6)


def Mesh_Prism15_Box(Lx: float, Ly: float, Lz: float, nx: int, ny: int, nz: int) -> Mesh:
    """Organised PRISM15 mesh with QUAD8 side faces and TRI6 end faces."""
    return _prism_box(Lx, Ly, Lz, nx, ny, nz, 15)


def Mesh_Prism18_Box(Lx: float, Ly: float, Lz: float, nx: int, ny: int, nz: int) -> Mesh:
    """Organised PRISM18 mesh with QUAD9 side faces and TRI6 end faces."""
    return _prism_box(Lx, Ly, Lz, nx, ny, nz, 18)


def Mesh_Rect(elemType: ElemType, L: float, h: float, nx: int, ny: int) -> Mesh:
    """Organised mesh of [0,L]x[0,h] with nx x ny cells of any 2D element type."""
    make = {ElemType.QUAD4: Mesh_Quad4_Rect, ElemType.TRI3: Mesh_Tri3_Rect, ElemType.QUAD9: Mesh_Quad9_Rect,
            ElemType.TRI6: Mesh_Tri6_Rect, ElemType.QUAD8: Mesh_Quad8_Rect, ElemType.TRI10: Mesh_Tri10_Rect,
            ElemType.TRI15: Mesh_Tri15_Rect}.get(ElemType(elemType))
    if make is None:
        raise NotImplementedError(elemType)
    return make(L, h, nx, ny)


def Mesh_Box(elemType: ElemType, Lx: float, Ly: float, Lz: float, nx: int, ny: int, nz: int) -> Mesh:
    """Organised mesh of [0,Lx]x[0,Ly]x[0,Lz] with nx x ny x nz cells of any 3D element type."""
    make = {ElemType.HEXA8: Mesh_Hexa8_Box, ElemType.HEXA20: Mesh_Hexa20_Box, ElemType.HEXA27: Mesh_Hexa27_Box,
            ElemType.TETRA4: Mesh_Tetra4_Box, ElemType.TETRA10: Mesh_Tetra10_Box, ElemType.PRISM6: Mesh_Prism6_Box,
            ElemType.PRISM15: Mesh_Prism15_Box, ElemType.PRISM18: Mesh_Prism18_Box}.get(ElemType(elemType))
    if make is None:
        raise NotImplementedError(elemType)
    return make(Lx, Ly, Lz, nx, ny, nz)
