"""CPU oracle for the EasyFEA finite-element hot path -- TEST INFRASTRUCTURE ONLY.

A plain numpy/scipy restatement of the reference algorithms (matnoel/EasyFEA
v3.5.1), used by ``tests/``, ``__graft_entry__.smoke()`` and the CPU baseline
leg of ``bench.py`` as the checker.  Nothing in the product package imports it.

Parity is pinned: ``tests/golden/make_golden.py`` runs the reference itself (in
a container where its sources are importable) and stores its outputs under
``tests/golden/``; ``tests/test_oracle_golden.py`` checks this module against
them.

Each function cites the reference file:line it restates.  All arithmetic is
float64, as in the reference.
"""

from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as sla

SQRT2 = np.sqrt(2.0)

# ---------------------------------------------------------------------------
# quadrature (EasyFEA/FEM/_gauss.py)
# ---------------------------------------------------------------------------


def gauss(elem: str, matrixType: str):
    """Gauss points (nPg, dim) and weights (nPg,).

    EasyFEA/FEM/_gauss.py:364-480 (Gauss_factory); triangle table :55-108,
    quadrangle :111-138, hexahedron :201-..., SEG2 Gauss-Legendre :373-382.
    """
    if elem == "SEG2":
        n = 1 if matrixType == "rigi" else 2
        x, w = np.polynomial.legendre.leggauss(n)
        return x.reshape(-1, 1), w
    if elem == "TRI3":
        if matrixType == "rigi":
            xi, eta, w = [1 / 3], [1 / 3], [1 / 2]
        else:
            xi, eta, w = [1 / 6, 2 / 3, 1 / 6], [1 / 6, 1 / 6, 2 / 3], [1 / 6] * 3
        return np.array([xi, eta]).T, np.array(w)
    if elem == "QUAD4":
        a = 1 / np.sqrt(3)
        return np.array([[-a, a, a, -a], [-a, -a, a, a]]).T, np.ones(4)
    if elem == "QUAD9":
        a = 0.774596669241483
        xi = [-a, a, a, -a, 0.0, a, 0.0, -a, 0.0]
        eta = [-a, -a, a, a, -a, 0.0, a, 0.0, 0.0]
        w = [25 / 81] * 4 + [40 / 81] * 4 + [64 / 81]
        return np.array([xi, eta]).T, np.array(w)
    if elem == "HEXA8":
        a = 1 / np.sqrt(3)
        x = [-a, -a, -a, -a, a, a, a, a]
        y = [-a, -a, a, a, -a, -a, a, a]
        z = [-a, a, -a, a, -a, a, -a, a]
        return np.array([x, y, z]).T, np.ones(8)
    if elem == "SEG3":  # Gauss-Legendre, rigi 1 / mass 3 (_gauss.py:384-394)
        n = 1 if matrixType == "rigi" else 3
        x, w = np.polynomial.legendre.leggauss(n)
        return x.reshape(-1, 1), w
    if elem == "TRI6":  # rigi 3 / mass 6 (_gauss.py:64-79, :431-438)
        if matrixType == "rigi":
            return gauss("TRI3", "mass")
        a, b = 0.445948490915965, 0.091576213509771
        p1, p2 = 0.11169079483905, 0.0549758718227661
        xi = [b, 1 - 2 * b, b, a, a, 1 - 2 * a]
        eta = [b, b, 1 - 2 * b, 1 - 2 * a, a, a]
        return np.array([xi, eta]).T, np.array([p2, p2, p2, p1, p1, p1])
    if elem == "QUAD8":  # rigi 4 / mass 9 (_gauss.py:452-459)
        return gauss("QUAD4" if matrixType == "rigi" else "QUAD9", matrixType)
    if elem == "TETRA10":  # 4 points for both (_gauss.py:470-472)
        return gauss("TETRA4", "mass")
    if elem in ("HEXA20", "HEXA27"):  # 27 points for both (_gauss.py:216-261)
        a = np.sqrt(3 / 5)
        c1, c2 = 5 / 9, 8 / 9
        x = [-a] * 9 + [0.0] * 9 + [a] * 9
        y = [-a, -a, -a, 0.0, 0.0, 0.0, a, a, a] * 3
        z = [-a, 0.0, a] * 9
        c13, c23, c12, c22 = c1**3, c2**3, c1**2 * c2, c1 * c2**2
        by_zeros = {0: c13, 1: c12, 2: c22, 3: c23}
        w = [by_zeros[int(xi == 0) + int(yi == 0) + int(zi == 0)] for xi, yi, zi in zip(x, y, z)]
        return np.array([x, y, z]).T, np.array(w)
    if elem == "TETRA4":  # _gauss.py:142-163 (rigi 1 point, mass 4)
        if matrixType == "rigi":
            return np.array([[1 / 4, 1 / 4, 1 / 4]]), np.array([1 / 6])
        a = (5 - np.sqrt(5)) / 20
        b = (5 + 3 * np.sqrt(5)) / 20
        return np.array([[a, a, a, b], [a, a, b, a], [a, b, a, a]]).T, np.full(4, 1 / 24)
    if elem in ("SEG4", "SEG5"):  # Gauss-Legendre: SEG4 rigi 2 / mass 4, SEG5 rigi 4 / mass 5 (_gauss.py:396-419)
        n = {("SEG4", "rigi"): 2, ("SEG4", "mass"): 4, ("SEG5", "rigi"): 4, ("SEG5", "mass"): 5}[(elem, matrixType)]
        x, w = np.polynomial.legendre.leggauss(n)
        return x.reshape(-1, 1), w
    if elem == "TRI10":  # 6 points for both (_gauss.py:440-442)
        return gauss("TRI6", "mass")
    if elem == "TRI15":  # 12 points for both (_gauss.py:92-104, :444-446)
        a, b, c, d = 0.063089014491502, 0.249286745170910, 0.310352451033785, 0.053145049844816
        p1, p2, p3 = 0.025422453185103, 0.058393137863189, 0.041425537809187
        xi = [a, 1 - 2 * a, a, b, 1 - 2 * b, b, c, d, 1 - c - d, 1 - c - d, c, d]
        eta = [a, a, 1 - 2 * a, b, b, 1 - 2 * b, d, c, c, d, 1 - c - d, 1 - c - d]
        return np.array([xi, eta]).T, np.array([p1] * 3 + [p2] * 3 + [p3] * 6)
    if elem in ("PRISM6", "PRISM15"):  # 6 points (_gauss.py:275-282; x <- yc, y <- zc, z <- xc)
        a = 1 / np.sqrt(3)
        r = [0.5, 0.0, 0.5] * 2
        s_ = [0.5, 0.5, 0.0] * 2
        t = [-a] * 3 + [a] * 3
        return np.array([r, s_, t]).T, np.full(6, 1 / 6)
    if elem == "PRISM18":  # 21 points (_gauss.py:293-350): 7-point triangle x 3-point Gauss-Legendre
        al = np.sqrt(3 / 5)
        a, b = (6 + np.sqrt(15)) / 21, (6 - np.sqrt(15)) / 21
        cp, cm = (155 + np.sqrt(15)) / 2400, (155 - np.sqrt(15)) / 2400
        r = [1 / 3, a, 1 - 2 * a, a, b, 1 - 2 * b, b] * 3
        s_ = [1 / 3, a, a, 1 - 2 * a, b, b, 1 - 2 * b] * 3
        t = [-al] * 7 + [0.0] * 7 + [al] * 7
        wt = [9 / 80, cp, cp, cp, cm, cm, cm]
        w = [5 / 9 * x for x in wt] + [8 / 9 * x for x in wt] + [5 / 9 * x for x in wt]
        return np.array([r, s_, t]).T, np.array(w)
    raise NotImplementedError(elem)


# ---------------------------------------------------------------------------
# shape functions (EasyFEA/FEM/Elems/*.py)
# ---------------------------------------------------------------------------


def shape_N(elem: str, p: np.ndarray) -> np.ndarray:
    """N at one point -> (nPe,).  _seg.py:55-60, _tri.py:55-60, _quad.py:55-60,
    _quad.py:255-266 (QUAD9), _hexa.py:75-86."""
    if elem == "SEG2":
        (r,) = p
        return np.array([-(r - 1) / 2, (r + 1) / 2])
    if elem == "TRI3":
        r, s = p
        return np.array([-r - s + 1, r, s])
    if elem == "QUAD4":
        r, s = p
        return np.array([(r - 1) * (s - 1) / 4, -(r + 1) * (s - 1) / 4,
                         (r + 1) * (s + 1) / 4, -(r - 1) * (s + 1) / 4])
    if elem == "QUAD9":
        r, s = p
        return np.array([
            r * s * (r - 1) * (s - 1) / 4, r * s * (r + 1) * (s - 1) / 4,
            r * s * (r + 1) * (s + 1) / 4, r * s * (r - 1) * (s + 1) / 4,
            -s * (r - 1) * (r + 1) * (s - 1) / 2, -r * (r + 1) * (s - 1) * (s + 1) / 2,
            -s * (r - 1) * (r + 1) * (s + 1) / 2, -r * (r - 1) * (s - 1) * (s + 1) / 2,
            (r - 1) * (r + 1) * (s - 1) * (s + 1)])
    if elem == "HEXA8":
        r, s, t = p
        return np.array([
            -(r - 1) * (s - 1) * (t - 1) / 8, (r + 1) * (s - 1) * (t - 1) / 8,
            -(r + 1) * (s + 1) * (t - 1) / 8, (r - 1) * (s + 1) * (t - 1) / 8,
            (r - 1) * (s - 1) * (t + 1) / 8, -(r + 1) * (s - 1) * (t + 1) / 8,
            (r + 1) * (s + 1) * (t + 1) / 8, -(r - 1) * (s + 1) * (t + 1) / 8])
    if elem == "TETRA4":  # Elems/_tetra.py TETRA4._N
        r, s, t = p
        return np.array([-r - s - t + 1, r, s, t])
    if elem == "SEG3":  # Elems/_seg.py SEG3._N
        (r,) = p
        return np.array([r * (r - 1) / 2, r * (r + 1) / 2, -(r - 1) * (r + 1)])
    if elem in ("HEXA20", "HEXA27"):
        return _hexa_quadratic(elem, p)[0]
    if elem in LOCAL_NODES:
        return _interpolant(elem, p)[0]
    if elem == "TRI6":  # Elems/_tri.py TRI6._N
        r, s = p
        return np.array([(r + s - 1) * (2 * r + 2 * s - 1), r * (2 * r - 1), s * (2 * s - 1), -4 * r * (r + s - 1),
                         4 * r * s, -4 * s * (r + s - 1)])
    if elem == "QUAD8":  # Elems/_quad.py QUAD8._N
        r, s = p
        return np.array([-(r - 1) * (s - 1) * (r + s + 1) / 4, -(r + 1) * (s - 1) * (r - s - 1) / 4,
                         (r + 1) * (s + 1) * (r + s - 1) / 4, (r - 1) * (s + 1) * (r - s + 1) / 4,
                         (r - 1) * (r + 1) * (s - 1) / 2, -(r + 1) * (s - 1) * (s + 1) / 2,
                         -(r - 1) * (r + 1) * (s + 1) / 2, (r - 1) * (s - 1) * (s + 1) / 2])
    if elem == "TETRA10":  # Elems/_tetra.py TETRA10._N
        r, s, t = p
        return np.array([(r + s + t - 1) * (2 * r + 2 * s + 2 * t - 1), r * (2 * r - 1), s * (2 * s - 1),
                         t * (2 * t - 1), -4 * r * (r + s + t - 1), 4 * r * s, -4 * s * (r + s + t - 1),
                         -4 * t * (r + s + t - 1), 4 * s * t, 4 * r * t])
    raise NotImplementedError(elem)


def shape_dN(elem: str, p: np.ndarray) -> np.ndarray:
    """dN/dxi at one point -> (dim, nPe).  _seg.py:62-68, _tri.py:62-68,
    _quad.py:62-70, _quad.py:268-305 (QUAD9), _hexa.py:88-130."""
    if elem == "SEG2":
        return np.array([[-1 / 2, 1 / 2]])
    if elem == "TRI3":
        return np.array([[-1.0, 1.0, 0.0], [-1.0, 0.0, 1.0]])
    if elem == "QUAD4":
        r, s = p
        return np.array([[s / 4 - 1 / 4, 1 / 4 - s / 4, s / 4 + 1 / 4, -s / 4 - 1 / 4],
                         [r / 4 - 1 / 4, -r / 4 - 1 / 4, r / 4 + 1 / 4, 1 / 4 - r / 4]])
    if elem == "QUAD9":
        r, s = p
        dr = [
            r * s * (s - 1) / 4 + s * (r - 1) * (s - 1) / 4,
            r * s * (s - 1) / 4 + s * (r + 1) * (s - 1) / 4,
            r * s * (s + 1) / 4 + s * (r + 1) * (s + 1) / 4,
            r * s * (s + 1) / 4 + s * (r - 1) * (s + 1) / 4,
            -s * (r - 1) * (s - 1) / 2 - s * (r + 1) * (s - 1) / 2,
            -r * (s - 1) * (s + 1) / 2 - (r + 1) * (s - 1) * (s + 1) / 2,
            -s * (r - 1) * (s + 1) / 2 - s * (r + 1) * (s + 1) / 2,
            -r * (s - 1) * (s + 1) / 2 - (r - 1) * (s - 1) * (s + 1) / 2,
            (r - 1) * (s - 1) * (s + 1) + (r + 1) * (s - 1) * (s + 1),
        ]
        ds = [
            r * s * (r - 1) / 4 + r * (r - 1) * (s - 1) / 4,
            r * s * (r + 1) / 4 + r * (r + 1) * (s - 1) / 4,
            r * s * (r + 1) / 4 + r * (r + 1) * (s + 1) / 4,
            r * s * (r - 1) / 4 + r * (r - 1) * (s + 1) / 4,
            -s * (r - 1) * (r + 1) / 2 - (r - 1) * (r + 1) * (s - 1) / 2,
            -r * (r + 1) * (s - 1) / 2 - r * (r + 1) * (s + 1) / 2,
            -s * (r - 1) * (r + 1) / 2 - (r - 1) * (r + 1) * (s + 1) / 2,
            -r * (r - 1) * (s - 1) / 2 - r * (r - 1) * (s + 1) / 2,
            (r - 1) * (r + 1) * (s - 1) + (r - 1) * (r + 1) * (s + 1),
        ]
        return np.array([dr, ds])
    if elem == "HEXA8":
        r, s, t = p
        return np.array([
            [-(s - 1) * (t - 1) / 8, (s - 1) * (t - 1) / 8, -(s + 1) * (t - 1) / 8, (s + 1) * (t - 1) / 8,
             (s - 1) * (t + 1) / 8, -(s - 1) * (t + 1) / 8, (s + 1) * (t + 1) / 8, -(s + 1) * (t + 1) / 8],
            [-(r - 1) * (t - 1) / 8, (r + 1) * (t - 1) / 8, -(r + 1) * (t - 1) / 8, (r - 1) * (t - 1) / 8,
             (r - 1) * (t + 1) / 8, -(r + 1) * (t + 1) / 8, (r + 1) * (t + 1) / 8, -(r - 1) * (t + 1) / 8],
            [-(r - 1) * (s - 1) / 8, (r + 1) * (s - 1) / 8, -(r + 1) * (s + 1) / 8, (r - 1) * (s + 1) / 8,
             (r - 1) * (s - 1) / 8, -(r + 1) * (s - 1) / 8, (r + 1) * (s + 1) / 8, -(r - 1) * (s + 1) / 8],
        ])
    if elem == "TETRA4":  # Elems/_tetra.py TETRA4._dN
        return np.array([[-1.0, 1.0, 0.0, 0.0], [-1.0, 0.0, 1.0, 0.0], [-1.0, 0.0, 0.0, 1.0]])
    if elem == "SEG3":  # Elems/_seg.py SEG3._dN
        (r,) = p
        return np.array([[r - 1 / 2, r + 1 / 2, -2 * r]])
    if elem in ("HEXA20", "HEXA27"):
        return _hexa_quadratic(elem, p)[1]
    if elem in LOCAL_NODES:
        return _interpolant(elem, p)[1]
    if elem == "TRI6":  # Elems/_tri.py TRI6._dN
        r, s = p
        return np.array([[4 * r + 4 * s - 3, 4 * r - 1, 0.0, -8 * r - 4 * s + 4, 4 * s, -4 * s],
                         [4 * r + 4 * s - 3, 0.0, 4 * s - 1, -4 * r, 4 * r, -4 * r - 8 * s + 4]])
    if elem == "QUAD8":  # Elems/_quad.py QUAD8._dN
        r, s = p
        return np.array([
            [-(r - 1) * (s - 1) / 4 - (s - 1) * (r + s + 1) / 4, -(r + 1) * (s - 1) / 4 - (s - 1) * (r - s - 1) / 4,
             (r + 1) * (s + 1) / 4 + (s + 1) * (r + s - 1) / 4, (r - 1) * (s + 1) / 4 + (s + 1) * (r - s + 1) / 4,
             (r - 1) * (s - 1) / 2 + (r + 1) * (s - 1) / 2, -(s - 1) * (s + 1) / 2,
             -(r - 1) * (s + 1) / 2 - (r + 1) * (s + 1) / 2, (s - 1) * (s + 1) / 2],
            [-(r - 1) * (s - 1) / 4 - (r - 1) * (r + s + 1) / 4, (r + 1) * (s - 1) / 4 - (r + 1) * (r - s - 1) / 4,
             (r + 1) * (s + 1) / 4 + (r + 1) * (r + s - 1) / 4, -(r - 1) * (s + 1) / 4 + (r - 1) * (r - s + 1) / 4,
             (r - 1) * (r + 1) / 2, -(r + 1) * (s - 1) / 2 - (r + 1) * (s + 1) / 2, -(r - 1) * (r + 1) / 2,
             (r - 1) * (s - 1) / 2 + (r - 1) * (s + 1) / 2]])
    if elem == "TETRA10":  # Elems/_tetra.py TETRA10._dN
        r, s, t = p
        a = 4 * r + 4 * s + 4 * t - 3
        return np.array([
            [a, 4 * r - 1, 0, 0, -8 * r - 4 * s - 4 * t + 4, 4 * s, -4 * s, -4 * t, 0, 4 * t],
            [a, 0, 4 * s - 1, 0, -4 * r, 4 * r, -4 * r - 8 * s - 4 * t + 4, -4 * t, 4 * t, 0],
            [a, 0, 0, 4 * t - 1, -4 * r, 0, -4 * s, -4 * r - 4 * s - 8 * t + 4, 4 * s, 4 * r]], dtype=float)
    raise NotImplementedError(elem)


# local coordinates of the HEXA27 nodes in the reference's order
# (Elems/_hexa.py HEXA27.Get_Local_Coords); HEXA20 takes the first 20
HEXA_LOCAL = np.array([
    [-1, -1, -1], [1, -1, -1], [1, 1, -1], [-1, 1, -1], [-1, -1, 1], [1, -1, 1], [1, 1, 1], [-1, 1, 1],
    [0, -1, -1], [-1, 0, -1], [-1, -1, 0], [1, 0, -1], [1, -1, 0], [0, 1, -1], [1, 1, 0], [-1, 1, 0],
    [0, -1, 1], [-1, 0, 1], [1, 0, 1], [0, 1, 1], [0, 0, -1], [0, -1, 0], [-1, 0, 0], [1, 0, 0],
    [0, 1, 0], [0, 0, 1], [0, 0, 0]], dtype=float)


def _hexa_quadratic(elem, p):
    """N (nPe,) and dN (3, nPe) of HEXA20 (serendipity: corner
    (1+r ri)(1+s si)(1+t ti)(r ri+s si+t ti-2)/8, edge (1-r^2)(1+s si)(1+t ti)/4
    and permutations; Elems/_hexa.py HEXA20._N) or HEXA27 (products of the
    quadratic Lagrange polynomials; HEXA27._N)."""
    x = np.asarray(p, float)
    if elem == "HEXA27":
        def L(v, a):
            return 1 - v * v if a == 0 else v * (v + a) / 2

        def dL(v, a):
            return -2 * v if a == 0 else v + a / 2
        N = np.array([np.prod([L(x[k], c[k]) for k in range(3)]) for c in HEXA_LOCAL])
        dN = np.array([[np.prod([dL(x[k], c[k]) if k == d else L(x[k], c[k]) for k in range(3)]) for c in HEXA_LOCAL]
                       for d in range(3)])
        return N, dN
    N = np.zeros(20)
    dN = np.zeros((3, 20))
    for n, c in enumerate(HEXA_LOCAL[:20]):
        f = [1 + x[k] * c[k] for k in range(3)]
        if n < 8:
            q = x @ c - 2
            N[n] = f[0] * f[1] * f[2] * q / 8
            for d in range(3):
                e, g = (d + 1) % 3, (d + 2) % 3
                dN[d, n] = c[d] * f[e] * f[g] * (2 * x[d] * c[d] + x[e] * c[e] + x[g] * c[g] - 1) / 8
        else:
            z = int(np.where(c == 0)[0][0])
            f[z] = 1 - x[z] ** 2
            N[n] = f[0] * f[1] * f[2] / 4
            for d in range(3):
                e, g = (d + 1) % 3, (d + 2) % 3
                dN[d, n] = (-2 * x[d] if d == z else c[d]) * f[e] * f[g] / 4
    return N, dN


# Local coordinates of the nodes of the higher-order segments, triangles and
# prisms in the reference's order (EasyFEA/FEM/Elems/_seg.py, _tri.py,
# _prism.py Get_Local_Coords)
LOCAL_NODES = {
    "SEG4": [[-1], [1], [-1 / 3], [1 / 3]],
    "SEG5": [[-1], [1], [-1 / 2], [0], [1 / 2]],
    "TRI10": [[0, 0], [1, 0], [0, 1], [1 / 3, 0], [2 / 3, 0], [2 / 3, 1 / 3], [1 / 3, 2 / 3], [0, 2 / 3],
              [0, 1 / 3], [1 / 3, 1 / 3]],
    "TRI15": [[0, 0], [1, 0], [0, 1], [1 / 4, 0], [1 / 2, 0], [3 / 4, 0], [3 / 4, 1 / 4], [1 / 2, 1 / 2],
              [1 / 4, 3 / 4], [0, 3 / 4], [0, 1 / 2], [0, 1 / 4], [1 / 4, 1 / 4], [1 / 2, 1 / 4], [1 / 4, 1 / 2]],
    "PRISM18": [[0, 0, -1], [1, 0, -1], [0, 1, -1], [0, 0, 1], [1, 0, 1], [0, 1, 1], [0.5, 0, -1], [0, 0.5, -1],
                [0, 0, 0], [0.5, 0.5, -1], [1, 0, 0], [0, 1, 0], [0.5, 0, 1], [0, 0.5, 1], [0.5, 0.5, 1],
                [0.5, 0, 0], [0, 0.5, 0], [0.5, 0.5, 0]],
}
LOCAL_NODES["PRISM6"] = LOCAL_NODES["PRISM18"][:6]
LOCAL_NODES["PRISM15"] = LOCAL_NODES["PRISM18"][:15]


def _monomials(elem):
    """Exponent triples of the polynomial space each element interpolates in:
    complete degree p in 1D and on the triangle; on the prisms the triangle's
    degree-1 / degree-2 space times degree 1 / 2 in t, and for PRISM15 the
    serendipity space P2(r, s) x P1(t) + {t^2, r t^2, s t^2}."""
    p = {"SEG4": 3, "SEG5": 4, "TRI10": 3, "TRI15": 4}.get(elem)
    if elem.startswith("SEG"):
        return [(i, 0, 0) for i in range(p + 1)]
    if elem.startswith("TRI"):
        return [(i, j, 0) for i in range(p + 1) for j in range(p + 1 - i)]
    tri1 = [(0, 0), (1, 0), (0, 1)]
    tri2 = tri1 + [(2, 0), (1, 1), (0, 2)]
    if elem == "PRISM6":
        return [(i, j, k) for (i, j) in tri1 for k in (0, 1)]
    if elem == "PRISM18":
        return [(i, j, k) for (i, j) in tri2 for k in (0, 1, 2)]
    return [(i, j, k) for (i, j) in tri2 for k in (0, 1)] + [(i, j, 2) for (i, j) in tri1]


def _interpolant(elem, p):
    """N (nPe,) and dN (dim, nPe) at p: the Lagrange interpolants of the
    element's nodes in its polynomial space, N(x) = V^-T m(x) with V the
    monomials m evaluated at the nodes."""
    nodes = np.asarray(LOCAL_NODES[elem], float)
    dim = nodes.shape[1]
    mono = _monomials(elem)

    def m(x, d=None):
        x = np.concatenate([np.asarray(x, float), np.zeros(3 - dim)])
        out = []
        for e in mono:
            if d is None:
                out.append(np.prod([x[k] ** e[k] for k in range(3)]))
            elif e[d] == 0:
                out.append(0.0)
            else:
                out.append(e[d] * np.prod([x[k] ** (e[k] - (k == d)) for k in range(3)]))
        return np.array(out)
    V = np.array([m(x) for x in nodes])  # (nPe, nPe)
    Vt_inv = np.linalg.inv(V).T
    N = Vt_inv @ m(p)
    dN = np.array([Vt_inv @ m(p, d) for d in range(dim)])
    return N, dN


ELEM_DIM = {"SEG2": 1, "TRI3": 2, "QUAD4": 2, "QUAD9": 2, "HEXA8": 3, "TETRA4": 3, "SEG3": 1, "TRI6": 2,
            "QUAD8": 2, "TETRA10": 3, "HEXA20": 3, "HEXA27": 3, "SEG4": 1, "SEG5": 1, "TRI10": 2, "TRI15": 2,
            "PRISM6": 3, "PRISM15": 3, "PRISM18": 3}


def N_pg(elem, matrixType):
    """(nPg, nPe) -- _group_elem.py:990-1000 (Get_N_pg)."""
    xg, _ = gauss(elem, matrixType)
    return np.array([shape_N(elem, p) for p in xg])


def dN_pg(elem, matrixType):
    """(nPg, dim, nPe) -- _group_elem.py:1063-1081 (Get_dN_pg)."""
    xg, _ = gauss(elem, matrixType)
    return np.array([shape_dN(elem, p) for p in xg])


# ---------------------------------------------------------------------------
# element geometry (EasyFEA/FEM/_group_elem.py:833-915, _linalg.py:533-656)
# ---------------------------------------------------------------------------


def det(F):
    """Closed-form determinant, _linalg.py:533-573."""
    d = F.shape[-1]
    if d == 1:
        return F[..., 0, 0]
    if d == 2:
        return F[..., 0, 0] * F[..., 1, 1] - F[..., 1, 0] * F[..., 0, 1]
    a = F
    return (a[..., 0, 0] * (a[..., 1, 1] * a[..., 2, 2] - a[..., 2, 1] * a[..., 1, 2])
            - a[..., 0, 1] * (a[..., 1, 0] * a[..., 2, 2] - a[..., 2, 0] * a[..., 1, 2])
            + a[..., 0, 2] * (a[..., 1, 0] * a[..., 2, 1] - a[..., 2, 0] * a[..., 1, 1]))


def inv(F):
    """Adjugate inverse, _linalg.py:576-656."""
    d = F.shape[-1]
    D = det(F)
    if d == 1:
        return 1 / F
    adj = np.zeros_like(F)
    if d == 2:
        adj[..., 0, 0] = F[..., 1, 1]
        adj[..., 0, 1] = -F[..., 0, 1]
        adj[..., 1, 0] = -F[..., 1, 0]
        adj[..., 1, 1] = F[..., 0, 0]
        return adj / D[..., None, None]
    T = np.swapaxes(F, -1, -2)
    a = lambda i, j: T[..., i, j]  # noqa: E731
    adj[..., 0, 0] = a(1, 1) * a(2, 2) - a(2, 1) * a(1, 2)
    adj[..., 0, 1] = -(a(1, 0) * a(2, 2) - a(2, 0) * a(1, 2))
    adj[..., 0, 2] = a(1, 0) * a(2, 1) - a(2, 0) * a(1, 1)
    adj[..., 1, 0] = -(a(0, 1) * a(2, 2) - a(2, 1) * a(0, 2))
    adj[..., 1, 1] = a(0, 0) * a(2, 2) - a(2, 0) * a(0, 2)
    adj[..., 1, 2] = -(a(0, 0) * a(2, 1) - a(2, 0) * a(0, 1))
    adj[..., 2, 0] = a(0, 1) * a(1, 2) - a(1, 1) * a(0, 2)
    adj[..., 2, 1] = -(a(0, 0) * a(1, 2) - a(1, 0) * a(0, 2))
    adj[..., 2, 2] = a(0, 0) * a(1, 1) - a(1, 0) * a(0, 1)
    return adj / D[..., None, None]


class Geometry:
    """Per-(element, Gauss point) geometry of one group for one matrixType.

    F = dN_pg @ X_e (_group_elem.py:833-869), wJ = |det F| * w (:872-900),
    dN_e = inv(F) @ dN_pg (:903-915, :1084-1105).  Boundary groups (dim <
    embedding dim) use the element-local frame of _group_elem.py:404-500; for
    straight segments and flat faces |det F| equals the length / area scale
    computed here from the tangent vectors.
    """

    def __init__(self, elem, coord, connect, matrixType):
        self.elem = elem
        self.dim = ELEM_DIM[elem]
        xg, w = gauss(elem, matrixType)
        self.w = w
        self.N = N_pg(elem, matrixType)
        self.dN = dN_pg(elem, matrixType)
        X = coord[connect]  # (Ne, nPe, 3)
        if self.dim == coord_dim(coord) or self.dim == 3:
            Xd = X[:, :, : self.dim]
            F = np.einsum("pdn,enk->epdk", self.dN, Xd)
            self.F = F
            self.detJ = np.abs(det(F))
            self.invF = inv(F)
            self.dNx = np.einsum("epij,pjn->epin", self.invF, self.dN)
        else:
            # tangent vectors dx/dxi_k (Ne, nPg, dim, 3)
            T = np.einsum("pdn,enk->epdk", self.dN, X)
            if self.dim == 1:
                self.detJ = np.linalg.norm(T[:, :, 0, :], axis=-1)
            else:
                self.detJ = np.linalg.norm(np.cross(T[:, :, 0, :], T[:, :, 1, :]), axis=-1)
            self.dNx = None
        self.wJ = self.detJ * w[None, :]
        self.X = X


def coord_dim(coord):
    _, y, z = np.abs(coord.T)
    if z.size and z.max() > 0:
        return 3
    if y.size and y.max() > 0:
        return 2
    return 1


def B_e_pg(dNx):
    """Kelvin-Mandel strain-displacement operator, _group_elem.py:1242-1312."""
    Ne, nPg, dim, nPe = dNx.shape
    cM = 1 / np.sqrt(2)
    if dim == 2:
        B = np.zeros((Ne, nPg, 3, nPe * 2))
        dx, dy = dNx[:, :, 0], dNx[:, :, 1]
        B[:, :, 0, 0::2] = dx
        B[:, :, 1, 1::2] = dy
        B[:, :, 2, 0::2] = dy * cM
        B[:, :, 2, 1::2] = dx * cM
    else:
        B = np.zeros((Ne, nPg, 6, nPe * 3))
        dx, dy, dz = dNx[:, :, 0], dNx[:, :, 1], dNx[:, :, 2]
        B[:, :, 0, 0::3] = dx
        B[:, :, 1, 1::3] = dy
        B[:, :, 2, 2::3] = dz
        B[:, :, 3, 1::3] = dz * cM
        B[:, :, 3, 2::3] = dy * cM
        B[:, :, 4, 0::3] = dz * cM
        B[:, :, 4, 2::3] = dx * cM
        B[:, :, 5, 0::3] = dy * cM
        B[:, :, 5, 1::3] = dx * cM
    return B


# ---------------------------------------------------------------------------
# constitutive law (EasyFEA/Models/Elastic/_laws.py, Models/_utils.py)
# ---------------------------------------------------------------------------


def lame(E, v, dim, planeStress):
    """lambda, mu -- Elastic/_laws.py:376-403 (plane stress lambda = E v / (1 - v^2))."""
    E = np.asarray(E, dtype=float)
    lmbda = E * v / ((1 + v) * (1 - 2 * v))
    if dim == 2 and planeStress:
        lmbda = E * v / (1 - v**2)
    mu = E / (2 * (1 + v))
    return lmbda, mu


def isotropic_C(E, v, dim, planeStress=True):
    """Kelvin-Mandel C, Elastic/_laws.py:407-482 + Models/_utils.py:111-152.

    ``E`` scalar -> (3,3)/(6,6); ``E`` (Ne,) -> (Ne,3,3)/(Ne,6,6)
    (Heterogeneous_Array, Models/_utils.py:69-108).
    """
    lmbda, mu = lame(E, v, dim, planeStress)
    r2 = np.sqrt(2)
    if dim == 2:
        shape = np.shape(lmbda) + (3, 3)
        c = np.zeros(shape)
        c[..., 0, 0] = c[..., 1, 1] = lmbda + 2 * mu
        c[..., 0, 1] = c[..., 1, 0] = lmbda
        c[..., 2, 2] = mu
        T = np.array([[1, 1, r2], [1, 1, r2], [r2, r2, 2]])
    else:
        shape = np.shape(lmbda) + (6, 6)
        c = np.zeros(shape)
        for i in range(3):
            for j in range(3):
                c[..., i, j] = lmbda
            c[..., i, i] = lmbda + 2 * mu
        for i in range(3, 6):
            c[..., i, i] = mu
        T = np.ones((6, 6))
        T[3:, :3] = r2
        T[:3, 3:] = r2
        T[3:, 3:] = 2
    return c * T


# ---------------------------------------------------------------------------
# element operators (EasyFEA/FEM/Operators/Bilinear.py, Linear.py)
# ---------------------------------------------------------------------------


def K_elastic_e(geo: Geometry, C):
    """K_e = sum_pg wJ B^T C B -- Bilinear.py:62-79 (LinearizedElasticity).

    C: (n,n), (Ne,n,n) or (Ne,nPg,n,n)."""
    B = B_e_pg(geo.dNx)
    left = geo.wJ[:, :, None, None] * np.swapaxes(B, -1, -2)
    C = np.asarray(C)
    if C.ndim == 2:
        LC = left @ C
    elif C.ndim == 3:
        LC = left @ C[:, None]
    else:
        LC = left @ C
    return np.einsum("epij,epjk->eik", LC, B)


def UV_e(geo: Geometry, coef, dof_n=1):
    """M_e = sum_pg coef wJ N^T N -- Bilinear.py:42-59 with _group_elem.py:1338-1360."""
    N = geo.N  # (nPg, nPe)
    nPg, nPe = N.shape
    if dof_n == 1:
        Nr = N[:, None, :]
    else:
        Nr = np.zeros((nPg, dof_n, nPe * dof_n))
        for r in range(dof_n):
            Nr[:, r, r::dof_n] = N
    NtN = np.einsum("pri,prj->pij", Nr, Nr)
    coef = np.broadcast_to(np.asarray(coef, dtype=float), geo.wJ.shape) if np.ndim(coef) != 1 \
        else np.broadcast_to(np.asarray(coef, dtype=float)[:, None], geo.wJ.shape)
    return np.einsum("ep,pij->eij", coef * geo.wJ, NtN)


def GradU_A_GradV_e(geo: Geometry, A, k):
    """D_e = sum_pg k wJ dN^T A dN -- Bilinear.py:229-249 (_group_elem.py:1363-1380)."""
    A = np.asarray(A, dtype=float)
    return np.einsum("ep,epin,ij,epjm->enm", k * geo.wJ, geo.dNx, A, geo.dNx)


def V_e(geo: Geometry, f):
    """F_e = sum_pg f wJ N^T -- Linear.py:18-35 (_group_elem.py:1383-1407)."""
    return np.einsum("ep,pn->en", f * geo.wJ, geo.N)


# ---------------------------------------------------------------------------
# assembly (EasyFEA/Simulations/_simu.py:989-1102)
# ---------------------------------------------------------------------------


def assembly_e(connect, dof_n):
    """_group_elem.py:346-380."""
    Ne, nPe = connect.shape
    a = np.empty((Ne, nPe * dof_n), dtype=np.int64)
    for d in range(dof_n):
        a[:, d::dof_n] = connect * dof_n + d
    return a


def csr_map(connect, dof_n, Ndof):
    """(inv, indices, indptr, nnz) -- _simu.py:1062-1102 (__Get_csr_map).

    rows/cols from _group_elem.py:382-402 (row-major (i, j) over local DOFs);
    scipy builds the canonical pattern, searchsorted maps each element entry."""
    a = assembly_e(connect, dof_n)
    Ne, nd = a.shape
    rows = np.repeat(a, nd).reshape(Ne, nd * nd).ravel()
    cols = np.repeat(a, nd, axis=0).reshape(Ne, nd * nd).ravel()
    M = sp.csr_matrix((np.ones(rows.size), (rows, cols)), shape=(Ndof, Ndof))
    M.sort_indices()
    canon = np.repeat(np.arange(Ndof), np.diff(M.indptr)) * Ndof + M.indices
    invmap = np.searchsorted(canon, rows.astype(np.int64) * Ndof + cols).astype(np.int32)
    return invmap, M.indices, M.indptr, M.nnz


def assemble_csr(K_e, invmap, indices, indptr, nnz, Ndof):
    """np.bincount scatter, _simu.py:1044-1058."""
    data = np.bincount(invmap, weights=K_e.ravel(), minlength=nnz)
    A = sp.csr_matrix((data, indices, indptr), shape=(Ndof, Ndof))
    A.has_canonical_format = True
    return A


def assemble_vec(F_e, connect, dof_n, Ndof):
    """Vector assembly (isMatrix False), _simu.py:1086-1090 + :1044-1058."""
    a = assembly_e(connect, dof_n).ravel()
    return np.bincount(a, weights=np.asarray(F_e).ravel(), minlength=Ndof)


# ---------------------------------------------------------------------------
# boundary conditions (EasyFEA/Simulations/_simu.py:2400-2842)
# ---------------------------------------------------------------------------

UNKNOWNS = {1: ["d"], 2: ["x", "y"], 3: ["x", "y", "z"]}


def dofs_nodes(nodes, unknowns, available):
    """node * dof_n + index(unknown) -- FEM/_boundary_conditions.py:160-205."""
    nodes = np.asarray(nodes, dtype=np.int64)
    dof_n = len(available)
    out = np.zeros((nodes.size, len(unknowns)), dtype=np.int64)
    for i, u in enumerate(unknowns):
        out[:, i] = nodes * dof_n + available.index(u)
    return out.ravel()


def surf_load(elem, coord, connect, nodes, values, unknowns, available, thickness=1.0):
    """Neumann nodal loads -- _simu.py:2770-2842 (__Bc_Integration_Dim) with the
    2D thickness factor of :2572-2630.  A value is a constant or a function of
    (x, y, z), evaluated at the mass Gauss points (__Bc_evaluate, :2353-2385),
    or an array of one value per node of ``nodes``, integrated as
    value(node) x sum_g wJ N_node(g) (:2820-2826).

    Returns (dofs, dofsValues) in the COO form the reference appends."""
    nodes = np.asarray(nodes)
    mark = np.zeros(coord.shape[0], dtype=bool)
    mark[nodes] = True
    sel = np.nonzero(mark[connect].all(axis=1))[0]
    if sel.size == 0:
        return np.zeros(0, np.int64), np.zeros(0)
    con = connect[sel]
    geo = Geometry(elem, coord, con, "mass")
    Ne, nPe = con.shape
    vals = np.zeros((Ne * nPe, len(unknowns)))
    dofs = np.zeros((Ne * nPe, len(unknowns)), dtype=np.int64)
    for u, name in enumerate(unknowns):
        v = values[u]
        if isinstance(v, (int, float)) or callable(v):
            if callable(v):
                xg = np.einsum("pn,enk->epk", geo.N, coord[con])
                ev = np.zeros(geo.wJ.shape)
                ev[:, :] = v(xg[:, :, 0], xg[:, :, 1], xg[:, :, 2])
            else:
                ev = np.full(geo.wJ.shape, float(v))
            ve = np.einsum("ep,ep,pn->epn", geo.wJ, ev, geo.N)
        else:
            ev_n = np.zeros(coord.shape[0])
            ev_n[nodes] = v
            ve = np.einsum("ep,en,pn->epn", geo.wJ, ev_n[con], geo.N)
        vals[:, u] = ve.sum(1).ravel()
        dofs[:, u] = dofs_nodes(con.ravel(), [name], available)
    return dofs.ravel(), vals.ravel() * thickness


def solve_r1(A, b, known, known_values, orphan_dofs=()):
    """Dirichlet elimination + direct solve -- Solvers.py:502-553 (__Solver_1),
    _simu.py:1916-1968 (orphan diagonal fix), :2295-2316 (known/unknown sets),
    Solvers.py:361-362 (scipy spsolve)."""
    Ndof = A.shape[0]
    known = np.asarray(known, dtype=np.int64)
    x = sp.csr_matrix((np.asarray(known_values, float), (known, np.zeros_like(known))),
                      shape=(Ndof, 1)).toarray().ravel()
    if len(orphan_dofs):
        diag = np.zeros(Ndof)
        diag[np.asarray(orphan_dofs)] = 1.0
        A = A + sp.diags(diag, format="csr")
    mask = np.ones(Ndof, dtype=bool)
    mask[known] = False
    dk = np.nonzero(~mask)[0]
    du = np.nonzero(mask)[0]
    Ai = A[du, :].tocsc()
    Aii = Ai[:, du]
    Aic = Ai[:, dk]
    bi = b[du] - Aic @ x[dk]
    xi = sla.spsolve(Aii, bi)
    x[du] = xi
    return x


# ---------------------------------------------------------------------------
# phase-field split (EasyFEA/Models/_phasefield.py)
# ---------------------------------------------------------------------------


def vec_to_mat(v):
    """Project_vector_to_matrix, Models/_utils.py:155-188 (coef sqrt 2)."""
    n = v.shape[-1]
    dim = 2 if n == 3 else 3
    M = np.zeros(v.shape[:-1] + (dim, dim))
    for d in range(dim):
        M[..., d, d] = v[..., d]
    if dim == 2:
        M[..., 0, 1] = M[..., 1, 0] = v[..., 2] / SQRT2
    else:
        M[..., 1, 2] = M[..., 2, 1] = v[..., 3] / SQRT2
        M[..., 0, 2] = M[..., 2, 0] = v[..., 4] / SQRT2
        M[..., 0, 1] = M[..., 1, 0] = v[..., 5] / SQRT2
    return M


def mat_to_vec(M):
    """Project_matrix_to_vector, Models/_utils.py:191-222."""
    dim = M.shape[-1]
    if dim == 2:
        return np.stack([M[..., 0, 0], M[..., 1, 1], M[..., 0, 1] * SQRT2], -1)
    return np.stack([M[..., 0, 0], M[..., 1, 1], M[..., 2, 2],
                     M[..., 1, 2] * SQRT2, M[..., 0, 2] * SQRT2, M[..., 0, 1] * SQRT2], -1)


EIG_TOL_SQ = 1e-14
EIG_TOL_ARG = 1e-12
EIG_TOL_ZERO = 1e-12


def eigen_projectors(eps, robust=False):
    """Eigenvalues and eigenprojectors of the strain -- Models/_phasefield.py:751-1041.

    2D closed form :777-807; 3D Q.-C. He closed form with the Lode-angle cases
    :809-948 and the Frobenius normalisation of M1, M3 at :944-948.

    The reference chooses its repeated-eigenvalue branches by exact equality
    (v1 == v2, g == 0, theta == 0 or pi/3), and evaluates ``arccos`` of an
    argument that rounding can push just past +-1 (NaN there).  ``robust=False``
    reproduces that exactly; ``robust=True`` is the GPU kernels' form
    (_eigen_projectors_robust)."""
    if robust:
        return _eigen_projectors_robust(eps)
    M = vec_to_mat(eps)
    dim = M.shape[-1]
    I = np.zeros_like(M)
    for d in range(dim):
        I[..., d, d] = 1
    shp = eps.shape[:-1]
    if dim == 2:
        D = det(M)
        tr = M[..., 0, 0] + M[..., 1, 1]
        delta = tr**2 - 4 * D
        vals = np.zeros(shp + (2,))
        vals[..., 0] = (tr - np.sqrt(delta)) / 2
        vals[..., 1] = (tr + np.sqrt(delta)) / 2
        v1mv2 = vals[..., 0] - vals[..., 1]
        diff = vals[..., 0] != vals[..., 1]
        M1 = np.zeros_like(M)
        M1[..., 0, 0] = 1
        if diff.any():
            v = v1mv2.copy()
            v[v == 0] = 1
            m1 = (M - vals[..., 1][..., None, None] * I) / v[..., None, None]
            M1[diff] = m1[diff]
        M2 = I - M1
        return vals, [M1, M2]
    I1 = M[..., 0, 0] + M[..., 1, 1] + M[..., 2, 2]
    MM = M @ M
    I2 = 0.5 * (I1**2 - (MM[..., 0, 0] + MM[..., 1, 1] + MM[..., 2, 2]))
    I3 = det(M)
    g = I1**2 - 3 * I2
    sg = np.sqrt(g)
    gnz = g != 0
    arg = 0.5 * (2 * I1**3 - 9 * I1 * I2 + 27 * I3)
    arg = np.divide(arg, g ** (3 / 2), out=arg, where=gnz)
    with np.errstate(invalid="ignore"):
        theta = np.arccos(arg) / 3
    v1 = I1 / 3
    v2 = I1 / 3
    v3 = I1 / 3
    M1 = np.zeros_like(M)
    M1[..., 0, 0] = 1
    M3 = np.zeros_like(M)
    M3[..., 2, 2] = 1
    Irg = ((I1 - sg) / 3)[..., None, None] * I
    c2 = gnz & (theta == np.pi / 3)
    c3 = gnz & (theta == 0)
    c1 = gnz & (theta != 0) & (theta != np.pi / 3)
    c1 = c1 & ~c2 & ~c3
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        gm = g ** (-1 / 2)
    old = np.seterr(invalid="ignore", divide="ignore")
    if c2.any():
        v1 = np.where(c2, v1 - 2 / 3 * sg, v1)
        v2 = np.where(c2, v2 + 1 / 3 * sg, v2)
        v3 = np.where(c2, v3 + 1 / 3 * sg, v3)
        m1 = gm[..., None, None] * (Irg - M)
        M1 = np.where(c2[..., None, None], m1, M1)
        M3 = np.where(c2[..., None, None], 0.5 * (I - M1), M3)
    if c3.any():
        v1 = np.where(c3, v1 - 1 / 3 * sg, v1)
        v2 = np.where(c3, v2 - 1 / 3 * sg, v2)
        v3 = np.where(c3, v3 + 2 / 3 * sg, v3)
        m3 = gm[..., None, None] * (M - Irg)
        M3 = np.where(c3[..., None, None], m3, M3)
        M1 = np.where(c3[..., None, None], 0.5 * (I - M3), M1)
    if c1.any():
        v1 = np.where(c1, v1 + 2 / 3 * (sg * np.cos(2 * np.pi / 3 + theta)), v1)
        v2 = np.where(c1, v2 + 2 / 3 * (sg * np.cos(2 * np.pi / 3 - theta)), v2)
        v3 = np.where(c1, v3 + 2 / 3 * (sg * np.cos(theta)), v3)
        E3 = np.eye(3)
        a = v1[..., None, None]
        b = v2[..., None, None]
        c = v3[..., None, None]
        with np.errstate(divide="ignore", invalid="ignore"):
            m1 = (M - b * E3) @ (M - c * E3) / ((a - b) * (a - c))
            m3 = (M - a * E3) @ (M - b * E3) / ((c - a) * (c - b))
        M1 = np.where(c1[..., None, None], m1, M1)
        M3 = np.where(c1[..., None, None], m3, M3)
    np.seterr(**old)
    vals = np.stack([v1, v2, v3], -1)
    M1 = M1 / np.linalg.norm(M1, axis=(-2, -1))[..., None, None]
    M3 = M3 / np.linalg.norm(M3, axis=(-2, -1))[..., None, None]
    M2 = I - (M1 + M3)
    return vals, [M1, M2, M3]


def _eigen_projectors_robust(eps):
    """The GPU kernels' form of the same decomposition: eigenvalues from the
    deviator (2D: m -+ sqrt(h^2 + M01^2); 3D: g = 3/2 tr(s^2), arccos argument
    13.5 det(s) / g^1.5), repeated-eigenvalue branches chosen with the
    tolerances EIG_TOL_SQ / EIG_TOL_ARG, eigenvalues within EIG_TOL_ZERO of
    zero set to zero (Heaviside(0) = 1/2), projectors built from s."""
    M = vec_to_mat(eps)
    dim = M.shape[-1]
    I = np.broadcast_to(np.eye(dim), M.shape)
    shp = eps.shape[:-1]
    if dim == 2:
        tr = M[..., 0, 0] + M[..., 1, 1]
        h = (M[..., 0, 0] - M[..., 1, 1]) / 2
        rad2 = h * h + M[..., 0, 1] ** 2
        F2 = M[..., 0, 0] ** 2 + M[..., 1, 1] ** 2 + 2 * M[..., 0, 1] ** 2
        rep = rad2 <= 0.25 * EIG_TOL_SQ * F2
        rad = np.sqrt(np.where(rep, 0.0, rad2))
        vals = np.stack([tr / 2 - rad, tr / 2 + rad], -1)
        vals = np.where(np.abs(vals) <= EIG_TOL_ZERO * np.sqrt(F2)[..., None], 0.0, vals)
        safe = np.where(rep, 1.0, 2 * rad)
        M1 = np.zeros_like(M)
        M1[..., 0, 0] = np.where(rep, 1.0, (rad - h) / safe)
        M1[..., 1, 1] = np.where(rep, 0.0, (rad + h) / safe)
        M1[..., 0, 1] = M1[..., 1, 0] = np.where(rep, 0.0, -M[..., 0, 1] / safe)
        return vals, [M1, I - M1]
    I1 = M[..., 0, 0] + M[..., 1, 1] + M[..., 2, 2]
    trMM = np.einsum("...ik,...ki->...", M, M)
    S = M - (I1 / 3)[..., None, None] * I
    trSS = np.einsum("...ik,...ki->...", S, S)
    g = 1.5 * trSS
    g = np.where(g <= EIG_TOL_SQ * trMM, 0.0, g)
    sg = np.sqrt(g)
    gnz = g != 0
    sgs = np.where(gnz, sg, 1.0)
    arg = np.where(gnz, 13.5 * det(S) / (np.where(gnz, g, 1.0) * sgs), 0.0)
    arg = np.clip(arg, -1.0, 1.0)
    c2 = gnz & (arg <= -1 + EIG_TOL_ARG)
    c3 = gnz & ~c2 & (arg >= 1 - EIG_TOL_ARG)
    c1 = gnz & ~c2 & ~c3
    theta = np.arccos(arg) / 3
    sk = np.zeros(shp + (3,))
    sk[..., 0] = np.where(c2, -2 / 3 * sg, np.where(c3, -1 / 3 * sg, 2 / 3 * (sg * np.cos(2 * np.pi / 3 + theta))))
    sk[..., 1] = np.where(c2, 1 / 3 * sg, np.where(c3, -1 / 3 * sg, 2 / 3 * (sg * np.cos(2 * np.pi / 3 - theta))))
    sk[..., 2] = np.where(c2, 1 / 3 * sg, np.where(c3, 2 / 3 * sg, 2 / 3 * (sg * np.cos(theta))))
    sk = np.where(gnz[..., None], sk, 0.0)
    vals = (I1 / 3)[..., None] + sk
    vals = np.where(np.abs(vals) <= EIG_TOL_ZERO * np.sqrt(trMM)[..., None], 0.0, vals)
    M1 = np.zeros_like(M)
    M1[..., 0, 0] = 1
    M3 = np.zeros_like(M)
    M3[..., 2, 2] = 1
    Sp = S + (sg / 3)[..., None, None] * I
    gm = (1 / sgs)[..., None, None]
    m1c2 = -gm * Sp
    M1 = np.where(c2[..., None, None], m1c2, M1)
    M3 = np.where(c2[..., None, None], 0.5 * (I - m1c2), M3)
    m3c3 = gm * Sp
    M3 = np.where(c3[..., None, None], m3c3, M3)
    M1 = np.where(c3[..., None, None], 0.5 * (I - m3c3), M1)
    if c1.any():
        s0, s1, s2 = sk[..., 0, None, None], sk[..., 1, None, None], sk[..., 2, None, None]
        with np.errstate(divide="ignore", invalid="ignore"):
            m1 = (S - s1 * I) @ (S - s2 * I) / ((s0 - s1) * (s0 - s2))
            m3 = (S - s0 * I) @ (S - s1 * I) / ((s2 - s0) * (s2 - s1))
        M1 = np.where(c1[..., None, None], m1, M1)
        M3 = np.where(c1[..., None, None], m3, M3)
    M1 = M1 / np.linalg.norm(M1, axis=(-2, -1))[..., None, None]
    M3 = M3 / np.linalg.norm(M3, axis=(-2, -1))[..., None, None]
    return vals, [M1, I - (M1 + M3), M3]


def spectral_projectors(eps, robust=False):
    """projP, projM -- Models/_phasefield.py:1043-1243 (__Spectral_Decomposition)."""
    vals, Ms = eigen_projectors(eps, robust)
    dim = Ms[0].shape[-1]
    valp = (vals + np.abs(vals)) / 2
    dvalp = np.heaviside(vals, 0.5)
    if dim == 2:
        m1 = mat_to_vec(Ms[0])
        m2 = mat_to_vec(Ms[1])
        v = vals[..., 0] - vals[..., 1]
        v = np.where(v == 0, 1, v)
        BetaP = (valp[..., 0] - valp[..., 1]) / v
        gp = dvalp - BetaP[..., None]
        projP = (BetaP[..., None, None] * np.eye(3)
                 + gp[..., 0, None, None] * np.einsum("...i,...j->...ij", m1, m1)
                 + gp[..., 1, None, None] * np.einsum("...i,...j->...ij", m2, m2))
        return projP, np.eye(3) - projP
    M1, M2, M3 = Ms
    ms = [mat_to_vec(Mi) for Mi in Ms]
    th = dvalp / 2
    d12 = vals[..., 0] - vals[..., 1]
    d13 = vals[..., 0] - vals[..., 2]
    d23 = vals[..., 1] - vals[..., 2]
    d12 = np.where(d12 == 0, 1, d12)
    d13 = np.where(d13 == 0, 1, d13)
    d23 = np.where(d23 == 0, 1, d23)
    th = np.stack([(valp[..., 0] - valp[..., 1]) / (2 * d12),
                   (valp[..., 0] - valp[..., 2]) / (2 * d13),
                   (valp[..., 1] - valp[..., 2]) / (2 * d23)], -1)
    diag = sum(dvalp[..., k, None, None] * np.einsum("...i,...j->...ij", ms[k], ms[k]) for k in range(3))
    rI = np.array([0, 1, 2, 1, 0, 0])
    rJ = np.array([0, 1, 2, 2, 2, 1])
    scale = np.ones((6, 6))
    scale[3:, :3] = SQRT2
    scale[:3, 3:] = SQRT2
    scale[3:, 3:] = 2.0
    G = 0
    for t, (A, B) in enumerate([(M1, M2), (M1, M3), (M2, M3)]):
        A_ik = A[..., rI[:, None], rI[None, :]]
        A_il = A[..., rI[:, None], rJ[None, :]]
        A_jl = A[..., rJ[:, None], rJ[None, :]]
        B_ik = B[..., rI[:, None], rI[None, :]]
        B_il = B[..., rI[:, None], rJ[None, :]]
        B_jl = B[..., rJ[:, None], rJ[None, :]]
        Gab = (A_ik * B_jl + A_il * np.swapaxes(B_il, -1, -2)
               + B_ik * A_jl + B_il * np.swapaxes(A_il, -1, -2)) * scale
        G = G + th[..., t, None, None] * Gab
    projP = diag + G
    return projP, np.eye(6) - projP


def IxI(dim):
    I = np.array([1.0, 1.0, 0.0]) if dim == 2 else np.array([1.0, 1, 1, 0, 0, 0])
    return np.outer(I, I)


def split_C(eps, split, lmbda, mu, dim, C=None, robust=False, E=None, v=None, planeStress=False, S=None):
    """cP, cM -- Models/_phasefield.py:396-571 (Calc_C, Bourdin :433-449,
    Amor :451-483, Rp/Rm :485-501, Miehe :503-540), and the stress-based
    splits :573-687 (Zhang: projectors of sigma = C eps, cP = P+ C; Stress:
    cP = C s+ C with s+ from the isotropic compliance of sigma's positive
    part) and He :689-749 (projectors of C^1/2 eps mapped back, cP = C P+).

    ``lmbda``/``mu`` scalars or (Ne,) arrays; eps (Ne, nPg, 3|6); ``E``,
    ``v``, ``planeStress``: the isotropic material of the Stress split.

    Anisotropic splits (:541-567, 646-676): P+- of eps (AnisotStrain*) or of
    sigma = C eps (AnisotStress*, with the compliance ``S``), blocks
    Cab = Pa^T C Pb or (Pa C)^T S (Pb C), combined by variant."""
    Ne, nPg = eps.shape[:2]
    lm = np.broadcast_to(np.asarray(lmbda, float).reshape(-1, 1) if np.ndim(lmbda) else lmbda, (Ne, nPg))
    mm = np.broadcast_to(np.asarray(mu, float).reshape(-1, 1) if np.ndim(mu) else mu, (Ne, nPg))
    n = 3 if dim == 2 else 6
    II = IxI(dim)
    if split == "Bourdin":
        Cf = np.broadcast_to(C, (Ne, nPg, n, n)) if np.ndim(C) == 2 else np.broadcast_to(C[:, None], (Ne, nPg, n, n))
        return np.array(Cf), np.zeros((Ne, nPg, n, n))
    tr = eps[..., 0] + eps[..., 1] + (eps[..., 2] if dim == 3 else 0)
    Rp = (1 + np.sign(tr)) / 2
    Rm = (1 + np.sign(-tr)) / 2
    if split == "Amor":
        bulk = lm + 2 * mm / dim
        cP = bulk[..., None, None] * (Rp[..., None, None] * II) + 2 * mm[..., None, None] * (np.eye(n) - II / dim)
        cM = bulk[..., None, None] * (Rm[..., None, None] * II)
        return cP, cM
    if split.startswith("Anisot"):
        Cm = np.asarray(C, float)
        if split.startswith("AnisotStrain"):
            projP, projM = spectral_projectors(eps, robust)
            T = lambda X: np.swapaxes(X, -1, -2)  # noqa: E731
            Cpp, Cpm = T(projP) @ Cm @ projP, T(projP) @ Cm @ projM
            Cmp, Cmm = T(projM) @ Cm @ projP, T(projM) @ Cm @ projM
        else:
            sig = np.einsum("ij,epj->epi", Cm, eps)
            projP, projM = spectral_projectors(sig, robust)
            Cp, Cn = projP @ Cm, projM @ Cm
            T = lambda X: np.swapaxes(X, -1, -2)  # noqa: E731
            Sm = np.asarray(S, float)
            Cpp, Cpm = T(Cp) @ Sm @ Cp, T(Cp) @ Sm @ Cn
            Cmp, Cmm = T(Cn) @ Sm @ Cp, T(Cn) @ Sm @ Cn
        variant = split.split("_")[1] if "_" in split else ""
        if variant == "":
            return Cpp + Cpm + Cmp, Cmm
        if variant == "PM":
            return Cpp + Cpm, Cmm + Cmp
        if variant == "MP":
            return Cpp + Cmp, Cmm + Cpm
        return Cpp, Cmm + Cpm + Cmp
    if split == "Miehe":
        projP, projM = spectral_projectors(eps, robust)
        cP = lm[..., None, None] * (Rp[..., None, None] * II) + 2 * mm[..., None, None] * projP
        cM = lm[..., None, None] * (Rm[..., None, None] * II) + 2 * mm[..., None, None] * projM
        return cP, cM
    Cm = np.asarray(C, float)
    if split in ("Zhang", "Stress"):
        sig = np.einsum("ij,epj->epi", Cm, eps)
        projP, projM = spectral_projectors(sig, robust)
        if split == "Zhang":
            return projP @ Cm, projM @ Cm
        trs = sig[..., 0] + sig[..., 1] + (sig[..., 2] if dim == 3 else 0)
        Rp = ((1 + np.sign(trs)) / 2)[..., None, None]
        Rm = ((1 + np.sign(-trs)) / 2)[..., None, None]
        mu0 = float(np.ravel(mu)[0])
        if dim == 2:
            a1 = (1 + v) / E
            a2 = v / E if planeStress else v * (1 + v) / E
        else:
            a1 = 1 / (2 * mu0)
            a2 = v / E
        sP = a1 * projP - a2 * Rp * II
        sM = a1 * projM - a2 * Rm * II
        return Cm.T @ sP @ Cm, Cm.T @ sM @ Cm
    if split == "He":
        lam, Q = np.linalg.eigh(Cm)
        sqrtC = (Q * np.sqrt(lam)) @ Q.T
        sqrtS = (Q / np.sqrt(lam)) @ Q.T
        epst = np.einsum("ij,epj->epi", sqrtC, eps)
        pPt, pMt = spectral_projectors(epst, robust)
        projP = sqrtS @ pPt @ sqrtC
        projM = sqrtS @ pMt @ sqrtC
        return Cm @ projP, Cm @ projM
    raise NotImplementedError(split)


def psi_split(eps, cP, cM):
    """psi+- = 1/2 eps . (c+- eps) -- Models/_phasefield.py:335-394."""
    sP = np.einsum("epij,epj->epi", cP, eps)
    sM = np.einsum("epij,epj->epi", cM, eps)
    return np.sum(0.5 * eps * sP, -1), np.sum(0.5 * eps * sM, -1)


def pf_r_f_k(psiP, regu, Gc, l0):
    """Models/_phasefield.py:237-293."""
    if regu == "AT1":
        k = 3 / 4 * Gc * l0
        r = 2 * psiP
        f = 2 * psiP - (3 * Gc) / (8 * l0)
        f = (f + np.abs(f)) / 2
    else:
        k = Gc * l0
        r = 2 * psiP + Gc / l0
        f = 2 * psiP
    return r, f, k


# ---------------------------------------------------------------------------
# post-processing (EasyFEA/Models/_utils.py:302-430, Simulations/_elastic.py:
# 229-418, Simulations/_phasefield.py:682-915, FEM/_mesh.py:822-873,
# Simulations/_simu.py:3095-3151)
# ---------------------------------------------------------------------------

STRESS_COMPONENTS = {2: ("xx", "yy", "xy"), 3: ("xx", "yy", "zz", "yz", "xz", "xy")}


def strain_e_pg(geo: Geometry, connect, u):
    """eps = B u_e (Kelvin-Mandel) -- Models/Elastic/_laws.py:127-157."""
    dim = geo.dim
    u_e = np.asarray(u, float).reshape(-1, dim)[connect].reshape(len(connect), -1)
    return np.einsum("epij,ej->epi", B_e_pg(geo.dNx), u_e)


def stress_e_pg(C, eps):
    """sigma = C eps; C (n,n) or per element (Ne,n,n) -- Elastic/_laws.py:159-185."""
    C = np.asarray(C, float)
    if C.ndim == 2:
        return np.einsum("ij,epj->epi", C, eps)
    return np.einsum("eij,epj->epi", C, eps)


def result_in_field(field_e_pg, result, coef=SQRT2):
    """One result of a Kelvin-Mandel strain / stress field (Ne, nPg, n): a
    component with the shear ones times 1/coef, the von Mises equivalent, or
    the whole scaled field -- Models/_utils.py:302-392."""
    f = np.array(field_e_pg, dtype=float, copy=True)
    dim = 2 if f.shape[-1] == 3 else 3
    f[..., dim:] *= 1 / coef
    names = STRESS_COMPONENTS[dim]
    for i, nm in enumerate(names):
        if nm in result:
            return f[..., i]
    if "vm" in result:
        if dim == 2:
            xx, yy, xy = (f[..., i] for i in range(3))
            return np.sqrt(xx**2 + yy**2 - xx * yy + 3 * xy**2)
        xx, yy, zz, yz, xz, xy = (f[..., i] for i in range(6))
        return np.sqrt(0.5 * ((xx - yy) ** 2 + (yy - zz) ** 2 + (zz - xx) ** 2 + 6 * (xy**2 + yz**2 + xz**2)))
    if result in ("Strain", "Stress"):
        return f
    raise ValueError(result)


def node_values(connect, Nn, values_e):
    """Mean of the element values around each node -- FEM/_mesh.py:822-873
    (connect_n_e @ values_e * 1 / elements_n, _group_elem.py:322-345)."""
    values_e = np.asarray(values_e, float)
    is1d = values_e.ndim == 1
    ve = values_e.reshape(len(connect), -1)
    nPe = connect.shape[1]
    cne = sp.csr_matrix((np.ones(connect.size), (connect.ravel(), np.repeat(np.arange(len(connect)), nPe))),
                        shape=(Nn, len(connect)))
    cnt = np.asarray(cne.sum(axis=1)).reshape(-1, 1)
    with np.errstate(divide="ignore", invalid="ignore"):
        out = (cne @ ve) * 1 / cnt
    return out.ravel() if is1d else out


def reshape_values(values, nodeValues, connect, Nn):
    """Simulations/_simu.py:3095-3151: element values to nodes (node_values)
    or node values to elements (mean over the element's nodes); the size
    tests come first in the reference's order (a node-sized array is taken as
    node values)."""
    values = np.asarray(values, float)
    Ne = len(connect)
    is1d = values.ndim == 1
    if nodeValues:
        if values.size % Nn == 0:
            return values.ravel() if is1d else values.reshape(Nn, -1)
        vn = node_values(connect, Nn, values.reshape(Ne, -1))
        return vn.ravel() if is1d else vn.reshape(Nn, -1)
    if values.size % Ne == 0:
        return values.ravel() if is1d else values.reshape(Ne, -1)
    ve = np.mean(values.reshape(Nn, -1)[connect], axis=1)
    return ve.ravel() if is1d else ve.reshape(Ne, -1)


def psi_elas_e(geo: Geometry, eps, sig, thickness):
    """W_e = sum_pg thickness wJ 1/2 sig . eps -- Simulations/_elastic.py:322-395
    with Elastic/_laws.py:187-213."""
    psi = 0.5 * np.sum(sig * eps, -1)
    return (thickness * geo.wJ * psi).sum(1)


def zz1(geo: Geometry, connect, Nn, eps, sig, thickness):
    """ZZ1 error (global, per element) -- Simulations/_elastic.py:397-418:
    the energy of the node-averaged element-mean stress interpolated back
    with N against the plain energy."""
    W_e = psi_elas_e(geo, eps, sig, thickness)
    sig_n = node_values(connect, Nn, np.mean(sig, 1))
    sig_s = np.einsum("eni,pn->epi", sig_n[connect], geo.N)
    Ws_e = psi_elas_e(geo, eps, sig_s, thickness)
    Welas = W_e.sum()
    return abs(Welas - Ws_e.sum()) / Welas, np.abs(Ws_e - W_e).ravel() / Welas


def elastic_result(elem, coord, connect, u, C, result, thickness=1.0, nodeValues=True, coef=SQRT2):
    """Elastic.Result for the displacement, strain, stress and energy results
    (Simulations/_elastic.py:229-320)."""
    Nn = len(coord)
    dim = ELEM_DIM[elem]
    un = np.asarray(u, float).reshape(Nn, dim)
    if result in ("ux", "uy", "uz"):
        values = un[:, "xyz".index(result[1])]
    elif result == "displacement":
        values = np.asarray(u, float)
    elif result == "displacement_norm":
        values = np.linalg.norm(un, axis=1)
    elif result in ("Wdef", "Wdef_e", "ZZ1", "ZZ1_e"):
        geo = Geometry(elem, coord, connect, "rigi")
        eps = strain_e_pg(geo, connect, u)
        sig = stress_e_pg(C, eps)
        if result == "Wdef":
            return float(psi_elas_e(geo, eps, sig, thickness).sum())
        if result == "Wdef_e":
            values = psi_elas_e(geo, eps, sig, thickness)
        else:
            err, err_e = zz1(geo, connect, Nn, eps, sig, thickness)
            if result == "ZZ1":
                return err
            values = err_e
    else:
        geo = Geometry(elem, coord, connect, "rigi")
        eps = strain_e_pg(geo, connect, u)
        isStress = "S" in result and result != "Strain"
        field = stress_e_pg(C, eps) if isStress else eps
        res = result if result in ("Strain", "Stress") else result[-2:]
        values = result_in_field(field, res, coef).mean(1)
    return reshape_values(values, nodeValues, connect, Nn)


def degradation_e_pg(d, N, connect, k_res=1e-12):
    """g = (1 - N d_e)^2 + k_res -- Models/_phasefield.py:295-317."""
    d_pg = np.einsum("pn,en->ep", N, np.asarray(d, float)[connect])
    return (1 - d_pg) ** 2 + k_res


def pf_result(elem, coord, connect, u, d, split, lmbda, mu, C, result, thickness=1.0, nodeValues=True,
              H_old=None, coef=SQRT2, **split_kw):
    """PhaseField.Result for the strain, stress, damage and psiP results
    (Simulations/_phasefield.py:682-760): sigma = g(d) cP eps + cM eps at the
    rigi Gauss points (:868-915), psiP the mean of psi+ at the mass Gauss
    points, max'ed with the committed History field (:494-530, :706-714)."""
    Nn = len(coord)
    dim = ELEM_DIM[elem]
    if result == "damage":
        values = np.asarray(d, float)
    elif result in ("ux", "uy", "uz", "displacement", "displacement_norm"):
        return elastic_result(elem, coord, connect, u, C, result, thickness, nodeValues, coef)
    elif result == "psiP":
        geo = Geometry(elem, coord, connect, "mass")
        eps = strain_e_pg(geo, connect, u)
        cP, cM = split_C(eps, split, lmbda, mu, dim, C, **split_kw)
        psiP, _ = psi_split(eps, cP, cM)
        if H_old is not None:
            psiP = np.where(psiP - H_old.reshape(psiP.shape) < 0, H_old.reshape(psiP.shape), psiP)
        values = psiP.mean(1)
    else:
        geo = Geometry(elem, coord, connect, "rigi")
        eps = strain_e_pg(geo, connect, u)
        isStress = "S" in result and result != "Strain"
        if isStress:
            cP, cM = split_C(eps, split, lmbda, mu, dim, C, **split_kw)
            g = degradation_e_pg(d, geo.N, connect)
            sP = np.einsum("epij,epj->epi", cP, eps)
            sM = np.einsum("epij,epj->epi", cM, eps)
            field = g[..., None] * sP + sM
        else:
            field = eps
        res = result if result in ("Strain", "Stress") else result[-2:]
        values = result_in_field(field, res, coef).mean(1)
    return reshape_values(values, nodeValues, connect, Nn)
