"""The oracle's element tables on their own (CPU only): every element's shape
functions interpolate its nodes (Kronecker delta at the nodes' local
coordinates, EasyFEA/FEM/Elems/*.py Get_Local_Coords), sum to one, have
derivatives that match central differences, and its Gauss rules integrate
the reference element's measure and a low-degree monomial exactly
(EasyFEA/FEM/_gauss.py)."""

import numpy as np
import pytest

from oracle import fem

# local coordinates of the nodes in the reference's order, for the elements
# the oracle does not already list
NODES = {
    "SEG2": [[-1], [1]], "SEG3": [[-1], [1], [0]],
    "TRI3": [[0, 0], [1, 0], [0, 1]], "TRI6": [[0, 0], [1, 0], [0, 1], [0.5, 0], [0.5, 0.5], [0, 0.5]],
    "QUAD4": [[-1, -1], [1, -1], [1, 1], [-1, 1]],
    "QUAD8": [[-1, -1], [1, -1], [1, 1], [-1, 1], [0, -1], [1, 0], [0, 1], [-1, 0]],
    "QUAD9": [[-1, -1], [1, -1], [1, 1], [-1, 1], [0, -1], [1, 0], [0, 1], [-1, 0], [0, 0]],
    "TETRA4": [[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]],
    "TETRA10": [[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1], [0.5, 0, 0], [0.5, 0.5, 0], [0, 0.5, 0], [0, 0, 0.5],
                [0, 0.5, 0.5], [0.5, 0, 0.5]],
    "HEXA8": fem.HEXA_LOCAL[:8].tolist(), "HEXA20": fem.HEXA_LOCAL[:20].tolist(), "HEXA27": fem.HEXA_LOCAL.tolist(),
}
NODES.update({k: v for k, v in fem.LOCAL_NODES.items()})

# measure of each reference element
MEASURE = {"SEG": 2.0, "TRI": 0.5, "QUAD": 4.0, "TETRA": 1 / 6, "HEXA": 8.0, "PRISM": 1.0}
ELEMS = sorted(fem.ELEM_DIM)


def _inside(elem, rng):
    dim = fem.ELEM_DIM[elem]
    if elem.startswith(("SEG", "QUAD", "HEXA")):
        return rng.uniform(-0.9, 0.9, dim)
    if elem.startswith("TRI"):
        a, b = rng.uniform(0.05, 0.45, 2)
        return np.array([a, b])
    if elem.startswith("TETRA"):
        return rng.uniform(0.05, 0.3, 3)
    a, b = rng.uniform(0.05, 0.45, 2)
    return np.array([a, b, rng.uniform(-0.9, 0.9)])


@pytest.mark.parametrize("elem", ELEMS)
def test_shape_functions_interpolate_the_nodes(elem):
    nodes = np.asarray(NODES[elem], float)
    N = np.array([fem.shape_N(elem, x) for x in nodes])
    assert N.shape == (len(nodes), len(nodes))
    assert np.abs(N - np.eye(len(nodes))).max() <= 1e-12


@pytest.mark.parametrize("elem", ELEMS)
def test_partition_of_unity_and_derivatives(elem):
    rng = np.random.default_rng(1)
    h = 1e-6
    for _ in range(4):
        x = _inside(elem, rng)
        N = fem.shape_N(elem, x)
        dN = fem.shape_dN(elem, x)
        assert abs(N.sum() - 1.0) <= 1e-12
        assert np.abs(dN.sum(axis=1)).max() <= 1e-11
        for d in range(len(x)):
            e = np.zeros(len(x))
            e[d] = h
            fd = (fem.shape_N(elem, x + e) - fem.shape_N(elem, x - e)) / (2 * h)
            assert np.abs(fd - dN[d]).max() <= 1e-7 * max(1.0, np.abs(dN[d]).max())


@pytest.mark.parametrize("elem", ELEMS)
@pytest.mark.parametrize("matrixType", ["rigi", "mass"])
def test_gauss_rules_integrate_the_element(elem, matrixType):
    """Weights sum to the reference element's measure (within the 15-digit
    literals of the 6- and 12-point triangle rules) and every point lies in
    the element."""
    pts, w = fem.gauss(elem, matrixType)
    family = next(k for k in MEASURE if elem.startswith(k))
    tol = 1e-10 if family in ("TRI",) else 1e-13
    assert abs(w.sum() - MEASURE[family]) <= tol * MEASURE[family]
    assert np.all(w > 0)
    if family in ("TRI", "TETRA"):
        assert np.all(pts >= -1e-15) and np.all(pts.sum(axis=1) <= 1 + 1e-15)
    elif family == "PRISM":
        assert np.all(pts[:, :2] >= 0) and np.all(pts[:, :2].sum(axis=1) <= 1) and np.all(np.abs(pts[:, 2]) <= 1)
    else:
        assert np.all(np.abs(pts) <= 1)
