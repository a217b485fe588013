"""The oracle's post-processing (strain / stress / energy / ZZ1 / psiP
results) against EasyFEA's own Elastic.Result and PhaseField.Result on the
fixtures of tests/golden/res_*.npz (CPU only)."""

import numpy as np
import pytest

from oracle import fem

ELASTIC = ["res_quad4", "res_quad4_hetero", "res_tri3", "res_quad9", "res_hexa8", "res_tetra4", "res_quad8",
           "res_tetra10", "res_hexa27", "res_tri10", "res_tri15", "res_prism6", "res_prism15", "res_prism18"]
PHASEFIELD = ["res_pf_tri3_miehe", "res_pf_quad4_amor", "res_pf_hexa8_miehe"]


def elastic_C(g):
    dim = fem.ELEM_DIM[str(g["elem"])]
    return fem.isotropic_C(g["E"], float(g["v"]), dim, bool(g["planeStress"])), dim


def close(a, b, rtol=1e-11):
    a = np.asarray(a, float)
    b = np.asarray(b, float)
    assert a.shape == b.shape, (a.shape, b.shape)
    scale = max(np.abs(b).max(), 1e-300)
    return np.abs(a - b).max() <= rtol * scale


@pytest.mark.parametrize("case", ELASTIC)
def test_elastic_results_oracle(golden, case):
    g = golden(case)
    C, dim = elastic_C(g)
    elem, coord, connect, u = str(g["elem"]), g["coord"], g["connect"], g["u"]
    t = float(g["thickness"])
    for r in [str(n) for n in g["names"]]:
        for suffix, nodeValues in (("_n", True), ("_e", False)):
            got = fem.elastic_result(elem, coord, connect, u, C, r, t, nodeValues)
            assert close(got, g[r + suffix]), (case, r, suffix)
    assert abs(fem.elastic_result(elem, coord, connect, u, C, "Wdef", t) - float(g["Wdef"])) <= 1e-12 * float(g["Wdef"])
    assert abs(fem.elastic_result(elem, coord, connect, u, C, "ZZ1", t) - float(g["ZZ1"])) <= 1e-11 * float(g["ZZ1"])


@pytest.mark.parametrize("case", PHASEFIELD)
def test_phasefield_results_oracle(golden, case):
    g = golden(case)
    elem, coord, connect = str(g["elem"]), g["coord"], g["connect"]
    dim = fem.ELEM_DIM[elem]
    E, v = float(g["E"]), float(g["v"])
    lmbda, mu = fem.lame(E, v, dim, False)
    C = fem.isotropic_C(E, v, dim, False)
    for r in [str(n) for n in g["names"]]:
        for suffix, nodeValues in (("_n", True), ("_e", False)):
            got = fem.pf_result(elem, coord, connect, g["u"], g["d"], str(g["split"]), lmbda, mu, C, r,
                                nodeValues=nodeValues, H_old=g["H_old"])
            assert close(got, g[r + suffix]), (case, r, suffix)


def test_psiP_history_is_active(golden):
    """The fixture's committed History field is above psi+ at part of the
    Gauss points and below at the rest, so psiP checks both branches."""
    g = golden("res_pf_tri3_miehe")
    elem, coord, connect = str(g["elem"]), g["coord"], g["connect"]
    lmbda, mu = fem.lame(210000.0, 0.3, 2, False)
    C = fem.isotropic_C(210000.0, 0.3, 2, False)
    geo = fem.Geometry(elem, coord, connect, "mass")
    eps = fem.strain_e_pg(geo, connect, g["u"])
    psiP, _ = fem.psi_split(eps, *fem.split_C(eps, "Miehe", lmbda, mu, 2, C))
    above = g["H_old"].reshape(psiP.shape) > psiP
    assert 0.2 < above.mean() < 0.8


def test_node_values_orphan_node_is_nan():
    """A node of no element gets 0/0 as in the reference's Get_Node_Values."""
    connect = np.array([[0, 1, 2]])
    v = fem.node_values(connect, 4, np.array([2.0]))
    assert np.allclose(v[:3], 2.0) and np.isnan(v[3])
