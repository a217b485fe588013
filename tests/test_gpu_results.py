"""Post-processing on the GPU (gfea_element_fields, gfea_node_incidence,
gfea_node_average through Elastic.Result / PhaseField.Result) against the
results of EasyFEA's own Elastic.Result and PhaseField.Result
(tests/golden/res_*.npz), and against the oracle on a larger mesh."""

import numpy as np
import pytest
import torch

from helpers import mesh_from_golden
from oracle import fem

pytestmark = pytest.mark.gpu

ELASTIC = ["res_quad4", "res_quad4_hetero", "res_tri3", "res_quad9", "res_hexa8", "res_tetra4", "res_quad8",
           "res_tetra10", "res_hexa27", "res_tri10", "res_tri15", "res_prism6", "res_prism15", "res_prism18"]
PHASEFIELD = ["res_pf_tri3_miehe", "res_pf_quad4_amor", "res_pf_hexa8_miehe"]

# element means of Gauss-point values and their node averages: FP64 with a
# different summation order than numpy's, so a few ulps of the largest value
RTOL = 1e-12


def close(a, b, rtol=RTOL):
    a = np.asarray(a, float)
    b = np.asarray(b, float)
    assert a.shape == b.shape, (a.shape, b.shape)
    return np.abs(a - b).max() <= rtol * max(np.abs(b).max(), 1e-300)


def elastic_simu(g):
    from easyfea_gb300 import Models
    from easyfea_gb300 import simulations as Simulations

    m = mesh_from_golden(g)
    E = g["E"]
    E = float(E) if E.ndim == 0 else np.asarray(E, float)
    mat = Models.Elastic.Isotropic(m.dim, E=E, v=float(g["v"]), planeStress=bool(g["planeStress"]),
                                   thickness=float(g["thickness"]))
    simu = Simulations.Elastic(m, mat)
    simu._Set_solutions("elastic", g["u"])
    return simu


@pytest.mark.parametrize("case", ELASTIC)
def test_elastic_results_match_reference(golden, case):
    g = golden(case)
    simu = elastic_simu(g)
    for r in [str(n) for n in g["names"]]:
        for suffix, nodeValues in (("_n", True), ("_e", False)):
            got = simu.Result(r, nodeValues=nodeValues)
            # ZZ1_e is a difference of two energies divided by the total
            assert close(got, g[r + suffix], 1e-10 if r.startswith("ZZ1") else RTOL), (case, r, suffix)
    assert abs(simu.Result("Wdef") - float(g["Wdef"])) <= 1e-12 * float(g["Wdef"])
    assert abs(simu.Result("ZZ1") - float(g["ZZ1"])) <= 1e-10 * float(g["ZZ1"])


def pf_simu(g):
    from easyfea_gb300 import Models
    from easyfea_gb300 import simulations as Simulations

    m = mesh_from_golden(g)
    mat = Models.Elastic.Isotropic(m.dim, E=float(g["E"]), v=float(g["v"]), planeStress=False, thickness=1.0)
    pfm = Models.PhaseField(mat, str(g["split"]), str(g["regu"]), float(g["Gc"]), float(g["l0"]))
    simu = Simulations.PhaseField(m, pfm)
    simu._Set_solutions("elastic", g["u"])
    simu._Set_solutions("damage", g["d"])
    simu.set_history(g["H_old"])
    return simu


@pytest.mark.parametrize("case", PHASEFIELD)
def test_phasefield_results_match_reference(golden, case):
    g = golden(case)
    simu = pf_simu(g)
    for r in [str(n) for n in g["names"]]:
        for suffix, nodeValues in (("_n", True), ("_e", False)):
            got = simu.Result(r, nodeValues=nodeValues)
            assert close(got, g[r + suffix], 1e-11), (case, r, suffix)
    assert abs(simu.Result("Wdef") - float(g["Wdef"])) <= 1e-11 * float(g["Wdef"])
    assert abs(simu.Result("Psi_Crack") - float(g["Psi_Crack"])) <= 1e-11 * float(g["Psi_Crack"])


def test_incidence_sorted_and_complete():
    """gfea_node_incidence: every (node, element) pair once, each list ascending."""
    from easyfea_gb300 import mesh as gmesh
    from easyfea_gb300.device import DeviceMesh

    m = gmesh.Mesh_Tetra4_Box(3.0, 2.0, 1.0, 9, 6, 4)
    dm = DeviceMesh(m)
    ptr, lst = (t.cpu().numpy() for t in dm.incidence())
    conn = m.groupElem.connect
    ref = [[] for _ in range(m.Nn)]
    for e, row in enumerate(conn):
        for a in row:
            ref[a].append(e)
    assert ptr[-1] == conn.size
    for a in range(m.Nn):
        assert list(lst[ptr[a]:ptr[a + 1]]) == ref[a]


@pytest.mark.parametrize("elem", ["QUAD4", "HEXA8"])
def test_results_larger_mesh_against_oracle(elem):
    """A mesh with tens of thousands of elements (many warps, grid-stride
    loop): Svm at the nodes, Strain on the elements and ZZ1 against the
    oracle."""
    from easyfea_gb300 import Models
    from easyfea_gb300 import mesh as gmesh
    from easyfea_gb300 import simulations as Simulations

    m = gmesh.Mesh_Quad4_Rect(10.0, 2.0, 250, 50) if elem == "QUAD4" else gmesh.Mesh_Hexa8_Box(4.0, 1.0, 1.0, 40, 10, 10)
    rng = np.random.default_rng(3)
    mat = Models.Elastic.Isotropic(m.dim, E=70000.0, v=0.33, planeStress=True, thickness=0.5)
    simu = Simulations.Elastic(m, mat)
    u = 1e-3 * rng.standard_normal(m.Nn * m.dim)
    simu._Set_solutions("elastic", u)
    C = fem.isotropic_C(70000.0, 0.33, m.dim, True)
    gr = m.groupElem
    for r, nv in (("Svm", True), ("Strain", False), ("Stress", True)):
        ref = fem.elastic_result(elem, m.coord, gr.connect, u, C, r, 0.5, nv)
        assert close(simu.Result(r, nodeValues=nv), ref), r
    assert abs(simu.Result("ZZ1") - fem.elastic_result(elem, m.coord, gr.connect, u, C, "ZZ1", 0.5)) <= 1e-9


def test_results_stay_on_device():
    """Result_device returns device tensors (no host round trip)."""
    from easyfea_gb300 import Models
    from easyfea_gb300 import mesh as gmesh
    from easyfea_gb300 import simulations as Simulations

    m = gmesh.Mesh_Quad4_Rect(2.0, 1.0, 20, 10)
    simu = Simulations.Elastic(m, Models.Elastic.Isotropic(2, E=1.0, v=0.3))
    simu._Set_solutions("elastic", np.linspace(0, 1e-3, m.Nn * 2))
    v = simu.Result_device("Svm")
    assert isinstance(v, torch.Tensor) and v.is_cuda and v.shape == (m.Nn,)
