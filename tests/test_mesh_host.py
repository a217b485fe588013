"""Mesh generators and host-side boundary-condition bookkeeping (CPU only)."""

import numpy as np
import pytest

from easyfea_gb300 import mesh as gmesh
from oracle import fem


@pytest.mark.parametrize("make,area", [
    (lambda: gmesh.Mesh_Quad4_Rect(120.0, 13.0, 24, 4), 120 * 13),
    (lambda: gmesh.Mesh_Tri3_Rect(1.0, 1.0, 8, 8), 1.0),
    (lambda: gmesh.Mesh_Quad9_Rect(3.0, 2.0, 4, 3), 6.0),
    (lambda: gmesh.Mesh_Hexa8_Box(3.0, 2.0, 1.0, 4, 3, 2), 6.0),
    (lambda: gmesh.Mesh_Tri10_Rect(3.0, 2.0, 4, 3), 6.0),
    (lambda: gmesh.Mesh_Tri15_Rect(3.0, 2.0, 4, 3), 6.0),
    (lambda: gmesh.Mesh_Prism6_Box(3.0, 2.0, 1.0, 4, 3, 2), 6.0),
    (lambda: gmesh.Mesh_Prism15_Box(3.0, 2.0, 1.0, 4, 3, 2), 6.0),
    (lambda: gmesh.Mesh_Prism18_Box(3.0, 2.0, 1.0, 4, 3, 2), 6.0),
])
def test_generators_positive_jacobian_and_measure(make, area):
    """Sum of wJ equals the domain measure (tests/FEM/mesh_test.py:135-149 of the reference)."""
    m = make()
    geo = fem.Geometry(m.elemType.value, m.coord, np.asarray(m.connect), "rigi")
    assert np.all(fem.det(geo.F) > 0), "elements must be positively oriented"
    # the reference's 6- and 12-point triangle rules have 15-digit literal
    # weights (the 6 weights sum to 1/2 - 1.5e-11)
    assert abs(geo.wJ.sum() - area) <= (1e-10 if m.elemType.value in ("TRI10", "TRI15") else 1e-11) * area


def test_boundary_groups_cover_the_boundary():
    m = gmesh.Mesh_Quad4_Rect(2.0, 1.0, 4, 2)
    seg = m.Get_list_groupElem(1)[0]
    assert seg.Ne == 2 * (4 + 2)
    h = gmesh.Mesh_Hexa8_Box(2.0, 1.0, 1.0, 4, 2, 2)
    faces = h.Get_list_groupElem(2)[0]
    assert faces.Ne == 2 * (4 * 2 + 4 * 2 + 2 * 2)
    assert h.orphanNodes.size == 0


@pytest.mark.parametrize("make", [gmesh.Mesh_Prism6_Box, gmesh.Mesh_Prism15_Box, gmesh.Mesh_Prism18_Box])
def test_prism_faces_cover_the_box(make):
    """The quadrangular side faces and the triangular end faces of a prism box
    (two boundary groups) add up to its surface, each face once, and every
    node belongs to an element."""
    m = make(3.0, 2.0, 1.0, 4, 3, 2)
    groups = m.Get_list_groupElem(2)
    assert sorted(g.elemType.value[:4] for g in groups) == ["QUAD", "TRI3" if make is gmesh.Mesh_Prism6_Box else "TRI6"]
    area = 0.0
    for g in groups:
        geo = fem.Geometry(g.elemType.value, m.coord, np.asarray(g.connect), "mass")
        area += geo.wJ.sum()
        assert len({tuple(sorted(r)) for r in g.connect}) == g.Ne
    # TRI6 faces: the 6-point rule's literal weights (sum 1/2 - 1.5e-11)
    assert abs(area - 2 * (3 * 2 + 3 * 1 + 2 * 1)) <= 1e-10 * area
    assert m.orphanNodes.size == 0


@pytest.mark.parametrize("make,p", [(gmesh.Mesh_Tri10_Rect, 3), (gmesh.Mesh_Tri15_Rect, 4)])
def test_higher_order_triangle_edges(make, p):
    """SEG4 / SEG5 boundary edges: the rectangle's perimeter, ends first and
    the inner nodes evenly spaced from the first end."""
    m = make(3.0, 2.0, 4, 3)
    seg = m.Get_list_groupElem(1)[0]
    x = m.coord[seg.connect]
    assert seg.Ne == 2 * (4 + 3)
    for k in range(1, p):
        assert np.allclose(x[:, 1 + k], x[:, 0] + k / p * (x[:, 1] - x[:, 0]))
    geo = fem.Geometry(seg.elemType.value, m.coord, np.asarray(seg.connect), "mass")
    assert abs(geo.wJ.sum() - 10.0) <= 1e-12


def test_rect_and_box_dispatch():
    """Mesh_Rect / Mesh_Box give every 2D / 3D element type its generator."""
    for et in ("TRI3", "TRI6", "TRI10", "TRI15", "QUAD4", "QUAD8", "QUAD9"):
        m = gmesh.Mesh_Rect(et, 2.0, 1.0, 2, 2)
        assert m.groupElem.elemType.value == et and m.dim == 2
    for et in ("TETRA4", "TETRA10", "HEXA8", "HEXA20", "HEXA27", "PRISM6", "PRISM15", "PRISM18"):
        m = gmesh.Mesh_Box(et, 2.0, 1.0, 1.0, 2, 1, 1)
        assert m.groupElem.elemType.value == et and m.dim == 3
    with pytest.raises(NotImplementedError):
        gmesh.Mesh_Box("QUAD4", 1.0, 1.0, 1.0, 1, 1, 1)


def test_assembly_e_layout():
    """Element DOF map node*dof_n + d (EasyFEA/FEM/_group_elem.py:346-380)."""
    m = gmesh.Mesh_Quad4_Rect(1.0, 1.0, 2, 2)
    a = m.groupElem.Get_assembly_e(2)
    np.testing.assert_array_equal(a, fem.assembly_e(np.asarray(m.connect), 2))


def test_get_elements_nodes_exclusively():
    m = gmesh.Mesh_Quad4_Rect(2.0, 1.0, 2, 1)
    seg = m.Get_list_groupElem(1)[0]
    right = m.Nodes_Conditions(lambda x, y, z: x == 2.0)
    els = seg.Get_Elements_Nodes(right)
    assert els.size == 1
    assert set(seg.connect[els[0]]) <= set(right)


def test_dirichlet_bookkeeping_sums_duplicates():
    """Duplicate Dirichlet DOFs add up (EasyFEA/Simulations/_simu.py:3013-3040)."""
    import types

    from easyfea_gb300 import Models
    from easyfea_gb300.simulations import Elastic

    m = gmesh.Mesh_Quad4_Rect(2.0, 1.0, 2, 1)
    mat = Models.Elastic.Isotropic(2, E=1.0, v=0.3)
    simu = Elastic.__new__(Elastic)
    # host bookkeeping only (no device): initialise the pieces Bc_* use
    simu.mesh = m
    simu._Elastic__K = None
    simu.model = mat
    simu.Bc_Init()
    left = m.Nodes_Conditions(lambda x, y, z: x == 0)
    simu.add_dirichlet(left, [1.0, 0.0], ["x", "y"])
    simu.add_dirichlet(left, [lambda x, y, z: y], ["x"])
    known, unknown = simu.Bc_dofs_known_unknown("elastic")
    np.testing.assert_array_equal(known, np.sort(np.concatenate([left * 2, left * 2 + 1])))
    xk = np.zeros(m.Nn * 2)
    for bc in simu._dirichlet["elastic"]:
        np.add.at(xk, bc.dofs, bc.values)
    np.testing.assert_allclose(xk[left * 2], 1.0 + m.coord[left, 1])
    assert isinstance(types, object)


def test_model_observers_trigger_update():
    from easyfea_gb300 import Models

    class Obs:
        n = 0

        def _Update(self, o):
            self.n += 1

    mat = Models.Elastic.Isotropic(2, E=210000.0, v=0.3)
    o = Obs()
    mat._Add_observer(o)
    mat.E = 100000.0
    mat.v = 0.25
    assert o.n == 2
    pfm = Models.PhaseField(mat, "Miehe", "AT2", 2.7, 0.01)
    o2 = Obs()
    pfm._Add_observer(o2)
    mat.E = 1.0
    pfm.Gc = 1.0
    assert o2.n == 2
    np.testing.assert_allclose(mat.C, fem.isotropic_C(1.0, 0.25, 2, True))


def test_isotropic_lame_detection():
    """Kelvin-Mandel matrices of isotropic laws are recognised (3D, plane
    strain, plane stress with its reduced lambda); anisotropic ones are not."""
    import numpy as np

    from easyfea_gb300 import Models
    from easyfea_gb300.simulations import isotropic_lame

    E, v = 210000.0, 0.3
    lam, mu = E * v / ((1 + v) * (1 - 2 * v)), E / (2 * (1 + v))
    for dim, ps, l_exp in ((3, False, lam), (2, False, lam), (2, True, 2 * lam * mu / (lam + 2 * mu))):
        got = isotropic_lame(Models.Elastic.Isotropic(dim, E=E, v=v, planeStress=ps).C)
        assert got is not None
        np.testing.assert_allclose(got, [l_exp, mu], rtol=1e-14)
    C = Models.Elastic.Isotropic(3, E=1.0, v=0.3).C.copy()
    C[0, 3] = C[3, 0] = 0.01
    assert isotropic_lame(C) is None
    assert isotropic_lame(np.zeros((6, 6))) is None
