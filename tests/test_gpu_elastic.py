"""Elastic assembly + solve on the GPU against the reference's outputs."""

import numpy as np
import pytest

from helpers import csr, mesh_from_golden, row_scaled_err, same_pattern

pytestmark = pytest.mark.gpu

CASES = ["el_quad4", "el_tri3", "el_quad9", "el_hexa8", "el_quad4_hetero", "el_hexa8_hetero", "el_cantilever_240x26",
         "el_tetra4", "el_tri6", "el_quad8", "el_tetra10", "el_hexa20", "el_hexa27", "el_tri10", "el_tri15", "el_prism6",
         "el_prism15", "el_prism18"]


def run_case(g, precision="fp64", rtol=1e-12):
    from easyfea_gb300 import Models
    from easyfea_gb300 import simulations as Simulations

    m = mesh_from_golden(g)
    dim = m.dim
    E = g["E"] if g["E"].ndim else float(g["E"])
    mat = Models.Elastic.Isotropic(dim, E=E, v=float(g["v"]), planeStress=bool(g["planeStress"]),
                                   thickness=float(g["thickness"]))
    simu = Simulations.Elastic(m, mat)
    simu.precision = precision
    simu.rtol = rtol
    unk = ["x", "y"] if dim == 2 else ["x", "y", "z"]
    simu.add_dirichlet(g["left"], [0.0] * dim, unk)
    simu.add_surfLoad(g["right"], [float(g["loadval"])], [str(g["loaddir"])])
    u = simu.Solve()
    return simu, u


@pytest.mark.parametrize("case", CASES)
def test_stiffness_matches_reference(golden, case):
    g = golden(case)
    simu, u = run_case(g)
    n = u.size
    K, C, M, F = simu.Get_K_C_M_F()
    Kref = csr(g, "K", n)
    assert same_pattern(K, Kref), "CSR pattern differs from the reference's"
    assert row_scaled_err(K, Kref) <= 1e-12
    assert row_scaled_err(M, csr(g, "M", n)) <= 1e-12
    b = simu._neumann_vec("elastic").cpu().numpy()
    np.testing.assert_allclose(b, g["b"], rtol=1e-12, atol=1e-13 * np.abs(g["b"]).max())


@pytest.mark.parametrize("case", CASES)
def test_displacement_matches_reference_direct_solve(golden, case):
    g = golden(case)
    simu, u = run_case(g)
    uref = g["u"]
    err = np.max(np.abs(u - uref)) / np.max(np.abs(uref))
    info = simu.last_solve
    assert info.status == 0
    # converged to 1e-12 or to the rounding floor of an FP64 residual
    assert info.rel_residual <= max(1e-12, info.floor_rel)
    assert err <= 1e-8, f"relative displacement error {err:.3e}"


@pytest.mark.parametrize("case", ["el_quad4", "el_hexa8", "el_cantilever_240x26"])
def test_mixed_precision_matches_fp64(golden, case):
    g = golden(case)
    simu, u = run_case(g, precision="mixed", rtol=1e-12)
    err = np.max(np.abs(u - g["u"])) / np.max(np.abs(g["u"]))
    info = simu.last_solve
    assert info.status == 0
    assert info.rel_residual <= max(1e-12, info.floor_rel)
    assert info.refinements >= 2
    assert err <= 1e-8, f"relative displacement error {err:.3e}"


def test_reaction_balances_load(golden):
    """Sum of reactions at the clamp equals minus the applied load."""
    g = golden("el_quad4")
    simu, u = run_case(g)
    dofs = simu.Bc_dofs_nodes(g["left"], ["y"])
    R = np.sum(simu.Calc_Reaction(dofs))
    total = float(g["loadval"]) * 13.0 * float(g["thickness"])
    assert abs(R + total) <= 1e-8 * abs(total)


@pytest.mark.parametrize("case", ["el_quad4_field_load", "el_hexa8_field_load"])
def test_field_loads_match_reference(golden, case):
    """Surface loads given as functions of position (evaluated at the
    boundary Gauss points) and as per-node arrays (EasyFEA/Simulations/
    _simu.py:2811-2832): Neumann vector within 1e-12, displacements 1e-8."""
    from easyfea_gb300 import Models
    from easyfea_gb300 import simulations as Simulations
    from helpers import field_loads

    g = golden(case)
    m = mesh_from_golden(g)
    dim = m.dim
    mat = Models.Elastic.Isotropic(dim, E=float(g["E"]), v=float(g["v"]), planeStress=bool(g["planeStress"]),
                                   thickness=float(g["thickness"]))
    simu = Simulations.Elastic(m, mat)
    simu.rtol = 1e-12
    simu.add_dirichlet(g["left"], [0.0] * dim, ["x", "y"] if dim == 2 else ["x", "y", "z"])
    for nodes, vals, unk in field_loads(dim, g["coord"], g["right"]):
        simu.add_surfLoad(nodes, vals, unk)
    u = simu.Solve()
    b = simu._neumann_vec("elastic").cpu().numpy()
    np.testing.assert_allclose(b, g["b"], rtol=1e-12, atol=1e-13 * np.abs(g["b"]).max())
    assert np.abs(u - g["u"]).max() <= 1e-8 * np.abs(g["u"]).max()


@pytest.mark.parametrize("case", ["el_quad4", "el_tri3", "el_quad9", "el_hexa8", "el_quad4_hetero", "el_hexa8_hetero",
                                  "el_cantilever_240x26", "el_tetra4"])
def test_f32_element_path_matches_reference(golden, case):
    """The FP32 element path (gfea_assemble_elastic / gfea_assemble_mass with
    GFEA_F32: geometry on the FP32 pipe from coordinates relative to each
    element's first node) against the reference's K and M, row-scaled,
    within 1e-6 (FP32 values)."""
    import torch

    from easyfea_gb300 import _lib

    g = golden(case)
    simu, u = run_case(g)
    n = u.size
    op = simu.K_device
    op.ensure_f32()
    C, mode = simu._C_device()
    dm, grp = simu.dmesh, simu.dmesh.main
    L = _lib.load()
    t = float(g["thickness"]) if simu.dim == 2 else 1.0
    _lib.check(L.gfea_assemble_elastic(grp.code, _lib.ptr(dm.coord), _lib.ptr(grp.connect), grp.Ne,
                                       _lib.ptr(dm.node_ptr), _lib.ptr(dm.rank), _lib.ptr(C), int(mode), t,
                                       _lib.F32, _lib.ptr(op.vals32), op.nnz, 0, _lib.stream()), "assemble f32")
    K32 = simu.K_device.to_scipy()
    K32.data = op.vals32.double().cpu().numpy()
    assert row_scaled_err(K32, csr(g, "K", n)) <= 1e-6
    m32 = torch.zeros(op.nnz, dtype=torch.float32, device="cuda")
    _lib.check(L.gfea_assemble_mass(grp.code, _lib.ptr(dm.coord), _lib.ptr(grp.connect), grp.Ne, _lib.ptr(dm.node_ptr),
                                    _lib.ptr(dm.rank), simu.dim, 1.0, t, _lib.F32, _lib.ptr(m32), op.nnz, 0,
                                    _lib.stream()), "mass f32")
    M32 = simu.K_device.to_scipy()
    M32.data = m32.double().cpu().numpy()
    assert row_scaled_err(M32, csr(g, "M", n)) <= 1e-6


def test_function_load_on_nine_point_faces():
    """A traction given as a function of position on QUAD9 faces (HEXA27, 9
    mass Gauss points per face) and QUAD8 faces (HEXA20): the Gauss-point
    buffer is sized from the face type; the load's resultant equals the
    integral of the function over the loaded face."""
    from easyfea_gb300 import Models
    from easyfea_gb300 import mesh as gmesh
    from easyfea_gb300 import simulations as Simulations

    for m in (gmesh.Mesh_Hexa27_Box(2.0, 1.0, 1.0, 2, 2, 2), gmesh.Mesh_Hexa20_Box(2.0, 1.0, 1.0, 2, 2, 2)):
        simu = Simulations.Elastic(m, Models.Elastic.Isotropic(3, E=1000.0, v=0.3, planeStress=False))
        right = np.where(np.abs(m.coord[:, 0] - 2.0) < 1e-12)[0]
        simu.add_surfLoad(right, [lambda x, y, z: 1.0 + y * z], ["z"])
        b = simu._neumann_vec("elastic").cpu().numpy().reshape(-1, 3)
        # integral over [0,1]^2 of 1 + y z = 1.25 (the 27-point rule is exact)
        assert abs(b[:, 2].sum() - 1.25) <= 1e-12
        assert np.abs(b[:, :2]).max() == 0.0


@pytest.mark.parametrize("make,dim", [("Mesh_Tri10_Rect", 2), ("Mesh_Tri15_Rect", 2), ("Mesh_Prism6_Box", 3),
                                      ("Mesh_Prism18_Box", 3)])
def test_function_load_on_higher_order_faces(make, dim):
    """A traction given as a function of position on SEG4 / SEG5 edges (TRI10
    / TRI15 rectangles, 4 / 5 mass points) and on the triangular end faces of
    prism boxes (TRI3 / TRI6, beside the quadrangular side faces): the load's
    resultant equals the integral of the function over the loaded edge or
    face."""
    from easyfea_gb300 import Models
    from easyfea_gb300 import mesh as gmesh
    from easyfea_gb300 import simulations as Simulations

    if dim == 2:
        m = getattr(gmesh, make)(2.0, 1.0, 3, 2)
        simu = Simulations.Elastic(m, Models.Elastic.Isotropic(2, E=1000.0, v=0.3, planeStress=True, thickness=0.5))
        right = np.where(np.abs(m.coord[:, 0] - 2.0) < 1e-12)[0]
        simu.add_surfLoad(right, [lambda x, y, z: 1.0 + y * y], ["y"])
        b = simu._neumann_vec("elastic").cpu().numpy().reshape(-1, 2)
        # thickness x integral over [0, 1] of 1 + y^2 = 0.5 x 4/3 (both rules are exact)
        assert abs(b[:, 1].sum() - 0.5 * 4.0 / 3.0) <= 1e-12
        assert np.abs(b[:, 0]).max() == 0.0
    else:
        m = getattr(gmesh, make)(2.0, 1.0, 1.0, 2, 2, 2)
        simu = Simulations.Elastic(m, Models.Elastic.Isotropic(3, E=1000.0, v=0.3, planeStress=False))
        top = np.where(np.abs(m.coord[:, 2] - 1.0) < 1e-12)[0]
        simu.add_surfLoad(top, [lambda x, y, z: 1.0 + x * y], ["x"])
        b = simu._neumann_vec("elastic").cpu().numpy().reshape(-1, 3)
        # integral over [0, 2] x [0, 1] of 1 + x y = 2 + 1 (the triangle rules are exact for degree 2;
        # the 6-point rule of the TRI6 faces has 15-digit literal weights summing to 1/2 - 1.5e-11)
        tol = 1e-12 if make == "Mesh_Prism6_Box" else 3e-10
        assert abs(b[:, 0].sum() - 3.0) <= tol
        assert np.abs(b[:, 1:]).max() == 0.0

