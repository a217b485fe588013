"""Parity at the benchmark's full sizes, against the oracle.

* The 3D box of the benchmark (HEXA8 400 x 40 x 40, 2,022,243 DOF) is too large
  for the reference to assemble in one piece or to solve directly, so the
  oracle applies its operator element by element on chunks (y = sum_e K_e x_e
  with the reference's K_e formula): the GPU CSR operator must reproduce it,
  and the GPU mixed-precision solution's residual is measured with it.
* The notched phase-field plate (200 x 200 squares split into 80,000 TRI3,
  AT2, Miehe) runs its first load steps on the GPU and in the oracle.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def oracle_apply(coord, connect, C, x, chunk=32000):
    """(sum_e K_e x_e, sum_e |K_e| |x_e|) with the oracle's element matrices."""
    from oracle import fem

    N = x.size
    y = np.zeros(N)
    yabs = np.zeros(N)
    for s in range(0, connect.shape[0], chunk):
        conn = connect[s:s + chunk]
        geo = fem.Geometry("HEXA8", coord, conn, "rigi")
        Ke = fem.K_elastic_e(geo, C)
        ae = fem.assembly_e(conn, 3)
        xe = x[ae]
        y += np.bincount(ae.ravel(), weights=np.einsum("eij,ej->ei", Ke, xe).ravel(), minlength=N)
        yabs += np.bincount(ae.ravel(), weights=np.einsum("eij,ej->ei", np.abs(Ke), np.abs(xe)).ravel(),
                            minlength=N)
    return y, yabs


@pytest.fixture(scope="module")
def box():
    import torch

    from easyfea_gb300 import Models
    from easyfea_gb300 import mesh as gmesh
    from easyfea_gb300 import simulations as Simulations
    from oracle import fem

    m = gmesh.Mesh_Hexa8_Box(1000.0, 100.0, 100.0, 400, 40, 40)
    simu = Simulations.Elastic(m, Models.Elastic.Isotropic(3, E=210000.0, v=0.3, planeStress=False))
    simu.precision = "mixed"
    simu.rtol = 1e-10
    left = m.Nodes_Conditions(lambda x, y, z: x == 0)
    right = m.Nodes_Conditions(lambda x, y, z: x == 1000.0)
    simu.add_dirichlet(left, [0.0, 0.0, 0.0], ["x", "y", "z"])
    simu.add_surfLoad(right, [-1.0], ["z"])
    u = simu.Solve()
    C = fem.isotropic_C(210000.0, 0.3, 3)
    yield simu, m, u, C, left
    del simu
    torch.cuda.empty_cache()


def test_box_operator_matches_oracle_elementwise(box):
    """GPU SpMV with the assembled FP64 CSR = the oracle's sum of element
    products, to rounding (1e-13 of |K||x|)."""
    import torch

    simu, m, u, C, _ = box
    rng = np.random.default_rng(7)
    x = rng.standard_normal(3 * m.Nn)
    y_gpu = simu.K_device.matvec(torch.as_tensor(x, device="cuda")).cpu().numpy()
    y_ref, y_abs = oracle_apply(m.coord, np.asarray(m.connect, np.int64), C, x)
    err = np.abs(y_gpu - y_ref).max() / y_abs.max()
    assert err <= 1e-13, err


def test_box_solution_residual_with_oracle_operator(box):
    """The mixed-precision solution satisfies the oracle's FP64 equations to
    the FP64 rounding floor of this problem (reported by the solver)."""
    simu, m, u, C, left = box
    info = simu.last_solve
    assert info.status == 0
    b = simu._neumann_vec("elastic").cpu().numpy()
    Ku, Kabs = oracle_apply(m.coord, np.asarray(m.connect, np.int64), C, u)
    known = np.zeros(u.size, bool)
    known[simu.Bc_dofs_nodes(left, ["x", "y", "z"])] = True
    r = np.where(known, 0.0, b - Ku)
    rel = np.linalg.norm(r) / np.linalg.norm(np.where(known, 0.0, b))
    floor = 32 * np.finfo(float).eps * np.linalg.norm(np.where(known, 0.0, Kabs + np.abs(b))) / \
        np.linalg.norm(np.where(known, 0.0, b))
    assert rel <= max(1e-10, 2 * floor), (rel, floor)
    assert rel <= 2e-7


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_notched_plate_first_steps_match_oracle(precision):
    """The phase-field benchmark plate (80,000 TRI3): force, damage and
    displacement of the first load steps against the oracle's staggered
    scheme (SuperLU)."""
    import torch

    from easyfea_gb300 import Models
    from easyfea_gb300 import mesh as gmesh
    from easyfea_gb300 import simulations as Simulations
    from oracle.simulate import OracleMesh, PhaseFieldOracle

    m = gmesh.Mesh_Tri3_Rect(1.0, 1.0, 200, 200)
    x = m.coord
    bottom = np.where(x[:, 1] == 0)[0]
    top = np.where(x[:, 1] == 1.0)[0]
    notch = np.where((np.abs(x[:, 1] - 0.5) < 1e-12) & (x[:, 0] <= 0.5))[0]
    mat = Models.Elastic.Isotropic(2, E=210e3, v=0.3, planeStress=False)
    simu = Simulations.PhaseField(m, Models.PhaseField(mat, "Miehe", "AT2", 2.7, 0.01))
    simu.precision = precision
    simu.rtol = 1e-12
    pf = PhaseFieldOracle(OracleMesh.from_mesh(m), 210e3, 0.3, False, 1.0, "Miehe", "AT2", 2.7, 0.01)
    top_y = 2 * top + 1
    top_dofs = torch.as_tensor(top_y, device="cuda")
    dU = 1e-5
    for k in (1, 2, 3):
        simu.Bc_Init()
        simu.add_dirichlet(notch, [1.0], ["d"], problemType="damage")
        simu.add_dirichlet(bottom, [0.0, 0.0], ["x", "y"])
        simu.add_dirichlet(top, [0.0, k * dU], ["x", "y"])
        u, d, _ = simu.Solve(1e-3, 500, convOption=0)
        simu.Save_Iter()
        F = simu.reaction_sum(top_dofs)
        pf.dir_d = [(notch, [1.0], ["d"])]
        pf.dir_u = [(bottom, [0.0, 0.0], ["x", "y"]), (top, [0.0, k * dU], ["x", "y"])]
        u_ref, d_ref, _ = pf.solve(1e-3, 500, 0)
        pf.save_iter()
        F_ref = float(np.sum(pf.reaction(top_y)))
        assert simu.staggered_iterations == pf.Niter, (k, simu.staggered_iterations, pf.Niter)
        assert abs(F - F_ref) <= 1e-6 * abs(F_ref), (k, F, F_ref)
        assert np.abs(d - d_ref).max() <= 1e-6, k
        assert np.abs(u - u_ref).max() <= 1e-6 * np.abs(u_ref).max(), k


def test_notched_plate_load_curve_matches_reference(golden):
    """The phase-field benchmark through its whole load history: the
    reference's own run of the 200x200 notched plate (80,000 TRI3, AT2,
    Miehe, top displacement k x 1e-5 mm, Solve(1e-3, 500, convOption=0) and
    Save_Iter per step; make_golden.py pf_curve_tri3_200x200) against the
    GPU staggered loop in FP64: the same staggered iteration count at every
    step, the top reaction within 1e-6 relative, the damage field within 1e-6
    at the stored steps (every 50th, the force peak, the last)."""
    import torch

    from easyfea_gb300 import Models
    from easyfea_gb300 import mesh as gmesh
    from easyfea_gb300 import simulations as Simulations

    g = golden("pf_curve_tri3_200x200")
    m = gmesh.Mesh_Tri3_Rect(1.0, 1.0, 200, 200)
    mat = Models.Elastic.Isotropic(2, E=210e3, v=0.3, planeStress=False)
    simu = Simulations.PhaseField(m, Models.PhaseField(mat, "Miehe", "AT2", 2.7, 0.01))
    simu.precision = "fp64"
    simu.rtol = 1e-12
    top_dofs = torch.as_tensor(g["top_dofs"], device="cuda")
    kept = {int(k): i for i, k in enumerate(g["d_steps"])}
    dU, tol, maxIter = float(g["dU"]), float(g["tol"]), int(g["maxIter"])
    for k in range(1, len(g["F"]) + 1):
        simu.Bc_Init()
        simu.add_dirichlet(g["notch"], [1.0], ["d"], problemType="damage")
        simu.add_dirichlet(g["bottom"], [0.0, 0.0], ["x", "y"])
        simu.add_dirichlet(g["top"], [0.0, k * dU], ["x", "y"])
        u, d, conv = simu.Solve(tol, maxIter, convOption=0)
        simu.Save_Iter()
        F = simu.reaction_sum(top_dofs)
        assert simu.staggered_iterations == g["Niter"][k - 1], f"step {k}: {simu.staggered_iterations} staggered iterations, reference {g['Niter'][k - 1]}"
        assert bool(conv) == bool(g["converged"][k - 1]), f"step {k}"
        assert abs(F - g["F"][k - 1]) <= 1e-6 * abs(g["F"][k - 1]), f"step {k}: F {F} vs {g['F'][k - 1]}"
        if k in kept:
            assert np.abs(d - g["d"][kept[k]]).max() <= 1e-6, f"step {k}"
