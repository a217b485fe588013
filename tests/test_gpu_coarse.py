"""Two-level preconditioner (block-Jacobi + rigid-body-mode coarse level)
against the reference's direct solves, and its options."""

import numpy as np
import pytest

from helpers import mesh_from_golden

pytestmark = pytest.mark.gpu


def elastic(g, precision="fp64", rtol=1e-12, coarse=-1):
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
    simu.coarse = coarse
    unk = ["x", "y"] if dim == 2 else ["x", "y", "z"]
    simu.add_dirichlet(g["left"], [0.0] * dim, unk)
    simu.add_surfLoad(g["right"], [float(g["loadval"])], [str(g["loaddir"])])
    return simu


def rel_err(u, uref):
    return np.max(np.abs(u - uref)) / np.max(np.abs(uref))


@pytest.mark.parametrize("case", ["el_quad4", "el_tri3", "el_quad9", "el_hexa8", "el_quad4_hetero",
                                  "el_cantilever_240x26"])
@pytest.mark.parametrize("coarse", [0, 1, 7, 64, 100000])
def test_any_coarse_size_matches_reference(golden, case, coarse):
    """Block-Jacobi alone, one aggregate, odd counts and a request above the
    cap all converge to the reference's direct solution."""
    g = golden(case)
    simu = elastic(g, coarse=coarse)
    u = simu.Solve()
    info = simu.last_solve
    assert info.status == 0
    assert info.rel_residual <= max(1e-12, info.floor_rel)
    assert rel_err(u, g["u"]) <= 1e-8


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_coarse_level_cuts_iterations(golden, precision):
    g = golden("el_cantilever_240x26")
    its = {}
    for coarse in (0, -1):
        simu = elastic(g, precision=precision, rtol=1e-10, coarse=coarse)
        u = simu.Solve()
        assert rel_err(u, g["u"]) <= 1e-8
        its[coarse] = simu.last_solve.iterations
    assert its[-1] * 3 <= its[0], its


def test_reused_aggregation_gives_the_same_solution(golden):
    """A second solve on the same mesh keeps the workspace's aggregation and
    rebuilds only the coarse matrix (new values)."""
    from easyfea_gb300.device import Workspace, pcg

    g = golden("el_hexa8")
    simu = elastic(g)
    simu.Solve()
    op = simu.K_device
    b = simu._neumann_vec("elastic")
    ws = Workspace()
    out = []
    for scale in (1.0, 2.0, 2.0):
        op.vals64.mul_(scale)
        known, x = simu._dirichlet_state("elastic", b)
        pcg(op, b, x, known, rtol=1e-12, coarse=-1, workspace=ws)
        assert ws.key is not None
        out.append(x.cpu().numpy())
    fresh_known, fresh = simu._dirichlet_state("elastic", b)
    pcg(op, b, fresh, fresh_known, rtol=1e-12, coarse=-1)
    # K scaled by 2 then by 4: u scales by 1/2 then 1/4
    assert rel_err(out[1] * 2, out[0]) <= 1e-9
    assert rel_err(out[2] * 2, out[1]) <= 1e-9
    assert rel_err(out[2], fresh.cpu().numpy()) <= 1e-9


@pytest.mark.parametrize("coarse_scalar", [-1, 5])
def test_scalar_damage_system_with_coarse_level(golden, coarse_scalar):
    """dof_n = 1 (the damage system of each staggered iteration): the coarse
    modes are constants per aggregate; the loop still follows the reference."""
    import torch

    from easyfea_gb300 import Models
    from easyfea_gb300 import simulations as Simulations

    g = golden("pf_tri3_miehe_at2")
    m = mesh_from_golden(g)
    mat = Models.Elastic.Isotropic(m.dim, E=float(g["E"]), v=float(g["v"]), planeStress=bool(g["planeStress"]),
                                   thickness=1.0)
    pfm = Models.PhaseField(mat, str(g["split"]), str(g["regu"]), float(g["Gc"]), float(g["l0"]))
    simu = Simulations.PhaseField(m, pfm)
    simu.coarse_scalar = coarse_scalar
    top_dofs = torch.as_tensor(g["top_dofs"], device="cuda")
    for k in range(1, g["u"].shape[0] + 1):
        simu.Bc_Init()
        simu.add_dirichlet(g["notch"], [1.0], ["d"], problemType="damage")
        simu.add_dirichlet(g["bottom"], [0.0, 0.0], ["x", "y"])
        simu.add_dirichlet(g["top"], [0.0, k * float(g["dU"])], ["x", "y"])
        u, d, conv = simu.Solve(float(g["tol"]), int(g["maxIter"]), convOption=0)
        simu.Save_Iter()
        F = simu.reaction_sum(top_dofs)
        assert simu.staggered_iterations == g["Niter"][k - 1]
        assert abs(F - g["F"][k - 1]) <= 1e-6 * abs(g["F"][k - 1]), f"step {k}"
        assert np.max(np.abs(d - g["d"][k - 1])) <= 1e-6, f"step {k}"


def test_known_everywhere_but_one_aggregate(golden):
    """Aggregates whose DOFs are all known get an identity coarse block."""
    g = golden("el_quad4")
    simu = elastic(g, coarse=16)
    m = simu.mesh
    # clamp the left half as well: many aggregates become fully constrained
    half = np.where(m.coord[:, 0] <= 0.5 * m.coord[:, 0].max())[0]
    simu.add_dirichlet(half, [0.0, 0.0], ["x", "y"])
    u = simu.Solve()
    assert simu.last_solve.status == 0
    ref = elastic(g, coarse=0)
    ref.add_dirichlet(half, [0.0, 0.0], ["x", "y"])
    uref = ref.Solve()
    assert rel_err(u, uref) <= 1e-9
