"""The drop-in inside EasyFEA itself: the reference's own Mesh, Models,
boundary-condition calls and Solve() loop, with ``GpuElastic`` /
``GpuPhaseField`` (easyfea_gb300/easyfea_binding.py) in place of
``Simulations.Elastic`` / ``Simulations.PhaseField``, against the fixtures the
reference produced.

EasyFEA is imported from an install of it (``EASYFEA_PATH``, else
``baseline/_ref`` in this repository); gmsh, which it imports at start-up,
is replaced by an empty module when absent (no mesher is used: meshes are
built from the fixtures' arrays with GroupElemFactory + Mesh).
"""

import os
import sys
import types

import numpy as np
import pytest

from helpers import csr, row_scaled_err, same_pattern

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def ref():
    path = os.environ.get("EASYFEA_PATH") or os.path.join(ROOT, "baseline", "_ref")
    if not os.path.isdir(os.path.join(path, "EasyFEA")):
        pytest.skip("EasyFEA is not installed (set EASYFEA_PATH or install it into baseline/_ref)")
    try:
        import gmsh  # noqa: F401
    except ImportError:
        sys.modules["gmsh"] = types.ModuleType("gmsh")
    if path not in sys.path:
        sys.path.insert(0, path)
    import EasyFEA  # noqa: F401
    from EasyFEA import Models, Simulations
    from EasyFEA.FEM._group_elem import GroupElemFactory
    from EasyFEA.FEM._mesh import Mesh
    from EasyFEA.FEM._utils import ElemType

    from easyfea_gb300 import easyfea_binding

    assert issubclass(easyfea_binding.GpuElastic, Simulations.Elastic)
    assert issubclass(easyfea_binding.GpuPhaseField, Simulations.PhaseField)
    return types.SimpleNamespace(Models=Models, Simulations=Simulations, GEF=GroupElemFactory, Mesh=Mesh,
                                 ElemType=ElemType, B=easyfea_binding)


def ref_mesh(R, g):
    from helpers import boundary_groups

    coord = np.asarray(g["coord"], dtype=float)
    groups = {}
    for e, c in boundary_groups(g) + [(str(g["elem"]), g["connect"])]:
        et = getattr(R.ElemType, e)
        groups[et] = R.GEF.Create(et, np.asarray(c, dtype=np.int64), coord.copy())
    return R.Mesh(groups)


@pytest.mark.parametrize("case", ["el_cantilever_240x26", "el_quad4_hetero", "el_hexa8", "el_tri15", "el_prism15"])
def test_gpu_elastic_inside_easyfea(ref, golden, case):
    """EasyFEA's Elastic.Solve() on the GPU subclass: u within 1e-8 of the
    reference's direct solve, K and M within 1e-12 (row-scaled) with the
    reference's CSR pattern, reactions through the reference's Calc_Reaction."""
    g = golden(case)
    R = ref
    mesh = ref_mesh(R, g)
    dim = mesh.dim
    E = np.asarray(g["E"], float)
    mat = R.Models.Elastic.Isotropic(dim, E=float(E) if E.ndim == 0 else E, v=float(g["v"]),
                                     planeStress=bool(g["planeStress"]), thickness=float(g["thickness"]))
    simu = R.B.GpuElastic(mesh, mat, rtol=1e-12)
    L = mesh.coord[:, 0].max()
    left = mesh.Nodes_Conditions(lambda x, y, z: x == 0)
    right = mesh.Nodes_Conditions(lambda x, y, z: x == L)
    unk = ["x", "y"] if dim == 2 else ["x", "y", "z"]
    simu.add_dirichlet(left, [0.0] * dim, unk)
    simu.add_surfLoad(right, [float(g["loadval"])], [str(g["loaddir"])])
    u = simu.Solve()
    assert simu.last_solve is not None and simu.last_solve.status == 0  # the GPU solver ran
    assert np.abs(u - g["u"]).max() <= 1e-8 * np.abs(g["u"]).max()
    K, C, M, F = simu.Get_K_C_M_F()
    Kref = csr(g, "K", u.size)
    assert same_pattern(K, Kref) and row_scaled_err(K, Kref) <= 1e-12
    assert row_scaled_err(M, csr(g, "M", u.size)) <= 1e-12
    assert C.nnz == K.nnz and np.abs(C.data).max() == 0.0 and F.shape == (u.size, 1)
    # the reference's own post-processing reads the GPU-assembled K
    f = np.sum(simu.Calc_Reaction(simu.Bc_dofs_nodes(left, unk)))
    f_ref = np.sum((Kref @ g["u"])[simu.Bc_dofs_nodes(left, unk)])
    assert abs(f - f_ref) <= 1e-8 * np.abs(Kref @ g["u"]).max() * len(left)
    # Rayleigh damping through the reference's own setter: C = coefK K + coefM M
    simu.Set_Rayleigh_Damping_Coefs(coefM=0.5, coefK=2e-3)
    K2, C2, M2, _ = simu.Get_K_C_M_F()
    assert abs(C2 - (2e-3 * K2 + 0.5 * M2)).max() <= 1e-15 * abs(K2).max()


@pytest.mark.parametrize("case,opt", [("pf_tri3_miehe_at2", 0), ("pf_tri3_conv2", 2)])
def test_gpu_phasefield_inside_easyfea(ref, golden, case, opt):
    """EasyFEA's staggered load loop (Bc_Init, add_dirichlet, Solve, Save_Iter,
    Calc_Reaction) on the GPU subclass: iterations per step equal to the
    reference's, force within 1e-6, damage within 1e-6."""
    g = golden(case)
    R = ref
    mesh = ref_mesh(R, g)
    mat = R.Models.Elastic.Isotropic(2, E=float(g["E"]), v=float(g["v"]), planeStress=bool(g["planeStress"]),
                                     thickness=1.0)
    pfm = R.Models.PhaseField(mat, str(g["split"]), str(g["regu"]), float(g["Gc"]), float(g["l0"]))
    simu = R.B.GpuPhaseField(mesh, pfm)
    top_dofs = simu.Bc_dofs_nodes(g["top"], ["y"])
    for k in range(1, g["F"].shape[0] + 1):
        simu.Bc_Init()
        simu.add_dirichlet(g["notch"], [1.0], ["d"], problemType="damage")
        simu.add_dirichlet(g["bottom"], [0.0, 0.0], ["x", "y"])
        simu.add_dirichlet(g["top"], [0.0, k * float(g["dU"])], ["x", "y"])
        u, d, conv = simu.Solve(float(g["tol"]), int(g["maxIter"]), convOption=opt)
        simu.Save_Iter()
        F = np.sum(simu.Calc_Reaction(top_dofs, simu.ProblemTypes.elastic))
        # staggered iterations as the reference's Save_Iter recorded them
        niter = simu._Simu__list_results[-1]["Niter"]
        assert niter == g["Niter"][k - 1], f"step {k}: {niter} vs {g['Niter'][k - 1]}"
        assert abs(F - g["F"][k - 1]) <= 1e-6 * abs(g["F"][k - 1]), f"step {k}: F {F} vs {g['F'][k - 1]}"
        assert np.abs(d - g["d"][k - 1]).max() <= 1e-6


@pytest.mark.parametrize("algo", ["newmark", "hht", "midpoint", "euler_implicit", "parabolic"])
def test_gpu_time_schemes_inside_easyfea(ref, golden, algo):
    """EasyFEA's time integration (Solver_Set_Hyperbolic_Algorithm /
    Parabolic; EasyFEA/Simulations/_simu.py:1173-1456, Solvers.py:69-182) with
    Rayleigh damping on the GPU subclass, against the reference's own Elastic
    (scipy SuperLU) run step by step in the same script: u, v and a within
    1e-8 of their scale after every step."""
    from EasyFEA.Simulations.Solvers import AlgoType, SolverType

    g = golden("el_quad4")
    R = ref
    mesh = ref_mesh(R, g)
    sims = []
    for cls in (R.Simulations.Elastic, R.B.GpuElastic):
        mat = R.Models.Elastic.Isotropic(2, E=210000.0, v=0.3, planeStress=True, thickness=13.0)
        simu = cls(mesh, mat) if cls is R.Simulations.Elastic else cls(mesh, mat, rtol=1e-13)
        if cls is R.Simulations.Elastic:
            simu.solver = SolverType.scipy
        simu.rho = 7.8e-9
        simu.Set_Rayleigh_Damping_Coefs(coefM=1e-3, coefK=1e-5)
        dt = 2e-5
        if algo == "parabolic":
            simu.Solver_Set_Parabolic_Algorithm(dt)
        else:
            simu.Solver_Set_Hyperbolic_Algorithm(dt, algo=getattr(AlgoType, algo))
        sims.append(simu)
    left = mesh.Nodes_Conditions(lambda x, y, z: x == 0)
    right = mesh.Nodes_Conditions(lambda x, y, z: x == mesh.coord[:, 0].max())
    for step in range(6):
        for simu in sims:
            simu.Bc_Init()
            simu.add_dirichlet(left, [0.0, 0.0], ["x", "y"])
            simu.add_surfLoad(right, [-800 / 13**2 * (1.0 if step < 3 else 0.5)], ["y"])
            simu.Solve()
            simu.Save_Iter()
        ref_s, gpu_s = sims
        assert gpu_s.last_solve is not None and gpu_s.last_solve.status == 0
        # v and a are differences of displacements over dt and dt^2: a
        # displacement difference e (solver rounding) moves them by e/dt and
        # e/dt^2, which the tolerance allows for
        umax = np.abs(ref_s.displacement).max()
        for name, amp in (("displacement", 1.0), ("speed", 1.0 / dt), ("accel", 1.0 / dt**2)):
            a, b = getattr(gpu_s, name), getattr(ref_s, name)
            if b is None or np.size(b) == 0 or np.abs(b).max() == 0:
                continue
            tol = 1e-8 * (np.abs(b).max() if name == "displacement" else np.abs(b).max() + umax * amp)
            assert np.abs(a - b).max() <= tol, (algo, step, name, np.abs(a - b).max(), tol)


@pytest.mark.parametrize("case", ["res_quad4_hetero", "res_hexa8", "res_tetra4", "res_tri15", "res_prism15"])
def test_gpu_results_inside_easyfea(ref, golden, case):
    """The reference's Result() on the GPU subclass: strain, stress, von Mises,
    energy and ZZ1 results from the device against the reference's own."""
    g = golden(case)
    R = ref
    mesh = ref_mesh(R, g)
    E = np.asarray(g["E"], float)
    mat = R.Models.Elastic.Isotropic(mesh.dim, E=float(E) if E.ndim == 0 else E, v=float(g["v"]),
                                     planeStress=bool(g["planeStress"]), thickness=float(g["thickness"]))
    simu = R.B.GpuElastic(mesh, mat)
    simu._Set_solutions(simu.problemType, g["u"])
    for r in [str(n) for n in g["names"]]:
        for suffix, nodeValues in (("_n", True), ("_e", False)):
            got = np.asarray(simu.Result(r, nodeValues=nodeValues))
            want = g[r + suffix]
            tol = 1e-10 if r.startswith("ZZ1") else 1e-12
            assert np.abs(got - want).max() <= tol * np.abs(want).max(), (case, r, suffix)
    assert abs(simu.Result("ZZ1") - float(g["ZZ1"])) <= 1e-10 * float(g["ZZ1"])


def test_gpu_phasefield_results_inside_easyfea(ref, golden):
    """PhaseField.Result on the GPU subclass at a prescribed (u, d, History) state."""
    from EasyFEA.FEM import FeArray

    g = golden("res_pf_hexa8_miehe")
    R = ref
    mesh = ref_mesh(R, g)
    mat = R.Models.Elastic.Isotropic(mesh.dim, E=float(g["E"]), v=float(g["v"]), planeStress=False, thickness=1.0)
    pfm = R.Models.PhaseField(mat, str(g["split"]), str(g["regu"]), float(g["Gc"]), float(g["l0"]))
    simu = R.B.GpuPhaseField(mesh, pfm)
    simu._Set_solutions(simu.ProblemTypes.elastic, g["u"])
    simu._Set_solutions(simu.ProblemTypes.damage, g["d"])
    simu._PhaseField__old_psiP_e_pg = FeArray.asfearray(np.array(g["H_old"]))
    for r in [str(n) for n in g["names"]]:
        for suffix, nodeValues in (("_n", True), ("_e", False)):
            got = np.asarray(simu.Result(r, nodeValues=nodeValues))
            want = g[r + suffix]
            assert np.abs(got - want).max() <= 1e-11 * np.abs(want).max(), (r, suffix)
    assert abs(simu.Result("Wdef") - float(g["Wdef"])) <= 1e-11 * float(g["Wdef"])


def test_gpu_transversely_isotropic_inside_easyfea(ref, golden):
    """A transversely isotropic law of EasyFEA's own through GpuElastic."""
    g = golden("el_quad4_ti")
    R = ref
    mesh = ref_mesh(R, g)
    law = {k: (float(g["ti_" + k]) if g["ti_" + k].ndim == 0 else g["ti_" + k])
           for k in ("El", "Et", "Gl", "vl", "vt", "axis_l", "axis_t")}
    mat = R.Models.Elastic.TransverselyIsotropic(2, **law, planeStress=bool(g["planeStress"]),
                                                 thickness=float(g["thickness"]))
    simu = R.B.GpuElastic(mesh, mat, rtol=1e-12)
    L = mesh.coord[:, 0].max()
    left = mesh.Nodes_Conditions(lambda x, y, z: x == 0)
    right = mesh.Nodes_Conditions(lambda x, y, z: x == L)
    simu.add_dirichlet(left, [0.0, 0.0], ["x", "y"])
    simu.add_surfLoad(right, [float(g["loadval"])], [str(g["loaddir"])])
    u = simu.Solve()
    assert simu.last_solve is not None and simu.last_solve.status == 0
    assert np.abs(u - g["u"]).max() <= 1e-8 * np.abs(g["u"]).max()
    K = simu.Get_K_C_M_F()[0]
    assert row_scaled_err(K, csr(g, "K", u.size)) <= 1e-12
