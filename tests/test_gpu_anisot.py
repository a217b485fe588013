"""Anisotropic laws and splits on the GPU against EasyFEA's own outputs:
gfea_pf_split with the eight AnisotStrain / AnisotStress variants, the
elastic solve of a transversely isotropic cantilever (2D and 3D), and the
staggered loop with the AnisotStrain and AnisotStress splits."""

import ctypes

import numpy as np
import pytest
import torch

from helpers import csr, mesh_from_golden, row_scaled_err, same_pattern
from test_anisot_host import CASES, SPLITS, ti_law

pytestmark = pytest.mark.gpu


def gpu_split(eps, split, dim, C, S):
    from easyfea_gb300 import _lib

    L = _lib.load()
    p = _lib.PfParams()
    p.version = _lib.ABI_VERSION
    p.split = _lib.SPLIT_CODE[split]
    p.regularization = 1
    p.dim = dim
    p.Gc, p.l0, p.thickness, p.k_res = 2.7, 0.01, 1.0, 1e-12
    for i, v in enumerate(np.asarray(C).ravel()):
        p.C[i] = v
    for i, v in enumerate(np.asarray(S).ravel()):
        p.S[i] = v
    n = 3 if dim == 2 else 6
    e = torch.as_tensor(np.ascontiguousarray(eps.reshape(-1, n)), device="cuda")
    npt = e.shape[0]
    cP = torch.empty(npt, n, n, dtype=torch.float64, device="cuda")
    cM = torch.empty_like(cP)
    psiP = torch.empty(npt, dtype=torch.float64, device="cuda")
    psiM = torch.empty_like(psiP)
    _lib.check(L.gfea_pf_split(_lib.ptr(e), npt, ctypes.byref(p), _lib.ptr(cP), _lib.ptr(cM), _lib.ptr(psiP),
                               _lib.ptr(psiM), _lib.stream()), "split")
    return cP.cpu().numpy(), cM.cpu().numpy(), psiP.cpu().numpy(), psiM.cpu().numpy()


@pytest.mark.parametrize("dim,ps", CASES)
@pytest.mark.parametrize("split", SPLITS)
def test_anisot_split_kernel_matches_reference(golden, dim, ps, split):
    g = golden("anisot")
    key = f"ti_d{dim}_ps{int(ps)}"
    C, S, eps = g[key + "_C"], g[key + "_S"], g[key + "_eps"]
    cP, cM, psiP, psiM = gpu_split(eps, split, dim, C, S)
    n = cP.shape[-1]
    sc = np.abs(C).max()
    assert np.abs(cP - g[f"{key}_{split}_cP"].reshape(-1, n, n)).max() <= 1e-12 * sc
    assert np.abs(cM - g[f"{key}_{split}_cM"].reshape(-1, n, n)).max() <= 1e-12 * sc
    gp, gm = g[f"{key}_{split}_psiP"].ravel(), g[f"{key}_{split}_psiM"].ravel()
    s = np.abs(gp).max() + np.abs(gm).max()
    assert np.abs(psiP - gp).max() <= 1e-12 * s
    assert np.abs(psiM - gm).max() <= 1e-12 * s


@pytest.mark.parametrize("case", ["el_quad4_ti", "el_hexa8_ti"])
def test_ti_elastic_solve_matches_reference(golden, case):
    from easyfea_gb300 import simulations as Simulations

    g = golden(case)
    m = mesh_from_golden(g)
    dim = m.dim
    mat = ti_law(g, dim, bool(g["planeStress"]), float(g["thickness"]), prefix="ti_")
    assert np.abs(mat.C - g["C"]).max() <= 1e-13 * np.abs(g["C"]).max()
    simu = Simulations.Elastic(m, mat)
    simu.rtol = 1e-12
    unk = ["x", "y"] if dim == 2 else ["x", "y", "z"]
    simu.add_dirichlet(g["left"], [0.0] * dim, unk)
    simu.add_surfLoad(g["right"], [float(g["loadval"])], [str(g["loaddir"])])
    u = simu.Solve()
    K = simu.Get_K_C_M_F()[0]
    Kref = csr(g, "K", u.size)
    assert same_pattern(K, Kref) and row_scaled_err(K, Kref) <= 1e-12
    assert np.abs(u - g["u"]).max() <= 1e-8 * np.abs(g["u"]).max()


@pytest.mark.parametrize("split", ["AnisotStrain", "AnisotStress"])
def test_ti_staggered_loop_matches_reference(golden, split):
    from easyfea_gb300 import Models
    from easyfea_gb300 import simulations as Simulations

    g = golden(f"pf_tri3_ti_{split.lower()}")
    m = mesh_from_golden(g)
    mat = ti_law(g, 2, bool(g["planeStress"]), prefix="ti_")
    simu = Simulations.PhaseField(m, Models.PhaseField(mat, split, str(g["regu"]), float(g["Gc"]), float(g["l0"])))
    top_dofs = torch.as_tensor(g["top_dofs"], device="cuda")
    for k in range(1, g["u"].shape[0] + 1):
        simu.Bc_Init()
        simu.add_dirichlet(g["notch"], [1.0], ["d"], problemType="damage")
        simu.add_dirichlet(g["bottom"], [0.0, 0.0], ["x", "y"])
        simu.add_dirichlet(g["top"], [0.0, k * float(g["dU"])], ["x", "y"])
        u, d, conv = simu.Solve(float(g["tol"]), int(g["maxIter"]), convOption=0)
        simu.Save_Iter()
        F = simu.reaction_sum(top_dofs)
        assert simu.staggered_iterations == g["Niter"][k - 1], f"step {k}"
        assert abs(F - g["F"][k - 1]) <= 1e-6 * abs(g["F"][k - 1]), f"step {k}: F {F} vs {g['F'][k - 1]}"
        assert np.max(np.abs(d - g["d"][k - 1])) <= 1e-6, f"step {k}"
