"""Isotropic laws assemble through the (lambda, mu) form of the element
kernel (modes 3 and 4); it must give the same stiffness as the general
Kelvin-Mandel path (modes 0 and 2) and as the reference."""

import ctypes

import numpy as np
import pytest
import torch

from helpers import csr, mesh_from_golden, row_scaled_err

pytestmark = pytest.mark.gpu


def assemble(simu, C, mode):
    from easyfea_gb300 import _lib

    dm = simu.dmesh
    g = dm.main
    op = simu.K_device
    factor = simu.material.thickness if simu.dim == 2 else 1.0
    vals = torch.zeros_like(op.vals64)
    L = _lib.load()
    _lib.check(L.gfea_assemble_elastic(g.code, _lib.ptr(dm.coord), _lib.ptr(g.connect), g.Ne, _lib.ptr(dm.node_ptr),
                                       _lib.ptr(dm.rank), _lib.ptr(C), int(mode), factor, _lib.F64, _lib.ptr(vals),
                                       op.nnz, 0, _lib.stream()), "assemble")
    torch.cuda.synchronize()
    return vals.cpu().numpy()


@pytest.mark.parametrize("case", ["el_quad4", "el_quad9", "el_hexa8", "el_tri3", "el_quad4_hetero", "el_hexa8_hetero"])
def test_lame_form_equals_kelvin_mandel(golden, case):
    import scipy.sparse as sp

    from easyfea_gb300 import Models
    from easyfea_gb300 import simulations as Simulations

    g = golden(case)
    m = mesh_from_golden(g)
    E = g["E"] if g["E"].ndim else float(g["E"])
    mat = Models.Elastic.Isotropic(m.dim, E=E, v=float(g["v"]), planeStress=bool(g["planeStress"]),
                                   thickness=float(g["thickness"]))
    simu = Simulations.Elastic(m, mat)
    dev = torch.device("cuda", 0)
    if np.ndim(E):
        ref = Models.Elastic.Isotropic(m.dim, E=1.0, v=float(g["v"]), planeStress=bool(g["planeStress"])).C
        lame = Simulations.isotropic_lame(ref)
        Ev = np.asarray(E, dtype=np.float64).ravel()
        k_km = assemble(simu, torch.as_tensor(np.concatenate([ref.ravel(), Ev]), device=dev), 2)
        k_iso = assemble(simu, torch.as_tensor(np.concatenate([lame, Ev]), device=dev), 4)
    else:
        C = np.ascontiguousarray(mat.C, dtype=np.float64)
        k_km = assemble(simu, torch.as_tensor(C, device=dev), 0)
        k_iso = assemble(simu, torch.as_tensor(Simulations.isotropic_lame(C), device=dev), 3)
    indptr, indices = simu.dmesh.pattern(simu.dim)
    ip, ix = indptr.cpu().numpy(), indices.cpu().numpy()
    N = simu.dim * m.Nn
    K0 = sp.csr_matrix((k_km, ix, ip), shape=(N, N))
    K1 = sp.csr_matrix((k_iso, ix, ip), shape=(N, N))
    assert row_scaled_err(K1, K0) <= 1e-13
    # and the simulation's own assembly (which picks the isotropic form) matches the reference
    assert row_scaled_err(simu.K_device.to_scipy(), csr(g, "K", N)) <= 1e-12
