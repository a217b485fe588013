"""Row-owned assembly (gfea_assemble_elastic_parts) against the atomic element
kernel and against the reference's K."""

import ctypes

import numpy as np
import pytest
import torch

from helpers import csr, mesh_from_golden, row_scaled_err
from oracle import fem

pytestmark = pytest.mark.gpu


def meshes():
    from easyfea_gb300 import mesh as gmesh

    return {"TRI3": gmesh.Mesh_Tri3_Rect(1.0, 1.0, 30, 30), "QUAD4": gmesh.Mesh_Quad4_Rect(12.0, 3.0, 60, 20),
            "QUAD9": gmesh.Mesh_Quad9_Rect(6.0, 2.0, 20, 8), "HEXA8": gmesh.Mesh_Hexa8_Box(4.0, 1.0, 1.0, 20, 6, 6),
            "TETRA4": gmesh.Mesh_Tetra4_Box(3.0, 1.0, 1.0, 8, 4, 4), "TRI6": gmesh.Mesh_Tri6_Rect(1.0, 1.0, 20, 20),
            "QUAD8": gmesh.Mesh_Quad8_Rect(6.0, 2.0, 24, 8), "TETRA10": gmesh.Mesh_Tetra10_Box(2.0, 1.0, 1.0, 4, 2, 2),
            "HEXA20": gmesh.Mesh_Hexa20_Box(2.0, 1.0, 1.0, 6, 3, 3), "HEXA27": gmesh.Mesh_Hexa27_Box(2.0, 1.0, 1.0, 6, 3, 3),
            "TRI10": gmesh.Mesh_Tri10_Rect(1.0, 1.0, 12, 12), "TRI15": gmesh.Mesh_Tri15_Rect(1.0, 1.0, 10, 10),
            "PRISM6": gmesh.Mesh_Prism6_Box(3.0, 1.0, 1.0, 12, 4, 4), "PRISM15": gmesh.Mesh_Prism15_Box(2.0, 1.0, 1.0, 6, 3, 3),
            "PRISM18": gmesh.Mesh_Prism18_Box(2.0, 1.0, 1.0, 6, 3, 3)}


def law(mode, dim, Ne, rng):
    """The C argument of each c_per_elem mode (gfea.h) for E = 210000, nu = 0.3."""
    C = fem.isotropic_C(210000.0, 0.3, dim, dim == 2)
    lmbda, mu = fem.lame(210000.0, 0.3, dim, dim == 2)
    f = np.exp(0.3 * rng.standard_normal(Ne))
    if mode == 0:
        return C.ravel()
    if mode == 1:
        return (f[:, None, None] * C[None]).ravel()
    if mode == 2:
        return np.concatenate([C.ravel(), f])
    if mode == 3:
        return np.array([lmbda, mu])
    return np.concatenate([[lmbda, mu], f])


@pytest.mark.parametrize("elem", ["TRI3", "QUAD4", "QUAD9", "HEXA8", "TETRA4", "TRI6", "QUAD8", "TETRA10", "HEXA20",
                                  "HEXA27", "TRI10", "TRI15", "PRISM6", "PRISM15", "PRISM18"])
@pytest.mark.parametrize("vt", ["f64", "f32"])
@pytest.mark.parametrize("mode", [0, 1, 2, 3, 4])
def test_parts_match_atomic_kernel(elem, vt, mode):
    from easyfea_gb300 import _lib
    from easyfea_gb300.device import DeviceMesh

    m = meshes()[elem]
    dm = DeviceMesh(m)
    g = dm.main
    dim = m.dim
    rng = np.random.default_rng(4)
    C = torch.as_tensor(law(mode, dim, g.Ne, rng), device="cuda")
    code = _lib.F64 if vt == "f64" else _lib.F32
    dtype = torch.float64 if vt == "f64" else torch.float32
    nnz = dm.nnz(dim)
    ref = torch.zeros(nnz, dtype=dtype, device="cuda")
    got = torch.full((nnz,), float("nan"), dtype=dtype, device="cuda")
    L = _lib.load()
    _lib.check(L.gfea_assemble_elastic(g.code, _lib.ptr(dm.coord), _lib.ptr(g.connect), g.Ne, _lib.ptr(dm.node_ptr),
                                       _lib.ptr(dm.rank), _lib.ptr(C), mode, 1.5, code, _lib.ptr(ref), nnz, 0,
                                       _lib.stream()), "atomic")
    plan, _ = dm.part_plan(dim, code)
    assert plan.n_parts > 1
    _lib.check(L.gfea_assemble_elastic_parts(g.code, _lib.ptr(dm.coord), _lib.ptr(g.connect), g.Ne,
                                             _lib.ptr(dm.node_ptr), _lib.ptr(dm.rank), _lib.ptr(C), mode, 1.5, code,
                                             _lib.ptr(got), ctypes.byref(plan), _lib.stream()), "parts")
    a, b = got.double().cpu().numpy(), ref.double().cpu().numpy()
    assert np.isfinite(a).all()  # every value written
    indptr, _ = dm.pattern(dim)
    ip = indptr.cpu().numpy()
    rows = np.repeat(np.arange(len(ip) - 1), np.diff(ip))
    rmax = np.maximum.reduceat(np.abs(b), ip[:-1])
    err = np.abs(a - b) / rmax[rows]
    # the same element blocks summed in another order (FP64), or FP32 element
    # geometry evaluated in another order
    assert err.max() <= (1e-13 if vt == "f64" else 2e-5), err.max()


@pytest.mark.parametrize("case", ["el_hexa8", "el_tetra4", "el_quad4_hetero", "el_tetra10", "el_quad8", "el_tri15",
                                  "el_prism18"])
def test_parts_assembly_matches_reference(golden, case):
    """Elastic.Assembly with the row-owned schedule: K within 1e-12 of the
    reference's (row-scaled), as the atomic schedule."""
    from easyfea_gb300 import Models
    from easyfea_gb300 import simulations as Simulations

    g = golden(case)
    m = mesh_from_golden(g)
    E = g["E"]
    mat = Models.Elastic.Isotropic(m.dim, E=float(E) if E.ndim == 0 else np.asarray(E, float), v=float(g["v"]),
                                   planeStress=bool(g["planeStress"]), thickness=float(g["thickness"]))
    simu = Simulations.Elastic(m, mat)
    simu.assembly_schedule = "parts"
    K = simu.Get_K_C_M_F()[0]
    assert row_scaled_err(K, csr(g, "K", K.shape[0])) <= 1e-12
