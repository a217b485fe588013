"""Autotuner on the GPU: tuned schedules give the same operators and
solutions as the fixed rules, and decisions are recorded per class."""

import ctypes

import numpy as np
import pytest

from helpers import mesh_from_golden, row_scaled_err

pytestmark = pytest.mark.gpu


def elastic(g, precision="mixed"):
    from easyfea_gb300 import Models
    from easyfea_gb300 import simulations as Simulations

    m = mesh_from_golden(g)
    dim = m.dim
    E = g["E"] if g["E"].ndim else float(g["E"])
    mat = Models.Elastic.Isotropic(dim, E=E, v=float(g["v"]), planeStress=bool(g["planeStress"]),
                                   thickness=float(g["thickness"]))
    simu = Simulations.Elastic(m, mat)
    simu.precision = precision
    simu.rtol = 1e-12
    unk = ["x", "y"] if dim == 2 else ["x", "y", "z"]
    simu.add_dirichlet(g["left"], [0.0] * dim, unk)
    simu.add_surfLoad(g["right"], [float(g["loadval"])], [str(g["loaddir"])])
    return simu


@pytest.mark.parametrize("case", ["el_quad4", "el_hexa8", "el_cantilever_240x26"])
def test_tuned_spmv_solution_matches(golden, case):
    from easyfea_gb300 import _lib, autotune

    g = golden(case)
    autotune.clear()
    autotune.set_mode(autotune.USE)
    simu = elastic(g)
    u0 = simu.Solve()
    lanes, ms = autotune.tune_spmv(simu.K_device, _lib.F32)
    assert lanes in (4, 8, 16, 32) and ms > 0
    assert any((k >> 32) == 1 and v == lanes for k, v in autotune.decisions().items())
    simu.Need_Update()
    u1 = simu.Solve()
    assert simu.last_solve.status == 0
    err = np.abs(u1 - g["u"]).max() / np.abs(g["u"]).max()
    assert err <= 1e-8
    assert np.abs(u1 - u0).max() <= 1e-8 * np.abs(u0).max()
    autotune.clear()


@pytest.mark.parametrize("case", ["el_quad4", "el_quad9", "el_hexa8", "el_quad4_hetero"])
def test_tuned_assembly_is_the_same_operator(golden, case):
    from easyfea_gb300 import _lib, autotune

    g = golden(case)
    autotune.clear()
    simu = elastic(g, precision="fp64")
    K0 = simu.Get_K_C_M_F()[0]
    op = simu.K_device
    dm = simu.dmesh
    gr = dm.main
    C, mode = simu._C_device()
    factor = simu.material.thickness if simu.dim == 2 else 1.0
    best, ms = ctypes.c_int32(), ctypes.c_float()
    L = _lib.load()
    _lib.check(L.gfea_tune_assemble_elastic(gr.code, _lib.ptr(dm.coord), _lib.ptr(gr.connect), gr.Ne,
                                            _lib.ptr(dm.node_ptr), _lib.ptr(dm.rank), _lib.ptr(C), int(mode), factor,
                                            _lib.F64, _lib.ptr(op.vals64), op.nnz, ctypes.byref(best),
                                            ctypes.byref(ms), _lib.stream()), "tune assembly")
    assert best.value in (4, 8, 16, 32, 64)
    K1 = op.to_scipy()
    assert row_scaled_err(K1, K0) <= 1e-14
    assert any((k >> 32) == 2 for k in autotune.decisions())
    autotune.clear()


def test_tune_on_first_use(golden):
    """Mode 2: the first assembly and solve of a class tune themselves and
    give the reference's answer."""
    from easyfea_gb300 import autotune

    g = golden("el_cantilever_240x26")
    autotune.clear()
    autotune.set_mode(autotune.TUNE)
    try:
        simu = elastic(g)
        u = simu.Solve()
        kinds = {k >> 32 for k in autotune.decisions()}
        assert kinds == {1, 2}
        assert np.abs(u - g["u"]).max() <= 1e-8 * np.abs(g["u"]).max()
    finally:
        autotune.set_mode(autotune.USE)
        autotune.clear()
