"""The allocation-free PCG entry point (gfea_pcg_solve_noalloc).

It serves callers that cannot allocate device memory (an embedding
application owns it, or allocation is not allowed in their loop): its
scratch is a static array inside the library.  Called through the C ABI, it
must give the same solution as gfea_pcg_solve with a caller workspace, on two
calls in a row (the second reuses the array with the first call's contents),
and reject a problem larger than the array without touching the device.

This file is collected last so that a run stopping at the first failure has
run every other test first; it builds everything it uses itself.
"""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _problem():
    import torch

    from easyfea_gb300 import Models, _lib
    from easyfea_gb300 import mesh as gmesh
    from easyfea_gb300.device import CsrOperator, DeviceMesh

    L = _lib.load()
    m = gmesh.Mesh_Quad4_Rect(120.0, 13.0, 48, 8)
    dm = DeviceMesh(m)
    op = CsrOperator(dm, 2, translation_invariant=True)
    C = torch.as_tensor(Models.Elastic.Isotropic(2, E=210000.0, v=0.3, planeStress=True, thickness=13.0).C,
                        device="cuda")
    g = dm.main
    _lib.check(L.gfea_assemble_elastic(g.code, _lib.ptr(dm.coord), _lib.ptr(g.connect), g.Ne, _lib.ptr(dm.node_ptr),
                                       _lib.ptr(dm.rank), _lib.ptr(C), 0, 13.0, _lib.F64, _lib.ptr(op.vals64),
                                       op.nnz, 0, _lib.stream()), "assemble")
    N = 2 * m.Nn
    b = torch.zeros(N, dtype=torch.float64, device="cuda")
    right = m.Nodes_Conditions(lambda x, y, z: x == 120.0)
    mask = torch.zeros(m.Nn, dtype=torch.uint8, device="cuda")
    mask[torch.as_tensor(right, device="cuda")] = 1
    seg = dm.boundary[0]
    _lib.check(L.gfea_surface_load(seg.code, _lib.ptr(dm.coord), _lib.ptr(seg.connect), seg.Ne, _lib.ptr(mask), 2, 1,
                                   (ctypes.c_int32 * 1)(1), (ctypes.c_double * 1)(-800 / 13**2), 13.0, _lib.ptr(b),
                                   _lib.stream()), "load")
    known = torch.zeros(N, dtype=torch.uint8, device="cuda")
    left = m.Nodes_Conditions(lambda x, y, z: x == 0)
    known[torch.as_tensor(np.concatenate([2 * left, 2 * left + 1]), device="cuda")] = 1
    return L, op, b, known, N


def _opts(precision):
    from easyfea_gb300 import _lib

    return _lib.PcgOpts(_lib.ABI_VERSION, precision, 200000, 64, 1e-12, 1e-4, 200, 0)


@pytest.mark.parametrize("precision", [0, 1])
def test_noalloc_matches_workspace_solver_on_two_calls(precision):
    import torch

    from easyfea_gb300 import _lib

    L, op, b, known, N = _problem()
    if precision == _lib.F32:
        op.ensure_f32()
    sys_ = op.system(known)
    opts = _opts(precision)
    # reference: the same solve with a caller-allocated workspace
    ws = ctypes.c_size_t()
    _lib.check(L.gfea_pcg_workspace_size(ctypes.byref(sys_), ctypes.byref(opts), ctypes.byref(ws)), "ws")
    work = torch.empty(ws.value, dtype=torch.uint8, device="cuda")
    x_ref = torch.zeros(N, dtype=torch.float64, device="cuda")
    res = _lib.PcgResult()
    _lib.check(L.gfea_pcg_solve(ctypes.byref(sys_), _lib.ptr(b), _lib.ptr(x_ref), ctypes.byref(opts), _lib.ptr(work),
                                ws.value, ctypes.byref(res), _lib.stream()), "pcg")
    ref = x_ref.cpu().numpy()
    scale = np.abs(ref).max()
    assert scale > 0
    for call in range(2):
        x = torch.zeros(N, dtype=torch.float64, device="cuda")
        r2 = _lib.PcgResult()
        st = L.gfea_pcg_solve_noalloc(ctypes.byref(sys_), _lib.ptr(b), _lib.ptr(x), ctypes.byref(opts),
                                      ctypes.byref(r2), _lib.stream())
        assert st == 0, f"call {call}: status {st}"
        err = np.abs(x.cpu().numpy() - ref).max() / scale
        assert err <= 1e-12, f"call {call}: relative difference {err:.3e}"
        assert r2.rel_residual <= max(1e-12, r2.floor_rel)


def test_noalloc_rejects_problem_beyond_static_scratch():
    import torch

    from easyfea_gb300 import _lib

    L = _lib.load()
    t = torch.zeros(16, dtype=torch.float64, device="cuda")
    k = torch.zeros(16, dtype=torch.uint8, device="cuda")
    i = torch.zeros(16, dtype=torch.int32, device="cuda")
    # 2M DOF in 3D needs ~160 MB of scratch: rejected before any device work
    sys_ = _lib.System(_lib.ABI_VERSION, 3, 674081, 17583841, _lib.ptr(i), _lib.ptr(i), _lib.ptr(t), 0,
                       _lib.ptr(k), 1, 0)
    res = _lib.PcgResult()
    st = L.gfea_pcg_solve_noalloc(ctypes.byref(sys_), _lib.ptr(t), _lib.ptr(t), ctypes.byref(_opts(0)),
                                  ctypes.byref(res), _lib.stream())
    assert st == 8  # GFEA_ERR_WORKSPACE
    assert L.gfea_status_string(st) == b"workspace too small"
