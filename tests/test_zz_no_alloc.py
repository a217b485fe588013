"""The allocation-free PCG entry point (gfea_pcg_solve_noalloc).

It serves callers that cannot allocate device memory (an embedding
application owns it, or allocation is not allowed in their loop): its
scratch is a static array inside the library, and it launches its kernels
directly, so it instantiates no CUDA graph and creates no stream or event.
Called through the C ABI, it must give the same solution as gfea_pcg_solve
with a caller workspace, on two calls in a row (the second reuses the array
with the first call's contents), leave the library's graph counter
unchanged, and reject a problem larger than the array without touching the
device.

This file is collected last so that a run stopping at the first failure has
run every other test first; it builds everything it uses itself.
"""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _problem(kind):
    """Assembled stiffness, load and Dirichlet mask of a clamped cantilever:
    'quad4' 2D plane stress 48x8, 'hexa8' 3D box 24x4x4, 'hexa8_limit' a 3D
    box of 204,828 DOF (just under the array's FP64 block-Jacobi limit)."""
    import torch

    from easyfea_gb300 import Models, _lib
    from easyfea_gb300 import mesh as gmesh
    from easyfea_gb300.device import CsrOperator, DeviceMesh

    L = _lib.load()
    if kind == "quad4":
        m = gmesh.Mesh_Quad4_Rect(120.0, 13.0, 48, 8)
        dim, t, Lx, load, comp = 2, 13.0, 120.0, -800 / 13**2, 1
        C = Models.Elastic.Isotropic(2, E=210000.0, v=0.3, planeStress=True, thickness=t).C
    else:
        n = (24, 4, 4) if kind == "hexa8" else (100, 25, 25)
        m = gmesh.Mesh_Hexa8_Box(1000.0, 100.0, 100.0, *n)
        dim, t, Lx, load, comp = 3, 1.0, 1000.0, -1.0, 2
        C = Models.Elastic.Isotropic(3, E=210000.0, v=0.3, planeStress=False).C
    dm = DeviceMesh(m)
    op = CsrOperator(dm, dim, translation_invariant=True)
    Cd = torch.as_tensor(C, device="cuda")
    g = dm.main
    _lib.check(L.gfea_assemble_elastic(g.code, _lib.ptr(dm.coord), _lib.ptr(g.connect), g.Ne, _lib.ptr(dm.node_ptr),
                                       _lib.ptr(dm.rank), _lib.ptr(Cd), 0, t, _lib.F64, _lib.ptr(op.vals64),
                                       op.nnz, 0, _lib.stream()), "assemble")
    N = dim * m.Nn
    b = torch.zeros(N, dtype=torch.float64, device="cuda")
    right = m.Nodes_Conditions(lambda x, y, z: x == Lx)
    mask = torch.zeros(m.Nn, dtype=torch.uint8, device="cuda")
    mask[torch.as_tensor(right, device="cuda")] = 1
    seg = dm.boundary[0]
    _lib.check(L.gfea_surface_load(seg.code, _lib.ptr(dm.coord), _lib.ptr(seg.connect), seg.Ne, _lib.ptr(mask), dim,
                                   1, (ctypes.c_int32 * 1)(comp), (ctypes.c_double * 1)(load), t, _lib.ptr(b),
                                   _lib.stream()), "load")
    known = torch.zeros(N, dtype=torch.uint8, device="cuda")
    left = m.Nodes_Conditions(lambda x, y, z: x == 0)
    known[torch.as_tensor(np.concatenate([dim * left + c for c in range(dim)]), device="cuda")] = 1
    return L, op, b, known, N


def _opts(precision, coarse=0, reuse=0):
    from easyfea_gb300 import _lib

    return _lib.PcgOpts(_lib.ABI_VERSION, precision, 200000, 64, 1e-12, 1e-4, 200, 0, coarse, reuse)


def _solve_both(kind, precision, coarse, tol):
    import torch

    from easyfea_gb300 import _lib

    L, op, b, known, N = _problem(kind)
    if precision == _lib.F32:
        op.ensure_f32()
    sys_ = op.system(known)
    opts = _opts(precision, coarse)
    # coarse_reuse = 1 on purpose: the allocation-free solve ignores it
    opts_na = _opts(precision, coarse, 1)
    # reference: the same solve with a caller-allocated workspace
    ws = ctypes.c_size_t()
    _lib.check(L.gfea_pcg_workspace_size(ctypes.byref(sys_), ctypes.byref(opts), ctypes.byref(ws)), "ws")
    work = torch.empty(ws.value, dtype=torch.uint8, device="cuda")
    x_ref = torch.zeros(N, dtype=torch.float64, device="cuda")
    res = _lib.PcgResult()
    _lib.check(L.gfea_pcg_solve(ctypes.byref(sys_), _lib.ptr(b), _lib.ptr(x_ref), ctypes.byref(opts), _lib.ptr(work),
                                ws.value, ctypes.byref(res), _lib.stream()), "pcg")
    torch.cuda.synchronize()
    del work
    ref = x_ref.cpu().numpy()
    scale = np.abs(ref).max()
    assert scale > 0
    graphs0 = L.gfea_cuda_graph_count()
    for call in range(2):
        x = torch.zeros(N, dtype=torch.float64, device="cuda")
        r2 = _lib.PcgResult()
        st = L.gfea_pcg_solve_noalloc(ctypes.byref(sys_), _lib.ptr(b), _lib.ptr(x), ctypes.byref(opts_na),
                                      ctypes.byref(r2), _lib.stream())
        assert st == 0, f"call {call}: status {st}"
        err = np.abs(x.cpu().numpy() - ref).max() / scale
        assert err <= tol, f"call {call}: relative difference {err:.3e}"
        assert r2.rel_residual <= max(1e-12, r2.floor_rel)
    assert L.gfea_cuda_graph_count() == graphs0, "the allocation-free solve instantiated a CUDA graph"


@pytest.mark.parametrize("precision", [0, 1])
def test_noalloc_matches_workspace_solver_on_two_calls(precision):
    # same kernels in the same order, fixed-order reductions
    _solve_both("quad4", precision, 0, 1e-12)


@pytest.mark.parametrize("precision", [0, 1])
def test_noalloc_two_level_3d(precision):
    """The coarse level (aggregates, float-float inverse) inside the array.
    Its restriction sums with FP64 atomics, so the two solves agree within the
    displacement tolerance of the parity tests rather than bit for bit."""
    _solve_both("hexa8", precision, -1, 1e-8)


def test_noalloc_near_size_limit():
    """204,828 DOF in 3D, FP64 block-Jacobi: just under the 16 MiB array."""
    # the workspace solve may stage its SpMV (another summation order)
    _solve_both("hexa8_limit", 0, 0, 1e-8)


def test_graph_counter_moves_for_workspace_solve():
    """Control: the counter the tests above rely on does count the graphs of
    a workspace solve running alone (unless graphs are switched off)."""
    import os

    import torch

    from easyfea_gb300 import _lib

    if os.environ.get("GFEA_PCG_GRAPHS", "1").startswith("0"):
        pytest.skip("graphs switched off")
    L, op, b, known, N = _problem("quad4")
    sys_ = op.system(known)
    opts = _opts(0, 0)
    ws = ctypes.c_size_t()
    _lib.check(L.gfea_pcg_workspace_size(ctypes.byref(sys_), ctypes.byref(opts), ctypes.byref(ws)), "ws")
    work = torch.empty(ws.value, dtype=torch.uint8, device="cuda")
    x = torch.zeros(N, dtype=torch.float64, device="cuda")
    g0 = L.gfea_cuda_graph_count()
    res = _lib.PcgResult()
    _lib.check(L.gfea_pcg_solve(ctypes.byref(sys_), _lib.ptr(b), _lib.ptr(x), ctypes.byref(opts), _lib.ptr(work),
                                ws.value, ctypes.byref(res), _lib.stream()), "pcg")
    assert L.gfea_cuda_graph_count() > g0


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
