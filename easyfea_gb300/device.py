"""Device-resident mesh, sparsity pattern and CSR operators.

Host runtime around libgb300fea.so: PyTorch provides device memory and the
stream; every computation is a call into the C ABI.

``DeviceMesh``   coordinates + connectivity on the GPU, node graph and element
                 slot ranks built once per mesh (replaces the cached
                 ``__Get_csr_map`` of EasyFEA/Simulations/_simu.py:1062-1102).
``CsrOperator``  CSR values (FP64 and optionally FP32) over the node graph
                 for dof_n components per node; exports a scipy CSR identical
                 in layout to the reference's.
``pcg``          masked block-Jacobi PCG (FP64, or FP32 + FP64 refinement).
"""

from __future__ import annotations

import ctypes
import threading
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from .mesh import ELEM_INFO, ElemType, Mesh


def _dev():
    return torch.device("cuda", torch.cuda.current_device())


class DeviceGroup:
    """One element group on the device (coord shared with the mesh)."""

    def __init__(self, group, coord_d):
        self.elemType = group.elemType
        self.code = _lib.ELEM_CODE[group.elemType.value]
        self.nPe = group.nPe
        self.dim = group.dim
        self.Ne = group.Ne
        self.connect = torch.as_tensor(np.ascontiguousarray(group.connect, dtype=np.int32), device=_dev())
        self.coord = coord_d


# values of one part of the row-owned assembly: 76 KiB of shared memory in
# either value type (two blocks per SM with their scratch)
PART_VALUES = {_lib.F32: 19456, _lib.F64: 9728}


def part_plan_host(coord: np.ndarray, connect: np.ndarray, node_ptr: np.ndarray, dof_n: int, max_values: int):
    """The row-owned assembly's plan (gfea_part_plan_host) as host arrays:
    dict of node_off, part_node_ptr, part_nodes, part_nvals, visit_ptr,
    visit_elem, visit_mask."""
    coord = np.ascontiguousarray(coord, dtype=np.float64)
    connect = np.ascontiguousarray(connect, dtype=np.int32)
    node_ptr = np.ascontiguousarray(node_ptr, dtype=np.int32)
    Nn = coord.shape[0]
    Ne, nPe = connect.shape
    out = {"node_off": np.empty(Nn, np.int32), "part_node_ptr": np.empty(Nn + 1, np.int32),
           "part_nodes": np.empty(Nn, np.int32), "part_nvals": np.empty(Nn, np.int32),
           "visit_ptr": np.empty(Nn + 1, np.int32), "visit_elem": np.empty(Ne * nPe, np.int32),
           "visit_mask": np.empty(Ne * nPe, np.uint32)}
    n_parts = ctypes.c_int32()
    n_visits = ctypes.c_int64()
    h = lambda a: a.ctypes.data  # noqa: E731
    _lib.check(_lib.load().gfea_part_plan_host(h(coord), h(connect), Ne, nPe, Nn, h(node_ptr), dof_n, int(max_values),
                                               h(out["node_off"]), h(out["part_node_ptr"]), h(out["part_nodes"]),
                                               h(out["part_nvals"]), h(out["visit_ptr"]), h(out["visit_elem"]),
                                               h(out["visit_mask"]), ctypes.byref(n_parts), ctypes.byref(n_visits)),
               "part plan")
    P, V = n_parts.value, n_visits.value
    for k in ("part_node_ptr", "visit_ptr"):
        out[k] = out[k][:P + 1]
    out["part_nvals"] = out["part_nvals"][:P]
    out["visit_elem"] = out["visit_elem"][:V]
    out["visit_mask"] = out["visit_mask"][:V]
    return out


class DeviceMesh:
    """Mesh arrays on the GPU plus the node graph of the main element group."""

    def __init__(self, mesh: Mesh):
        _lib.require_gpu()
        self.mesh = mesh
        self.Nn = mesh.Nn
        self.dim = mesh.dim
        self.coord = torch.as_tensor(np.ascontiguousarray(mesh.coord, dtype=np.float64), device=_dev())
        self.main = DeviceGroup(mesh.groupElem, self.coord)
        self.boundary = [DeviceGroup(g, self.coord) for g in mesh.Get_list_groupElem(mesh.dim - 1)]
        self._build_graph()
        self._patterns = {}

    def _build_graph(self):
        L = _lib.load()
        g = self.main
        ws = ctypes.c_size_t()
        _lib.check(L.gfea_graph_workspace_size(self.Nn, g.Ne, g.nPe, ctypes.byref(ws)), "graph workspace")
        work = torch.empty(int(ws.value), dtype=torch.uint8, device=_dev())
        self.node_ptr = torch.empty(self.Nn + 1, dtype=torch.int32, device=_dev())
        npairs = ctypes.c_int64()
        s = _lib.stream()
        _lib.check(L.gfea_graph_count(_lib.ptr(g.connect), g.Ne, g.nPe, self.Nn, _lib.ptr(self.node_ptr),
                                      ctypes.byref(npairs), _lib.ptr(work), work.numel(), s), "graph count")
        self.n_pairs = int(npairs.value)
        self.nbr = torch.empty(self.n_pairs, dtype=torch.int32, device=_dev())
        self.rank = torch.empty(g.Ne * g.nPe * g.nPe, dtype=torch.uint8, device=_dev())
        _lib.check(L.gfea_graph_fill(_lib.ptr(g.connect), g.Ne, g.nPe, self.Nn, _lib.ptr(self.node_ptr),
                                     _lib.ptr(self.nbr), _lib.ptr(self.rank), _lib.ptr(work), work.numel(), s),
                   "graph fill")

    def nnz(self, dof_n: int) -> int:
        return dof_n * dof_n * self.n_pairs

    def part_plan(self, dof_n: int, value_type: int, max_values: int | None = None, threads: int = 0):
        """The row-owned assembly's plan on the device (built once per dof_n,
        value type and part size; ``threads`` per block, 0 for the default):
        (gfea_part_plan struct, its tensors)."""
        mv = int(max_values or PART_VALUES[value_type])
        key = ("parts", dof_n, value_type, mv, threads)
        if key not in self._patterns:
            h = part_plan_host(self.mesh.coord, self.mesh.groupElem.connect, self.node_ptr.cpu().numpy(), dof_n, mv)
            t = {k: torch.as_tensor(v.view(np.int32) if v.dtype == np.uint32 else v, device=_dev())
                 for k, v in h.items()}
            plan = _lib.PartPlan(_lib.ABI_VERSION, len(h["part_nvals"]), mv, int(threads), _lib.ptr(t["node_off"]),
                                 _lib.ptr(t["part_node_ptr"]), _lib.ptr(t["part_nodes"]), _lib.ptr(t["part_nvals"]),
                                 _lib.ptr(t["visit_ptr"]), _lib.ptr(t["visit_elem"]), _lib.ptr(t["visit_mask"]))
            self._patterns[key] = (plan, t)
        return self._patterns[key]

    def incidence(self):
        """(inc_ptr, inc_list) int32 device tensors: each node's elements of the
        main group, ascending (built once)."""
        if getattr(self, "_incidence", None) is None:
            L = _lib.load()
            g = self.main
            ws = ctypes.c_size_t()
            _lib.check(L.gfea_graph_workspace_size(self.Nn, g.Ne, g.nPe, ctypes.byref(ws)), "graph workspace")
            work = torch.empty(int(ws.value), dtype=torch.uint8, device=_dev())
            inc_ptr = torch.empty(self.Nn + 1, dtype=torch.int32, device=_dev())
            inc_list = torch.empty(g.Ne * g.nPe, dtype=torch.int32, device=_dev())
            _lib.check(L.gfea_node_incidence(_lib.ptr(g.connect), g.Ne, g.nPe, self.Nn, _lib.ptr(inc_ptr),
                                             _lib.ptr(inc_list), _lib.ptr(work), work.numel(), _lib.stream()),
                       "node incidence")
            self._incidence = (inc_ptr, inc_list)
        return self._incidence

    def node_values(self, values_e: torch.Tensor) -> torch.Tensor:
        """Mean of element values (Ne,) or (Ne, k) around each node, on the
        device (Mesh.Get_Node_Values)."""
        ve = values_e.contiguous()
        k = 1 if ve.dim() == 1 else ve.shape[1]
        out = torch.empty((self.Nn,) if ve.dim() == 1 else (self.Nn, k), dtype=torch.float64, device=_dev())
        inc_ptr, inc_list = self.incidence()
        _lib.check(_lib.load().gfea_node_average(_lib.ptr(inc_ptr), _lib.ptr(inc_list), self.Nn, _lib.ptr(ve), k,
                                                 _lib.ptr(out), _lib.stream()), "node average")
        return out

    def pattern(self, dof_n: int):
        """(indptr int64, indices int32) device tensors of the dof_n CSR pattern."""
        if dof_n not in self._patterns:
            L = _lib.load()
            indptr = torch.empty(self.Nn * dof_n + 1, dtype=torch.int64, device=_dev())
            indices = torch.empty(self.nnz(dof_n), dtype=torch.int32, device=_dev())
            _lib.check(L.gfea_csr_pattern(_lib.ptr(self.node_ptr), _lib.ptr(self.nbr), self.Nn, dof_n,
                                          _lib.ptr(indptr), _lib.ptr(indices), _lib.stream()), "csr pattern")
            self._patterns[dof_n] = (indptr, indices)
        return self._patterns[dof_n]


class CsrOperator:
    """CSR values on the node graph of a DeviceMesh (dof_n components/node)."""

    def __init__(self, dmesh: DeviceMesh, dof_n: int, with_f32: bool = False,
                 translation_invariant: bool = False):
        """``translation_invariant``: node block rows sum to zero (elastic
        stiffness); lets the FP32 products use the difference form."""
        self.dmesh = dmesh
        self.dof_n = dof_n
        self.translation_invariant = translation_invariant
        self.N = dmesh.Nn * dof_n
        self.nnz = dmesh.nnz(dof_n)
        self.vals64 = torch.zeros(self.nnz, dtype=torch.float64, device=_dev())
        self.vals32 = torch.zeros(self.nnz, dtype=torch.float32, device=_dev()) if with_f32 else None

    def ensure_f32(self):
        if self.vals32 is None:
            self.vals32 = torch.empty(self.nnz, dtype=torch.float32, device=_dev())
        _lib.check(_lib.load().gfea_cast_f64_f32(_lib.ptr(self.vals64), _lib.ptr(self.vals32), self.nnz,
                                                  _lib.stream()), "cast f64->f32")
        return self.vals32

    def system(self, known: torch.Tensor | None) -> _lib.System:
        d = self.dmesh
        return _lib.System(_lib.ABI_VERSION, self.dof_n, d.Nn, d.n_pairs, _lib.ptr(d.node_ptr), _lib.ptr(d.nbr),
                           _lib.ptr(self.vals64), _lib.ptr(self.vals32), _lib.ptr(known),
                           int(self.translation_invariant), 0, _lib.ptr(d.coord))

    def matvec(self, x: torch.Tensor) -> torch.Tensor:
        y = torch.empty_like(x)
        sys = self.system(None)
        vt = _lib.F64 if x.dtype == torch.float64 else _lib.F32
        _lib.check(_lib.load().gfea_spmv(ctypes.byref(sys), vt, _lib.ptr(x), _lib.ptr(y), _lib.stream()), "spmv")
        return y

    def to_scipy(self):
        """scipy CSR with the reference's canonical pattern (host copy)."""
        import scipy.sparse as sp

        indptr, indices = self.dmesh.pattern(self.dof_n)
        ip = indptr.cpu().numpy()
        idx_dtype = np.int32 if self.nnz < 2**31 else np.int64
        A = sp.csr_matrix((self.vals64.cpu().numpy(), indices.cpu().numpy().astype(idx_dtype),
                           ip.astype(idx_dtype)), shape=(self.N, self.N))
        A.has_sorted_indices = True
        A.has_canonical_format = True
        return A


@dataclass
class PcgInfo:
    status: int
    iterations: int
    refinements: int
    rel_residual: float
    floor_rel: float = 0.0


def pcg(op: CsrOperator, b: torch.Tensor, x: torch.Tensor, known: torch.Tensor, rtol: float = 1e-12,
        precision: str = "fp64", max_iters: int = 200000, check_every: int = 0, inner_rtol: float = 0.0,
        lanes: int = 0, raise_on_fail: bool = True, coarse: int = 0, workspace: "Workspace | None" = None
        ) -> PcgInfo:
    """Solve the Dirichlet-reduced system in place: x holds the known values on
    known DOFs and the initial guess elsewhere; on return, the solution.

    ``coarse``: aggregates of the two-level preconditioner's coarse level
    (0: block-Jacobi only, -1: chosen from the mesh size).  ``workspace``: a
    ``Workspace`` owned by the caller for solves on one mesh, which keeps the
    coarse aggregation between solves (otherwise a shared scratch buffer)."""
    L = _lib.load()
    prec = _lib.F64 if precision == "fp64" else _lib.F32
    if prec == _lib.F32:
        op.ensure_f32()
    sys = op.system(known)
    key = (id(op.dmesh), op.dmesh.Nn, op.dof_n, prec, int(coarse))
    reuse = int(workspace is not None and coarse != 0 and workspace.key == key)
    opts = _lib.PcgOpts(_lib.ABI_VERSION, prec, int(max_iters), int(check_every), float(rtol), float(inner_rtol),
                        30, int(lanes), int(coarse), reuse)
    ws = ctypes.c_size_t()
    _lib.check(L.gfea_pcg_workspace_size(ctypes.byref(sys), ctypes.byref(opts), ctypes.byref(ws)), "pcg workspace")
    if workspace is None:
        work = _workspace(int(ws.value))
    else:
        work = workspace.buffer(int(ws.value))
        if work is not workspace.last:
            opts.coarse_reuse = 0
        workspace.key = None
    res = _lib.PcgResult()
    st = L.gfea_pcg_solve(ctypes.byref(sys), _lib.ptr(b), _lib.ptr(x), ctypes.byref(opts), _lib.ptr(work),
                          work.numel(), ctypes.byref(res), _lib.stream())
    info = PcgInfo(int(res.status), int(res.iterations), int(res.refinements), float(res.rel_residual),
                   float(res.floor_rel))
    if workspace is not None and st in (_lib.OK, _lib.ERR_NOT_CONVERGED):
        workspace.key = key
        workspace.last = work
    if raise_on_fail:
        _lib.check(st, f"pcg (iterations {info.iterations}, rel residual {info.rel_residual:.3e})")
    return info


class Workspace:
    """Device scratch of the solves on one mesh; it keeps the coarse
    aggregation of the two-level preconditioner from one solve to the next."""

    def __init__(self):
        self.t = None
        self.key = None
        self.last = None

    def buffer(self, nbytes: int) -> torch.Tensor:
        if self.t is None or self.t.numel() < nbytes:
            self.t = torch.empty(max(nbytes, 1 << 20), dtype=torch.uint8, device=_dev())
            self.key = None
        return self.t


# shared scratch, one per device and host thread (solves on several threads,
# each with its own stream, run concurrently)
_TLS = threading.local()


def _per_thread(name: str) -> dict:
    d = getattr(_TLS, name, None)
    if d is None:
        d = {}
        setattr(_TLS, name, d)
    return d


def _workspace(nbytes: int) -> torch.Tensor:
    """Reusable scratch buffer (grown on demand)."""
    ws = _per_thread("ws")
    dev = torch.cuda.current_device()
    w = ws.get(dev)
    if w is None or w.numel() < nbytes:
        w = torch.empty(max(nbytes, 1 << 20), dtype=torch.uint8, device=_dev())
        ws[dev] = w
    return w


def reaction_energy(op: CsrOperator, x: torch.Tensor, dofs: torch.Tensor | None):
    """(sum (A x)[dofs], 1/2 x.A x, A x) on the device."""
    L = _lib.load()
    sys = op.system(None)
    Ax = torch.empty_like(x)
    out = (ctypes.c_double * 2)()
    work = _scratch_reduce()
    n = 0 if dofs is None else dofs.numel()
    _lib.check(L.gfea_reaction_energy(ctypes.byref(sys), _lib.ptr(x), _lib.ptr(dofs), n, _lib.ptr(Ax), out,
                                      _lib.ptr(work), _lib.stream()), "reaction")
    return out[0], out[1], Ax


def _scratch_reduce() -> torch.Tensor:
    red = _per_thread("red")
    dev = torch.cuda.current_device()
    if dev not in red:
        n = int(_lib.load().gfea_reduce_workspace_size())
        red[dev] = torch.empty(n, dtype=torch.uint8, device=_dev())
    return red[dev]


def max_abs_diff(a: torch.Tensor, b: torch.Tensor) -> float:
    out = ctypes.c_double()
    work = _scratch_reduce()
    _lib.check(_lib.load().gfea_max_abs_diff(_lib.ptr(a), _lib.ptr(b), a.numel(), ctypes.byref(out),
                                               _lib.ptr(work), _lib.stream()), "max_abs_diff")
    return float(out.value)
