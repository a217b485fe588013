"""Solve service: continuous batching of elastic solves and phase-field load
steps on one GPU.

The reference runs one ``Simulations.*.Solve`` at a time on the host
(EasyFEA/Simulations/_simu.py, Solvers.py:361).  Here requests of different
kinds and sizes arrive over time and share the device:

* ``Server`` keeps ``workers`` host threads, each with its own CUDA stream.
  A request is admitted as soon as a worker is free and its estimated HBM
  footprint fits the remaining budget (a request that does not fit waits;
  smaller ones behind it may pass, up to ``max_bypass`` times).  Admitted
  requests run concurrently: their assembly and PCG launches interleave on
  the device, and each solve keeps its own convergence test, so a result does
  not depend on what else is running.
* Meshes (host arrays, device node graph, slot ranks) are built once per
  ``MeshSpec`` and stay resident; phase-field sessions keep their
  displacement, damage and history fields on the device between load steps.
* ``run_stream`` replays a timed arrival list (e.g. ``poisson_stream``) and
  reports per-request latency (completion - arrival).

``run_plain`` is the comparison path: the same requests one at a time through
the drop-in API on the default stream, FP64.
"""

from __future__ import annotations

import math
import queue
import threading
import time
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Tuple

import numpy as np
import torch

from . import mesh as gmesh
from .models import Elastic as ElasticModels
from .models import PhaseField as PhaseFieldModel


# ---------------------------------------------------------------------------
# meshes
# ---------------------------------------------------------------------------

@dataclass(frozen=True)
class MeshSpec:
    """An organised mesh: ``kind`` in quad4 / quad9 (cantilever L=120, h=13),
    hexa8 (box 1000 x 100 x 100), tri3_sen (1 x 1 notched plate)."""

    kind: str
    nx: int
    ny: int
    nz: int = 0

    @property
    def dim(self) -> int:
        return 3 if self.kind == "hexa8" else 2

    @property
    def n_nodes(self) -> int:
        if self.kind == "quad9":
            return (2 * self.nx + 1) * (2 * self.ny + 1)
        if self.kind == "hexa8":
            return (self.nx + 1) * (self.ny + 1) * (self.nz + 1)
        return (self.nx + 1) * (self.ny + 1)

    @property
    def dof(self) -> int:
        return self.dim * self.n_nodes

    @property
    def n_elems(self) -> int:
        e = self.nx * self.ny * (self.nz if self.kind == "hexa8" else 1)
        return 2 * e if self.kind == "tri3_sen" else e

    def build(self) -> gmesh.Mesh:
        if self.kind == "quad4":
            return gmesh.Mesh_Quad4_Rect(120.0, 13.0, self.nx, self.ny)
        if self.kind == "quad9":
            return gmesh.Mesh_Quad9_Rect(120.0, 13.0, self.nx, self.ny)
        if self.kind == "hexa8":
            return gmesh.Mesh_Hexa8_Box(1000.0, 100.0, 100.0, self.nx, self.ny, self.nz)
        if self.kind == "tri3_sen":
            return gmesh.Mesh_Tri3_Rect(1.0, 1.0, self.nx, self.ny)
        raise ValueError(self.kind)

    def footprint(self, precision: str) -> int:
        """Device bytes of a solve on this mesh (graph, values, vectors, PCG
        workspace with the packed tiles of the staged SpMV), an upper estimate
        used for admission."""
        D = self.dim
        nbr = {"quad4": 9, "quad9": 25, "hexa8": 27, "tri3_sen": 7}[self.kind]
        Nn = self.n_nodes
        pairs = Nn * nbr
        nnz = D * D * pairs
        npe = {"quad4": 4, "quad9": 9, "hexa8": 8, "tri3_sen": 3}[self.kind]
        graph = 4 * (Nn + 1) + 4 * pairs + self.n_elems * npe * (npe + 4) + 24 * Nn
        iterated = 4 if precision == "mixed" else 8
        values = nnz * (12 if precision == "mixed" else 8)
        vectors = D * Nn * 8 * 6 + D * Nn * iterated * (8 + D)
        coarse = 1536 * 1536 * 8 + 20 * Nn
        packed = int(1.2 * (nnz * iterated + 4 * pairs)) + 64 * Nn
        return graph + values + vectors + coarse + packed + (1 << 20)


def cantilever_spec(kind: str, dof: float) -> MeshSpec:
    """2D cantilever with about ``dof`` DOF and elements of aspect ~1."""
    n = dof / 2 if kind == "quad4" else dof / 8  # quad9: 4 nodes per element
    ny = max(1, int(round(math.sqrt(n * 13.0 / 120.0))))
    nx = max(1, int(round(ny * 120.0 / 13.0)))
    return MeshSpec(kind, nx, ny)


def box_spec(dof: float) -> MeshSpec:
    """3D box 10:1:1 with about ``dof`` DOF."""
    ny = max(1, int(round((dof / 3 / 10) ** (1 / 3))))
    return MeshSpec("hexa8", 10 * ny, ny, ny)


class MeshCache:
    """Host meshes and device meshes built once per spec (thread-safe)."""

    def __init__(self):
        self._lock = threading.Lock()
        self._building: Dict[MeshSpec, threading.Event] = {}
        self._meshes: Dict[MeshSpec, Tuple[gmesh.Mesh, object, dict]] = {}

    def get(self, spec: MeshSpec):
        """(mesh, device mesh, boundary node sets)."""
        from .device import DeviceMesh

        while True:
            with self._lock:
                if spec in self._meshes:
                    return self._meshes[spec]
                ev = self._building.get(spec)
                if ev is None:
                    ev = threading.Event()
                    self._building[spec] = ev
                    owner = True
                else:
                    owner = False
            if not owner:
                ev.wait()
                continue
            try:
                m = spec.build()
                dm = DeviceMesh(m)
                torch.cuda.current_stream().synchronize()  # visible to every stream
                x = m.coord
                if spec.kind == "tri3_sen":
                    nodes = {"bottom": np.where(x[:, 1] == 0)[0], "top": np.where(x[:, 1] == 1.0)[0],
                             "notch": np.where((np.abs(x[:, 1] - 0.5) < 1e-12) & (x[:, 0] <= 0.5))[0]}
                else:
                    Lx = x[:, 0].max()
                    nodes = {"left": np.where(x[:, 0] == 0)[0], "right": np.where(x[:, 0] == Lx)[0]}
                entry = (m, dm, nodes)
                with self._lock:
                    self._meshes[spec] = entry
                return entry
            finally:
                with self._lock:
                    self._building.pop(spec, None)
                ev.set()

    def prebuild(self, specs):
        for s in specs:
            self.get(s)


# ---------------------------------------------------------------------------
# requests
# ---------------------------------------------------------------------------

@dataclass
class Result:
    rid: int
    kind: str
    dof: int
    arrival: float = 0.0
    start: float = 0.0
    end: float = 0.0
    iterations: int = 0
    rel_residual: float = 0.0
    status: int = 0
    u: Optional[np.ndarray] = None
    d: Optional[np.ndarray] = None
    error: Optional[str] = None

    @property
    def latency(self) -> float:
        return self.end - self.arrival


@dataclass
class ElasticRequest:
    """Linear-elastic solve on a cached mesh: cantilever (clamped at x = 0,
    surface load -800/13^2 in y (2D) or -1 in z (3D) at x = L), E = 210000,
    nu = 0.3; an optional per-element modulus field."""

    spec: MeshSpec
    E: Optional[np.ndarray] = None
    rid: int = 0
    keep_solution: bool = True

    kind = "elastic"

    def footprint(self, precision: str) -> int:
        return self.spec.footprint(precision)


@dataclass
class PhaseFieldStep:
    """One staggered load step (damage + displacement until the damage
    converges) of a phase-field session kept on the device."""

    session: "PhaseFieldSession"
    rid: int = 0
    keep_solution: bool = True

    kind = "phasefield"

    @property
    def spec(self) -> MeshSpec:
        return self.session.spec

    def footprint(self, precision: str) -> int:
        return self.session.spec.footprint(precision) * 2


class PhaseFieldSession:
    """Single-edge-notched plate (AT2, Miehe split, plane strain, E = 210 GPa,
    nu = 0.3, Gc = 2.7, l0 = 0.01, bottom clamped, top uy += dU per step, notch
    as initial damage); state (u, d, history) stays on the device."""

    def __init__(self, spec: MeshSpec, dU: float = 1e-5, tol: float = 1e-3, max_iter: int = 500,
                 split: str = "Miehe", regu: str = "AT2"):
        assert spec.kind == "tri3_sen"
        self.spec = spec
        self.dU = dU
        self.tol = tol
        self.max_iter = max_iter
        self.split = split
        self.regu = regu
        self.step = 0
        self.simu = None
        self.lock = threading.Lock()

    def _ensure(self, cache: MeshCache, precision: str, coarse: int = -1):
        if self.simu is None:
            from .simulations import PhaseField

            m, dm, nodes = cache.get(self.spec)
            mat = ElasticModels.Isotropic(2, E=210e3, v=0.3, planeStress=False)
            pfm = PhaseFieldModel(mat, self.split, self.regu, 2.7, 0.01)
            simu = PhaseField(m, pfm)
            simu._dmesh = dm
            simu.precision = precision
            simu.rtol = 1e-10
            simu.coarse = coarse
            self.simu = simu
            self.nodes = nodes
        return self.simu

    def run_step(self, cache: MeshCache, precision: str, coarse: int = -1):
        simu = self._ensure(cache, precision, coarse)
        self.step += 1
        k = self.step
        n = self.nodes
        simu.Bc_Init()
        simu.add_dirichlet(n["notch"], [1.0], ["d"], problemType="damage")
        simu.add_dirichlet(n["bottom"], [0.0, 0.0], ["x", "y"])
        simu.add_dirichlet(n["top"], [0.0, k * self.dU], ["x", "y"])
        u, d, conv = simu.Solve(self.tol, self.max_iter, convOption=0)
        simu.Save_Iter()
        return u, d, simu.staggered_iterations


def run_elastic(req: ElasticRequest, cache: MeshCache, precision: str, rtol: float = 1e-10, coarse: int = -1):
    """Assemble and solve one elastic request on the current stream
    (``coarse``: aggregates of the two-level preconditioner, 0 = block-Jacobi)."""
    from .simulations import Elastic

    m, dm, nodes = cache.get(req.spec)
    dim = req.spec.dim
    E = req.E if req.E is not None else 210000.0
    if dim == 2:
        mat = ElasticModels.Isotropic(2, E=E, v=0.3, planeStress=True, thickness=13.0)
    else:
        mat = ElasticModels.Isotropic(3, E=E, v=0.3, planeStress=False)
    simu = Elastic(m, mat)
    simu._dmesh = dm
    simu.precision = precision
    simu.rtol = rtol
    simu.coarse = coarse
    simu.add_dirichlet(nodes["left"], [0.0] * dim, ["x", "y"] if dim == 2 else ["x", "y", "z"])
    if dim == 2:
        simu.add_surfLoad(nodes["right"], [-800 / 13**2], ["y"])
    else:
        simu.add_surfLoad(nodes["right"], [-1.0], ["z"])
    u = simu.Solve_device()
    return simu, u


# ---------------------------------------------------------------------------
# batched small solves
# ---------------------------------------------------------------------------

class _Slot:
    """Device state of one batch position on one mesh: stiffness operator
    (FP64 + FP32), load vector, Dirichlet mask and initial x, kept across
    batches so that the coarse aggregation is built once per slot."""

    def __init__(self, spec: MeshSpec, cache: MeshCache):
        from . import _lib
        from .batching import BatchSystem
        from .device import CsrOperator
        from .simulations import isotropic_lame

        m, dm, nodes = cache.get(spec)
        D = spec.dim
        self.dm = dm
        self.op = CsrOperator(dm, D, with_f32=True, translation_invariant=True)
        if D == 2:
            ref = ElasticModels.Isotropic(2, E=1.0, v=0.3, planeStress=True, thickness=13.0)
        else:
            ref = ElasticModels.Isotropic(3, E=1.0, v=0.3, planeStress=False)
        self.lame = isotropic_lame(ref.C)
        self.thickness = 13.0 if D == 2 else 1.0
        self.C_hom = torch.as_tensor(self.lame * 210000.0)
        L = _lib.load()
        b = torch.zeros(D * m.Nn, dtype=torch.float64)
        b = b.cuda()
        mask = torch.zeros(m.Nn, dtype=torch.uint8, device=b.device)
        mask[torch.as_tensor(nodes["right"], device=b.device)] = 1
        for g in dm.boundary:
            if g.dim != D - 1:
                continue
            comp, val = (1, -800 / 13**2) if D == 2 else (2, -1.0)
            _lib.check(L.gfea_surface_load(g.code, _lib.ptr(dm.coord), _lib.ptr(g.connect), g.Ne, _lib.ptr(mask), D,
                                           1, (__import__("ctypes").c_int32 * 1)(comp),
                                           (__import__("ctypes").c_double * 1)(val), self.thickness, _lib.ptr(b),
                                           _lib.stream()), "surface load")
        known = torch.zeros(D * m.Nn, dtype=torch.uint8, device=b.device)
        left = nodes["left"]
        known[torch.as_tensor(np.concatenate([D * left + c for c in range(D)]), device=b.device)] = 1
        self.C_hom = self.C_hom.to(b.device)
        self.system = BatchSystem(self.op, b, torch.zeros(D * m.Nn, dtype=torch.float64, device=b.device), known)

    def assemble(self, E: Optional[np.ndarray]):
        """K of this request (homogeneous E = 210000, or per element) in FP64 and FP32; x reset."""
        from . import _lib

        L = _lib.load()
        g = self.dm.main
        if E is None:
            C, mode = self.C_hom, 3
        else:
            C = torch.as_tensor(np.concatenate([self.lame, np.asarray(E, dtype=np.float64)]), device=self.op.vals64.device)
            mode = 4
        _lib.check(L.gfea_assemble_elastic(g.code, _lib.ptr(self.dm.coord), _lib.ptr(g.connect), g.Ne,
                                           _lib.ptr(self.dm.node_ptr), _lib.ptr(self.dm.rank), _lib.ptr(C), mode,
                                           self.thickness, _lib.F64, _lib.ptr(self.op.vals64), self.op.nnz, 0,
                                           _lib.stream()), "assemble elastic")
        _lib.check(L.gfea_cast_f64_f32(_lib.ptr(self.op.vals64), _lib.ptr(self.op.vals32), self.op.nnz,
                                       _lib.stream()), "cast")
        self.system.x.zero_()
        return C  # kept alive until the batch has run


class SmallBatcher:
    """Serves small elastic requests (at most ``max_dof`` DOF) by batching
    their PCG iterations: requests admitted within ``window_s`` of the first
    one waiting (at most ``max_batch``) are assembled on the batcher's stream
    and solved together by one persistent launch of the batched two-level PCG
    (gfea_batch_pcg), each system with its own convergence test (its cluster
    stops when its residual does), so a result does not depend on the rest of
    the batch beyond rounding."""

    def __init__(self, server: "Server", max_dof: int, window_s: float, max_batch: int):
        from .batching import BatchSolver

        self.server = server
        self.max_dof = max_dof
        self.window_s = window_s
        self.max_batch = max_batch
        self.queue: "queue.Queue" = queue.Queue()
        self.solver = BatchSolver()
        self.slots: Dict[Tuple[MeshSpec, int], _Slot] = {}
        self.batches = 0
        self.thread = threading.Thread(target=self._run, daemon=True)
        self.thread.start()

    def accepts(self, req) -> bool:
        return req.kind == "elastic" and req.spec.dof <= self.max_dof

    def _run(self):
        torch.cuda.set_device(self.server.device)
        stream = torch.cuda.Stream()
        while True:
            item = self.queue.get()
            if item is None:
                return
            items = [item]
            t_end = time.perf_counter() + self.window_s
            while len(items) < self.max_batch:
                left = t_end - time.perf_counter()
                try:
                    nxt = self.queue.get(timeout=max(left, 0.0)) if left > 0 else self.queue.get_nowait()
                except queue.Empty:
                    break
                if nxt is None:
                    self.queue.put(None)
                    break
                items.append(nxt)
            self._execute(items, stream)

    def _execute(self, items, stream):
        srv = self.server
        results = []
        start = time.perf_counter()
        try:
            with torch.cuda.stream(stream):
                count: Dict[MeshSpec, int] = {}
                systems, keep = [], []
                for req, arrival, fp in items:
                    k = count.get(req.spec, 0)
                    count[req.spec] = k + 1
                    key = (req.spec, k)
                    if key not in self.slots:
                        self.slots[key] = _Slot(req.spec, srv.cache)
                    slot = self.slots[key]
                    keep.append(slot.assemble(req.E))
                    slot.system.rtol = srv.rtol
                    systems.append(slot.system)
                infos = self.solver.solve(systems, precision="fp64" if srv.precision == "fp64" else "mixed",
                                          raise_on_fail=False)
                self.batches += 1
                for (req, arrival, fp), s, info in zip(items, systems, infos):
                    res = Result(req.rid, req.kind, req.spec.dof, arrival=arrival, start=start)
                    res.iterations, res.rel_residual, res.status = info.iterations, info.rel_residual, info.status
                    if req.keep_solution:
                        res.u = s.x.cpu().numpy()
                    results.append((res, fp))
                stream.synchronize()
        except Exception as e:  # reported per request, the server keeps running
            results = []
            for req, arrival, fp in items:
                res = Result(req.rid, req.kind, req.spec.dof, arrival=arrival, start=start)
                res.error = f"{type(e).__name__}: {e}"
                res.status = -1
                results.append((res, fp))
        end = time.perf_counter()
        with srv._cv:
            for res, fp in results:
                res.end = end
                srv.results[res.rid] = res
                srv.in_use -= fp
                srv._outstanding -= 1
            srv._cv.notify_all()

    def close(self):
        self.queue.put(None)
        self.thread.join()


# ---------------------------------------------------------------------------
# server
# ---------------------------------------------------------------------------

class Server:
    """Continuous-batching solve service (see module docstring)."""

    def __init__(self, workers: int = 8, hbm_budget: Optional[int] = None, precision: str = "mixed",
                 rtol: float = 1e-10, max_bypass: int = 8, cache: Optional[MeshCache] = None,
                 executor=None, tune: bool = True, batch_max_dof: int = 0, batch_window_s: float = 0.002,
                 batch_max: int = 64):
        """``executor(request, result)``: runs one request (default: the GPU
        path on the worker's stream); replaceable to test the scheduling.
        ``tune``: the first request of each problem class tunes the SpMV and
        element-kernel schedules (process-wide autotuner mode 2).
        ``batch_max_dof`` > 0: elastic requests up to that many DOF skip the
        workers and are solved in batches (``SmallBatcher``: one persistent
        batched PCG launch per batch, ``batch_window_s`` to gather one, at
        most ``batch_max`` requests)."""
        if executor is None and tune:
            from . import autotune

            autotune.set_mode(autotune.TUNE)
        self.precision = precision
        self.rtol = rtol
        self.cache = cache or MeshCache()
        self._executor = executor
        if hbm_budget is None:
            free, _ = torch.cuda.mem_get_info()
            hbm_budget = int(0.8 * free)
        self.budget = hbm_budget
        self.in_use = 0
        self.max_bypass = max_bypass
        self._cv = threading.Condition()
        self._pending: List[Tuple[int, object, float]] = []  # (bypassed count, request, arrival)
        self._free_workers = workers
        self._ready: "queue.Queue" = queue.Queue()
        self.results: Dict[int, Result] = {}
        self._outstanding = 0
        self._stop = False
        self.peak_in_use = 0
        self._workers = [threading.Thread(target=self._worker, args=(i,), daemon=True) for i in range(workers)]
        self._dispatcher = threading.Thread(target=self._dispatch, daemon=True)
        self.device = torch.cuda.current_device() if executor is None else None
        self.batcher = (SmallBatcher(self, batch_max_dof, batch_window_s, batch_max)
                        if batch_max_dof > 0 and executor is None else None)
        for t in self._workers:
            t.start()
        self._dispatcher.start()

    # -- submission ---------------------------------------------------------
    def submit(self, req, arrival: Optional[float] = None) -> int:
        arrival = time.perf_counter() if arrival is None else arrival
        fp = req.footprint(self.precision)
        if fp > self.budget:
            raise ValueError(f"request {req.rid} needs {fp} bytes, more than the HBM budget {self.budget}")
        with self._cv:
            self._pending.append([0, req, arrival, fp])
            self._outstanding += 1
            self._cv.notify_all()
        return req.rid

    def _dispatch(self):
        """Admit pending requests in arrival order when a worker is free and
        the footprint fits; a request that does not fit may be passed by
        smaller ones at most max_bypass times."""
        while True:
            with self._cv:
                item = None
                while not self._stop:
                    item = self._take(self._free_workers > 0)
                    if item is not None:
                        break
                    self._cv.wait(timeout=0.05)
                if self._stop:
                    return
                _, req, arrival, fp = item
                self.in_use += fp
                self.peak_in_use = max(self.peak_in_use, self.in_use)
                batched = self.batcher is not None and self.batcher.accepts(req)
                if not batched:
                    self._free_workers -= 1
            if batched:
                self.batcher.queue.put((req, arrival, fp))
            else:
                self._ready.put((req, arrival, fp))

    def _take(self, worker_free: bool = True):
        """The next admissible request in arrival order: its footprint fits,
        and a worker is free unless the batcher takes it (requests waiting for
        a worker do not hold back batched ones).  A request that does not fit
        may be passed by later ones at most max_bypass times."""
        room = self.budget - self.in_use
        for i, p in enumerate(self._pending):
            needs_worker = self.batcher is None or not self.batcher.accepts(p[1])
            if needs_worker and not worker_free:
                continue
            if p[3] <= room:
                for q in self._pending[:i]:
                    if q[3] > room:
                        q[0] += 1
                return self._pending.pop(i)
            if p[0] >= self.max_bypass:  # the head has waited long enough: hold the rest
                return None
        return None

    def _gpu_execute(self, req, res: Result, stream):
        with torch.cuda.stream(stream):
            if req.kind == "elastic":
                simu, u = run_elastic(req, self.cache, self.precision, self.rtol)
                info = simu.last_solve
                res.iterations, res.rel_residual, res.status = info.iterations, info.rel_residual, info.status
                if req.keep_solution:
                    res.u = u.cpu().numpy()
                else:
                    stream.synchronize()
            else:
                with req.session.lock:
                    u, d, niter = req.session.run_step(self.cache, self.precision)
                res.iterations = niter
                if req.keep_solution:
                    res.u, res.d = u, d

    def _worker(self, idx: int):
        stream = None
        if self._executor is None:
            torch.cuda.set_device(self.device)
            stream = torch.cuda.Stream()
        while True:
            item = self._ready.get()
            if item is None:
                return
            req, arrival, fp = item
            res = Result(req.rid, req.kind, req.spec.dof, arrival=arrival, start=time.perf_counter())
            try:
                if self._executor is None:
                    self._gpu_execute(req, res, stream)
                else:
                    self._executor(req, res)
            except Exception as e:  # reported per request, the server keeps running
                res.error = f"{type(e).__name__}: {e}"
                res.status = -1
            res.end = time.perf_counter()
            with self._cv:
                self.results[req.rid] = res
                self.in_use -= fp
                self._free_workers += 1
                self._outstanding -= 1
                self._cv.notify_all()

    def drain(self, timeout: Optional[float] = None) -> bool:
        t_end = None if timeout is None else time.perf_counter() + timeout
        with self._cv:
            while self._outstanding > 0:
                left = None if t_end is None else t_end - time.perf_counter()
                if left is not None and left <= 0:
                    return False
                self._cv.wait(timeout=left if left is not None else 0.1)
        return True

    def close(self):
        self.drain()
        with self._cv:
            self._stop = True
            self._cv.notify_all()
        for _ in self._workers:
            self._ready.put(None)
        for t in self._workers:
            t.join()
        self._dispatcher.join()
        if self.batcher is not None:
            self.batcher.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


# ---------------------------------------------------------------------------
# streams of requests
# ---------------------------------------------------------------------------

@dataclass
class StreamMix:
    """Request mix of the serving workload: 2D QUAD4 / QUAD9 elastic solves
    (1k-500k DOF), 3D HEXA8 elastic solves (10k-2M DOF) and phase-field load
    steps on notched plates of 20k-320k elements; sizes log-uniform, snapped
    to ``classes`` size classes per kind so that meshes are reused."""

    p_quad4: float = 0.35
    p_quad9: float = 0.2
    p_hexa8: float = 0.25
    p_phasefield: float = 0.2
    quad_dof: Tuple[float, float] = (1e3, 5e5)
    hexa_dof: Tuple[float, float] = (1e4, 2e6)
    pf_elems: Tuple[int, ...] = (20000, 80000, 320000)
    classes: int = 6
    extra: dict = field(default_factory=dict)


def _classes(lo: float, hi: float, n: int) -> np.ndarray:
    return np.exp(np.linspace(np.log(lo), np.log(hi), n))


def poisson_stream(rate: float, n: int, seed: int = 0, mix: Optional[StreamMix] = None,
                   sessions: Optional[List[PhaseFieldSession]] = None):
    """n requests with exponential inter-arrival times (mean 1/rate s);
    returns (arrival offsets, requests, phase-field sessions)."""
    mix = mix or StreamMix()
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, size=n))
    t -= t[0]
    if sessions is None:
        sessions = []
        for ne in mix.pf_elems:
            k = int(round(math.sqrt(ne / 2)))
            sessions.append(PhaseFieldSession(MeshSpec("tri3_sen", k, k)))
    probs = np.array([mix.p_quad4, mix.p_quad9, mix.p_hexa8, mix.p_phasefield])
    probs = probs / probs.sum()
    q_cls = _classes(*mix.quad_dof, mix.classes)
    h_cls = _classes(*mix.hexa_dof, mix.classes)
    reqs = []
    for i in range(n):
        kind = rng.choice(4, p=probs)
        if kind == 0:
            reqs.append(ElasticRequest(cantilever_spec("quad4", rng.choice(q_cls)), rid=i))
        elif kind == 1:
            reqs.append(ElasticRequest(cantilever_spec("quad9", rng.choice(q_cls)), rid=i))
        elif kind == 2:
            reqs.append(ElasticRequest(box_spec(rng.choice(h_cls)), rid=i))
        else:
            reqs.append(PhaseFieldStep(sessions[rng.integers(len(sessions))], rid=i))
    return t, reqs, sessions


def run_stream(server: Server, offsets, reqs, time_scale: float = 1.0) -> List[Result]:
    """Submit each request at its arrival offset (seconds, scaled) and wait
    for all of them; returns results in request order."""
    t0 = time.perf_counter()
    for off, r in zip(offsets, reqs):
        target = t0 + off * time_scale
        now = time.perf_counter()
        if target > now:
            time.sleep(target - now)
        server.submit(r, arrival=target)
    server.drain()
    return [server.results[r.rid] for r in reqs]


def run_plain(reqs, cache: MeshCache, offsets=None, precision: str = "fp64", rtol: float = 1e-10,
              time_scale: float = 1.0, coarse: int = -1) -> List[Result]:
    """One request at a time on the default stream (the plain GPU path); with
    ``offsets`` a request starts no earlier than its arrival; ``coarse = 0``
    solves with block-Jacobi PCG alone."""
    out = []
    t0 = time.perf_counter()
    for i, r in enumerate(reqs):
        arrival = t0 + (offsets[i] * time_scale if offsets is not None else 0.0)
        now = time.perf_counter()
        if arrival > now:
            time.sleep(arrival - now)
        res = Result(r.rid, r.kind, r.spec.dof, arrival=arrival, start=time.perf_counter())
        if r.kind == "elastic":
            simu, u = run_elastic(r, cache, precision, rtol, coarse)
            info = simu.last_solve
            res.iterations, res.rel_residual, res.status = info.iterations, info.rel_residual, info.status
            res.u = u.cpu().numpy() if r.keep_solution else None
            torch.cuda.synchronize()
        else:
            u, d, niter = r.session.run_step(cache, precision, coarse)
            res.iterations = niter
            res.u, res.d = (u, d) if r.keep_solution else (None, None)
        res.end = time.perf_counter()
        out.append(res)
    return out


def latency_summary(results: List[Result]) -> dict:
    lat = np.array([r.latency for r in results]) * 1e3
    span = max(r.end for r in results) - min(r.arrival for r in results)
    return {"n": len(results), "solves_per_s": len(results) / span, "p50_ms": float(np.percentile(lat, 50)),
            "p99_ms": float(np.percentile(lat, 99)), "mean_ms": float(lat.mean()),
            "errors": sum(1 for r in results if r.error)}
