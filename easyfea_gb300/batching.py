"""Batched solves: many independent systems assembled and solved together.

The reference solves instances one after another (one ``Simulations.*.Solve``
and one SuperLU factorisation each, EasyFEA/Simulations/Solvers.py:361).
Here a batch of Dirichlet-reduced systems of any sizes goes to
``gfea_batch_pcg``: one persistent launch in which each thread-block cluster
solves one system at a time (largest first), with per-system scalars and
convergence, so a system's result does not depend on the rest of the batch.

``random_material_cantilevers`` builds the random-material workload: 2D
plane-stress cantilevers (the L = 120, h = 13 bar) with sizes drawn
log-uniform in DOF and a per-element Young's modulus
E_e = 210000 exp(0.3 g(x_e)), g a zero-mean, unit-variance Gaussian field from
64 random Fourier features (Rahimi & Recht 2007) with correlation length
0.1 L, evaluated at element centroids.
"""

from __future__ import annotations

import ctypes
from dataclasses import dataclass
from typing import List, Optional

import numpy as np
import torch

from . import _lib
from .device import CsrOperator, PcgInfo


def _dev():
    return torch.device("cuda", torch.cuda.current_device())


@dataclass
class BatchSystem:
    """One Dirichlet-reduced system: x holds the known values (and the initial
    guess) on entry and the solution on exit."""

    op: CsrOperator
    b: torch.Tensor
    x: torch.Tensor
    known: torch.Tensor
    rtol: float = 1e-10
    max_iters: int = 200000


RESULT_BYTES = ctypes.sizeof(_lib.PcgResult)


class CoarseLevels:
    """Coarse levels of the batched two-level preconditioner, one workspace
    per system operator, kept between batches: the aggregation (which depends
    only on the mesh) is built on a system's first sight; afterwards the
    coarse matrices and inverses of a whole batch are rebuilt from the current
    values by ``build`` -- device work only, one launch per stage for all
    systems, so that it can be captured in a CUDA graph."""

    def __init__(self):
        self._levels = {}  # id(op) -> (op, precision, workspace, CoarseLevel)
        self._scratch = None
        self._n = 0

    def level(self, s: BatchSystem, precision: int, coarse: int = -1) -> _lib.CoarseLevel:
        """The system's level; its first call builds the aggregation (and a first matrix)."""
        L = _lib.load()
        key = id(s.op)
        entry = self._levels.get(key)
        if entry is None or entry[0] is not s.op or entry[1] != precision:
            sys_ = s.op.system(s.known)
            opts = _lib.PcgOpts(_lib.ABI_VERSION, precision, 0, 0, 0.0, 0.0, 0, 0, int(coarse), 0)
            nb = ctypes.c_size_t()
            _lib.check(L.gfea_coarse_workspace_size(ctypes.byref(sys_), ctypes.byref(opts), ctypes.byref(nb)),
                       "coarse workspace")
            work = torch.empty(max(int(nb.value), 256), dtype=torch.uint8, device=_dev())
            level = _lib.CoarseLevel()
            _lib.check(L.gfea_coarse_setup(ctypes.byref(sys_), ctypes.byref(opts), 0, _lib.ptr(work), work.numel(),
                                           ctypes.byref(level), _lib.stream()), "coarse setup")
            entry = (s.op, precision, work, level)
            self._levels[key] = entry
        return entry[3]

    def prepare(self, systems: List[BatchSystem], precision: int, coarse: int = -1):
        """Levels of every system and the descriptors of the batched rebuild."""
        L = _lib.load()
        order = sorted(range(len(systems)), key=lambda i: systems[i].op.dof_n)
        n = len(order)
        sys_arr = (_lib.System * max(n, 1))()
        works = (ctypes.c_void_p * max(n, 1))()
        lvls = (_lib.CoarseLevel * max(n, 1))()
        keep = []  # the System structures hold raw pointers into these tensors
        for k, i in enumerate(order):
            s = systems[i]
            lvl = self.level(s, precision, coarse)
            sys_arr[k] = s.op.system(s.known)
            works[k] = self._levels[id(s.op)][2].data_ptr()
            lvls[k] = lvl
            keep.append(s)
        first = [n, n, n, n]
        for k, i in enumerate(order):
            d = systems[i].op.dof_n
            first[d - 1] = min(first[d - 1], k)
        for d in (2, 1, 0):  # no system of dof_n = d + 1: its range is empty at the next start
            if first[d] == n:
                first[d] = first[d + 1]
        self._first = (ctypes.c_int32 * 4)(*first)
        self._max_nc = max([lvls[k].nc for k in range(n)] + [0])
        nb = int(L.gfea_coarse_batch_scratch_size(n))
        if self._scratch is None or self._scratch.numel() < nb:
            self._scratch = torch.empty(max(nb, 256), dtype=torch.uint8, device=_dev())
        opts = _lib.PcgOpts(_lib.ABI_VERSION, precision, 0, 0, 0.0, 0.0, 0, 0, int(coarse), 0)
        _lib.check(L.gfea_coarse_batch_prepare(sys_arr, ctypes.byref(opts), n, works, lvls, _lib.ptr(self._scratch),
                                               self._scratch.numel(), _lib.stream()), "coarse batch prepare")
        self._n = n
        self._prec = precision
        return [self._levels[id(s.op)][3] for s in systems]

    def build(self):
        """Rebuild the prepared batch's coarse matrices and inverses (device work only)."""
        _lib.check(_lib.load().gfea_coarse_batch_build(_lib.ptr(self._scratch), self._n, self._first, self._max_nc,
                                                       self._prec, _lib.stream()), "coarse batch build")


class BatchSolver:
    """Reusable buffers for repeated batches (workspace arena, descriptors, results).

    ``coarse`` (prepare / launch / solve): 0 solves with block-Jacobi PCG
    alone; -1 (default) gives every system the two-level preconditioner's
    coarse level (aggregate count chosen from its size, coarse dimension
    capped at 512), built on the current stream before the launch."""

    def __init__(self):
        self._arena = None
        self._scratch = None
        self._results = None
        self.coarse_levels = CoarseLevels()

    def _ensure(self, t: Optional[torch.Tensor], nbytes: int) -> torch.Tensor:
        if t is None or t.numel() < nbytes:
            t = torch.empty(max(nbytes, 1 << 16), dtype=torch.uint8, device=_dev())
        return t

    def launch(self, systems: List[BatchSystem], precision: str = "mixed", inner_rtol: float = 0.0,
               coarse: int = -1):
        """Enqueue the batch on the current stream (asynchronous)."""
        self.prepare(systems, precision, inner_rtol, coarse)
        self.launch_prepared()

    def launch_prepared(self):
        """Enqueue the prepared batch's device work only (capturable)."""
        _lib.check(_lib.load().gfea_batch_launch(_lib.ptr(self._scratch), self._n, ctypes.byref(self._opts),
                                                 _lib.stream()), "batch launch")

    def setup_coarse(self, systems: List[BatchSystem], coarse: int = -1):
        """Rebuild every system's coarse matrix and inverse from its current
        values (device work only, one launch per stage for the batch)."""
        if coarse != 0 and self._levels and self._levels[0] is not None:
            self.coarse_levels.build()

    def prepare(self, systems: List[BatchSystem], precision: str = "mixed", inner_rtol: float = 0.0,
                coarse: int = -1):
        """Validate the systems, build their coarse levels (unless ``coarse`` is
        0) and upload their descriptors (largest first).  ``inner_rtol``: the
        FP32 reliable-update trigger (0: 0.01 with the coarse level, 0.1
        without)."""
        L = _lib.load()
        prec = _lib.F64 if precision == "fp64" else _lib.F32
        n = len(systems)
        sizes = []
        for s in systems:
            if prec == _lib.F32 and s.op.vals32 is None:
                s.op.ensure_f32()
            sizes.append(int(L.gfea_batch_workspace_size(s.op.dmesh.Nn, s.op.dof_n, prec)))
        offs = np.concatenate([[0], np.cumsum([(z + 255) // 256 * 256 for z in sizes])]).astype(np.int64)
        self._arena = self._ensure(self._arena, int(offs[-1]))
        self._results = self._ensure(self._results, n * RESULT_BYTES)
        nscr = int(L.gfea_batch_scratch_size(n))
        self._scratch = self._ensure(self._scratch, nscr)
        arr = (_lib.BatchInstance * n)()
        base = self._arena.data_ptr()
        rbase = self._results.data_ptr()
        self._prec = prec
        if coarse != 0:
            self._levels = self.coarse_levels.prepare(systems, prec, coarse)
            self.coarse_levels.build()
        else:
            self._levels = [None] * n
        for i, s in enumerate(systems):
            d = s.op.dmesh
            arr[i] = _lib.BatchInstance(
                _lib.ABI_VERSION, s.op.dof_n, d.Nn, d.n_pairs, _lib.ptr(d.node_ptr), _lib.ptr(d.nbr),
                _lib.ptr(s.op.vals64), _lib.ptr(s.op.vals32) if prec == _lib.F32 else 0, _lib.ptr(s.known),
                int(s.op.translation_invariant), int(s.max_iters), float(s.rtol), _lib.ptr(s.b), _lib.ptr(s.x),
                base + int(offs[i]), rbase + i * RESULT_BYTES,
                self._levels[i] if self._levels[i] is not None else _lib.CoarseLevel())
        d_rtol = inner_rtol if 0 < inner_rtol < 1 else (0.01 if coarse != 0 else 0.1)
        self._opts = _lib.PcgOpts(_lib.ABI_VERSION, prec, 0, 0, 0.0, float(d_rtol), 0, 0)
        _lib.check(L.gfea_batch_prepare(arr, n, _lib.ptr(self._scratch), self._scratch.numel(),
                                        ctypes.byref(self._opts), _lib.stream()), "batch prepare")
        self._n = n

    def results(self) -> List[PcgInfo]:
        """Per-system outcome (synchronises the stream)."""
        raw = self._results[: self._n * RESULT_BYTES].cpu().numpy().tobytes()
        out = []
        for i in range(self._n):
            r = _lib.PcgResult.from_buffer_copy(raw[i * RESULT_BYTES:(i + 1) * RESULT_BYTES])
            out.append(PcgInfo(int(r.status), int(r.iterations), int(r.refinements), float(r.rel_residual),
                               float(r.floor_rel)))
        return out

    def solve(self, systems: List[BatchSystem], precision: str = "mixed", inner_rtol: float = 0.0,
              raise_on_fail: bool = True, coarse: int = -1) -> List[PcgInfo]:
        self.launch(systems, precision, inner_rtol, coarse)
        infos = self.results()
        if raise_on_fail:
            for i, info in enumerate(infos):
                _lib.check(info.status, f"batch system {i} (iterations {info.iterations}, "
                                        f"rel residual {info.rel_residual:.3e})")
        return infos


class GraphBatch:
    """A batch captured as one CUDA graph: optional device work ``pre`` (e.g.
    re-assembling every instance's operator), the coarse matrices and their
    inverses rebuilt from those values, the reset of each x to its initial
    state and the persistent batched solve.  ``replay`` re-runs all of
    it with one graph launch; buffers (values, b, x) are read in place, so new
    values written into them between replays are picked up."""

    def __init__(self, systems: List[BatchSystem], precision: str = "mixed", inner_rtol: float = 0.0,
                 pre=None, coarse: int = -1):
        from . import autotune

        self.systems = systems
        self.x0 = [s.x.clone() for s in systems]
        self.solver = BatchSolver()
        self.solver.prepare(systems, precision, inner_rtol, coarse)
        torch.cuda.synchronize()
        self.graph = torch.cuda.CUDAGraph()
        stream = torch.cuda.Stream()
        stream.wait_stream(torch.cuda.current_stream())
        prev = autotune.get_mode()
        autotune.set_mode(autotune.USE)  # no timing runs inside the capture
        try:
            with torch.cuda.graph(self.graph, stream=stream):
                if pre is not None:
                    pre()
                # coarse matrices and inverses from the values 'pre' wrote
                self.solver.setup_coarse(systems, coarse)
                for s, x0 in zip(systems, self.x0):
                    s.x.copy_(x0)
                self.solver.launch_prepared()
        finally:
            autotune.set_mode(prev)
        torch.cuda.synchronize()

    def replay(self):
        self.graph.replay()

    def results(self) -> List[PcgInfo]:
        return self.solver.results()


def solve_batch(systems: List[BatchSystem], precision: str = "mixed", inner_rtol: float = 0.0,
                raise_on_fail: bool = True, coarse: int = -1) -> List[PcgInfo]:
    return BatchSolver().solve(systems, precision, inner_rtol, raise_on_fail, coarse)


# ---------------------------------------------------------------------------
# random-material workload
# ---------------------------------------------------------------------------

def fourier_field(points: np.ndarray, rng: np.random.Generator, ell: float, modes: int = 64) -> np.ndarray:
    """Zero-mean, unit-variance Gaussian field with squared-exponential
    correlation of length ``ell``: sqrt(2/M) sum cos(k_m . x + phi_m),
    k_m ~ N(0, ell^-2 I), phi_m ~ U(0, 2 pi)."""
    dim = points.shape[1]
    k = rng.normal(0.0, 1.0 / ell, size=(modes, dim))
    phi = rng.uniform(0.0, 2 * np.pi, size=modes)
    return np.sqrt(2.0 / modes) * np.cos(points @ k.T + phi).sum(axis=1)


def random_material_cantilevers(n: int = 256, seed: int = 0, dof_min: float = 2e3, dof_max: float = 2e5,
                                L: float = 120.0, h: float = 13.0):
    """[(mesh, E_e)] for ``n`` cantilevers with per-instance seeds ``seed + i``."""
    from .mesh import Mesh_Quad4_Rect

    out = []
    for i in range(n):
        rng = np.random.default_rng(seed + i)
        N = np.exp(rng.uniform(np.log(dof_min), np.log(dof_max)))
        ny = max(1, int(round(np.sqrt(N / 2 * h / L))))
        nx = max(1, int(round(ny * L / h)))
        m = Mesh_Quad4_Rect(L, h, nx, ny)
        cent = m.coord[np.asarray(m.connect)].mean(axis=1)[:, :2]
        g = fourier_field(cent, rng, 0.1 * L)
        E = 210000.0 * np.exp(0.3 * g)
        out.append((m, E))
    return out


class RandomMaterialBatch:
    """The random-material workload assembled and solved as one CUDA graph.

    Per instance (a plane-stress cantilever with per-element E, clamped at
    x = 0, surface load -800/13^2 in y at x = L, thickness 13): the device
    mesh, the load vector, the Dirichlet mask and the stiffness operator are
    built once.  The graph holds, for every instance, the element-stiffness
    kernel (FP64, per-element moduli) and its FP32 copy, the coarse matrix
    and inverse of its two-level preconditioner, the reset of x; then the
    one persistent batched PCG launch for all instances.  ``replay`` runs the
    whole thing with one graph launch."""

    def __init__(self, instances, precision: str = "mixed", rtol: float = 1e-10, coarse: int = -1):
        from . import models
        from .device import DeviceMesh
        from .simulations import isotropic_lame

        L = _lib.load()
        self.instances = instances
        self.systems: List[BatchSystem] = []
        self._assembly = []
        lame = isotropic_lame(models.Elastic.Isotropic(2, E=1.0, v=0.3, planeStress=True).C)
        for m, E in instances:
            dm = DeviceMesh(m)
            op = CsrOperator(dm, 2, with_f32=True, translation_invariant=True)
            C = torch.as_tensor(np.concatenate([lame, np.asarray(E, dtype=np.float64)]), device=_dev())
            Lx = m.coord[:, 0].max()
            left = np.where(m.coord[:, 0] == 0)[0]
            right = np.where(m.coord[:, 0] == Lx)[0]
            b = torch.zeros(2 * m.Nn, dtype=torch.float64, device=_dev())
            mask = torch.zeros(m.Nn, dtype=torch.uint8, device=_dev())
            mask[torch.as_tensor(right, device=_dev())] = 1
            seg = [g for g in dm.boundary if g.dim == 1][0]
            _lib.check(L.gfea_surface_load(seg.code, _lib.ptr(dm.coord), _lib.ptr(seg.connect), seg.Ne,
                                           _lib.ptr(mask), 2, 1, (ctypes.c_int32 * 1)(1),
                                           (ctypes.c_double * 1)(-800 / 13**2), 13.0, _lib.ptr(b), _lib.stream()),
                       "surface load")
            known = torch.zeros(2 * m.Nn, dtype=torch.uint8, device=_dev())
            kd = np.concatenate([2 * left, 2 * left + 1])
            known[torch.as_tensor(kd, device=_dev())] = 1
            x = torch.zeros(2 * m.Nn, dtype=torch.float64, device=_dev())
            self.systems.append(BatchSystem(op, b, x, known, rtol=rtol))
            self._assembly.append((dm, op, C))
        self.assemble()  # values for the coarse aggregation and the capture's first pass
        torch.cuda.synchronize()
        self.graph = GraphBatch(self.systems, precision=precision, pre=self.assemble, coarse=coarse)

    def assemble(self):
        """Element stiffness (FP64, per-element E, thickness 13) and its FP32
        copy for every instance: device work only."""
        L = _lib.load()
        for dm, op, C in self._assembly:
            g = dm.main
            _lib.check(L.gfea_assemble_elastic(g.code, _lib.ptr(dm.coord), _lib.ptr(g.connect), g.Ne,
                                               _lib.ptr(dm.node_ptr), _lib.ptr(dm.rank), _lib.ptr(C), 4, 13.0,
                                               _lib.F64, _lib.ptr(op.vals64), op.nnz, 0, _lib.stream()),
                       "assemble elastic")
            _lib.check(L.gfea_cast_f64_f32(_lib.ptr(op.vals64), _lib.ptr(op.vals32), op.nnz, _lib.stream()),
                       "cast")

    def replay(self):
        self.graph.replay()

    def results(self) -> List[PcgInfo]:
        return self.graph.results()
