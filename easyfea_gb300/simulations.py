"""Simulations mirroring EasyFEA's ``Simulations.Elastic`` / ``Simulations.PhaseField``.

Same user-facing calls as the reference -- ``add_dirichlet``, ``add_surfLoad``,
``add_lineLoad``, ``add_neumann``, ``Bc_Init``, ``Solve``, ``Save_Iter``,
``Get_K_C_M_F``, ``Calc_Reaction``, ``Need_Update`` -- with the assembly and
the solve running on the GPU (libgb300fea.so).  Boundary-condition bookkeeping
is host code, as in the reference (EasyFEA/Simulations/_simu.py:2400-3050).

Differences from the reference that a user sees:
  * the linear solve is PCG preconditioned by nodal block-Jacobi plus a
    rigid-body-mode coarse level (FP64, or FP32 with FP64 refinement when
    ``precision = "mixed"``) to relative residual ``rtol`` instead of SuperLU;
    ``last_solve`` reports iterations and the final residual;
  * state stays on the device between calls; ``Solve`` returns host copies.
"""

from __future__ import annotations

from typing import Optional

import numpy as np
import torch

from . import _lib
from .device import CsrOperator, DeviceMesh, Workspace, max_abs_diff, pcg, reaction_energy
from .mesh import Mesh
from .models import Elastic as ElasticModels
from .models import PhaseField as PhaseFieldModel
from .models import _Elastic


def _dev():
    return torch.device("cuda", torch.cuda.current_device())



def isotropic_lame(C: np.ndarray):
    """(lambda, mu) when the Kelvin-Mandel matrix C (3x3 in 2D, 6x6 in 3D) is
    isotropic, C = lambda 1 (x) 1 + 2 mu I on the normal / shear blocks
    (plane stress included, with its reduced lambda); else None."""
    C = np.asarray(C, dtype=np.float64)
    n = C.shape[0]
    if C.shape != (n, n) or n not in (3, 6):
        return None
    nn = 2 if n == 3 else 3
    lam = C[0, 1]
    mu = 0.5 * C[n - 1, n - 1]
    iso = np.zeros_like(C)
    iso[:nn, :nn] = lam
    iso += 2.0 * mu * np.eye(n)
    scale = np.abs(C).max()
    if not scale > 0 or np.abs(C - iso).max() > 1e-13 * scale:
        return None
    return np.array([lam, mu], dtype=np.float64)

class _BC:
    def __init__(self, problemType, nodes, dofs, values, unknowns, description):
        self.problemType = problemType
        self.nodes = nodes
        self.dofs = dofs
        self.values = values
        self.unknowns = unknowns
        self.description = description


class _Simu:
    """Shared machinery (EasyFEA/Simulations/_simu.py)."""

    def __init__(self, mesh: Mesh, model, verbosity: bool = False):
        assert isinstance(mesh, Mesh), "mesh must be an easyfea_gb300 Mesh"
        self.mesh = mesh
        self.model = model
        self._verbosity = verbosity
        self.rho = 1.0
        self.precision = "fp64"
        self.rtol = 1e-12
        self.max_iters = 200000
        # aggregates of the two-level preconditioner's coarse level for
        # vector (displacement) and scalar (damage) systems: -1 automatic,
        # 0 block-Jacobi only
        self.coarse = -1
        self.coarse_scalar = 0
        # stiffness assembly schedule: "atomic" (element kernel with global
        # atomic adds) or "parts" (row-owned parts in shared memory)
        self.assembly_schedule = "atomic"
        self._workspaces: dict = {}
        self.last_solve = None
        self._dmesh: Optional[DeviceMesh] = None
        self._results: list = []
        self.folder = ""
        model._Add_observer(self)
        self.Bc_Init()
        self.Need_Update()

    # ---- infrastructure ------------------------------------------------------
    @property
    def dmesh(self) -> DeviceMesh:
        if self._dmesh is None:
            self._dmesh = DeviceMesh(self.mesh)
        return self._dmesh

    @property
    def dim(self) -> int:
        return self.mesh.dim

    def _Update(self, observable) -> None:
        self.Need_Update()

    def Need_Update(self, value: bool = True) -> None:
        self._needUpdate = value

    @property
    def needUpdate(self) -> bool:
        return self._needUpdate

    def Get_problemTypes(self) -> list:
        return [self.problemType]

    def _check_pt(self, problemType):
        if problemType is None:
            problemType = self.problemType
        problemType = str(getattr(problemType, "value", problemType))
        assert problemType in self.Get_problemTypes(), f"unknown problemType {problemType}"
        return problemType

    def Ndof(self, problemType=None) -> int:
        return self.mesh.Nn * self.Get_dof_n(problemType)

    # ---- boundary conditions (EasyFEA/Simulations/_simu.py:2190-2842) --------
    def Bc_Init(self) -> None:
        self._dirichlet = {pt: [] for pt in self.Get_problemTypes()}
        self._neumann = {pt: [] for pt in self.Get_problemTypes()}
        self._b_neu = {pt: None for pt in self.Get_problemTypes()}

    def Bc_dofs_nodes(self, nodes, unknowns, problemType=None) -> np.ndarray:
        problemType = self._check_pt(problemType)
        nodes = np.asarray(nodes, dtype=np.int64)
        avail = self.Get_unknowns(problemType)
        dofs = np.zeros((nodes.size, len(unknowns)), dtype=np.int64)
        for i, u in enumerate(unknowns):
            assert u in avail, f"unknown {u} not in {avail}"
            dofs[:, i] = nodes * len(avail) + avail.index(u)
        return dofs.ravel()

    @staticmethod
    def _check_inputs(nodes, values, unknowns) -> bool:
        if len(nodes) == 0 or len(values) == 0:
            return False
        assert len(values) == len(unknowns), f"len(values)={len(values)} must equal len(unknowns)={len(unknowns)}."
        return True

    def _eval_nodes(self, nodes, value):
        coord = self.mesh.coord[nodes]
        if callable(value):
            return np.asarray(value(coord[:, 0], coord[:, 1], coord[:, 2]), dtype=float) * np.ones(len(nodes))
        return np.broadcast_to(np.asarray(value, dtype=float), (len(nodes),)).copy()

    def add_dirichlet(self, nodes, values: list, unknowns: list, problemType=None, description="") -> None:
        """Imposed values; duplicate DOFs add up (EasyFEA/Simulations/_simu.py:2400-2469, :3013-3040)."""
        if not self._check_inputs(nodes, values, unknowns):
            return
        problemType = self._check_pt(problemType)
        nodes = np.asarray(nodes, dtype=np.int64)
        vals = np.zeros((nodes.size, len(unknowns)))
        for d in range(len(unknowns)):
            vals[:, d] = self._eval_nodes(nodes, values[d])
        dofs = self.Bc_dofs_nodes(nodes, unknowns, problemType)
        self._dirichlet[problemType].append(_BC(problemType, nodes, dofs, vals.ravel(), unknowns, description))

    def _neumann_vec(self, problemType) -> torch.Tensor:
        if self._b_neu[problemType] is None:
            self._b_neu[problemType] = torch.zeros(self.Ndof(problemType), dtype=torch.float64, device=_dev())
        return self._b_neu[problemType]

    def add_neumann(self, nodes, values: list, unknowns: list, problemType=None, description="") -> None:
        """Point loads split evenly over the nodes (EasyFEA/Simulations/_simu.py:2743-2768)."""
        if not self._check_inputs(nodes, values, unknowns):
            return
        problemType = self._check_pt(problemType)
        nodes = np.asarray(nodes, dtype=np.int64)
        vals = np.zeros((nodes.size, len(unknowns)))
        for i in range(len(unknowns)):
            vals[:, i] = self._eval_nodes(nodes, values[i]) / len(nodes)
        dofs = self.Bc_dofs_nodes(nodes, unknowns, problemType)
        b = self._neumann_vec(problemType)
        b.index_add_(0, torch.as_tensor(dofs, device=_dev()), torch.as_tensor(vals.ravel(), device=_dev()))
        self._neumann[problemType].append(_BC(problemType, nodes, dofs, vals.ravel(), unknowns, description))

    def _integrate_load(self, nodes, values, unknowns, problemType, factor, bdim):
        """Boundary integral of a traction (EasyFEA/Simulations/_simu.py:2770-2842):
        constants and functions of (x, y, z) at the mass Gauss points of the
        boundary elements whose nodes all belong to ``nodes``; an array of one
        value per node of ``nodes`` integrated as value(node) x integral of N_node."""
        problemType = self._check_pt(problemType)
        L = _lib.load()
        avail = self.Get_unknowns(problemType)
        nodes = np.asarray(nodes, dtype=np.int64)
        mask = torch.zeros(self.mesh.Nn, dtype=torch.uint8, device=_dev())
        mask[torch.as_tensor(nodes, device=_dev())] = 1
        b = self._neumann_vec(problemType)
        groups = [g for g in self.dmesh.boundary if g.dim == bdim]
        if bdim == self.dim:
            groups = [self.dmesh.main]
        const = [i for i, v in enumerate(values) if isinstance(v, (int, float)) and not callable(v)]
        if const:
            uidx = (ctypes_int32 * len(const))(*[avail.index(unknowns[i]) for i in const])
            uval = (ctypes_double * len(const))(*[float(values[i]) for i in const])
            for g in groups:
                _lib.check(L.gfea_surface_load(g.code, _lib.ptr(self.dmesh.coord), _lib.ptr(g.connect), g.Ne,
                                               _lib.ptr(mask), len(avail), len(const), uidx, uval, float(factor),
                                               _lib.ptr(b), _lib.stream()), "surface load")
        for i, v in enumerate(values):
            if i in const:
                continue
            ui = avail.index(unknowns[i])
            for g in groups:
                if g.Ne == 0:
                    continue
                if callable(v):
                    npg = ctypes_int32()
                    # the number of points first (no element), then the points
                    _lib.check(L.gfea_boundary_gauss_points(g.code, _lib.ptr(self.dmesh.coord), _lib.ptr(g.connect),
                                                            0, 0, __import__("ctypes").byref(npg), _lib.stream()),
                               "gauss points")
                    xyz = torch.empty((g.Ne, npg.value, 3), dtype=torch.float64, device=_dev())
                    _lib.check(L.gfea_boundary_gauss_points(g.code, _lib.ptr(self.dmesh.coord), _lib.ptr(g.connect),
                                                            g.Ne, _lib.ptr(xyz), __import__("ctypes").byref(npg),
                                                            _lib.stream()), "gauss points")
                    pts = xyz.view(-1)[:g.Ne * npg.value * 3].view(g.Ne, npg.value, 3).cpu().numpy()
                    f = np.asarray(v(pts[:, :, 0], pts[:, :, 1], pts[:, :, 2]), dtype=np.float64)
                    f = np.array(np.broadcast_to(f, (g.Ne, npg.value)), dtype=np.float64)
                    vals, mode = torch.as_tensor(f, device=_dev()), 0
                else:
                    arr = np.asarray(v, dtype=np.float64)
                    full = np.zeros(self.mesh.Nn)
                    full[nodes] = arr
                    vals, mode = torch.as_tensor(full, device=_dev()), 1
                _lib.check(L.gfea_surface_load_field(g.code, _lib.ptr(self.dmesh.coord), _lib.ptr(g.connect), g.Ne,
                                                     _lib.ptr(mask), len(avail), ui, mode, _lib.ptr(vals),
                                                     float(factor), _lib.ptr(b), _lib.stream()), "surface load")
        self._neumann[problemType].append(_BC(problemType, nodes, None, None, unknowns, "load"))

    def add_surfLoad(self, nodes, values: list, unknowns: list, problemType=None, description="") -> None:
        """Surface load: lines x thickness in 2D, faces in 3D (EasyFEA/Simulations/_simu.py:2572-2630)."""
        if not self._check_inputs(nodes, values, unknowns):
            return
        if self.dim == 2:
            self._integrate_load(nodes, values, unknowns, problemType, self.model_thickness, 1)
        else:
            self._integrate_load(nodes, values, unknowns, problemType, 1.0, 2)

    def add_lineLoad(self, nodes, values: list, unknowns: list, problemType=None, description="") -> None:
        """Line load (EasyFEA/Simulations/_simu.py:2530-2570), no thickness factor."""
        if not self._check_inputs(nodes, values, unknowns):
            return
        self._integrate_load(nodes, values, unknowns, problemType, 1.0, 1)

    def Bc_dofs_known_unknown(self, problemType=None):
        problemType = self._check_pt(problemType)
        n = self.Ndof(problemType)
        mask = np.ones(n, dtype=bool)
        for bc in self._dirichlet[problemType]:
            mask[bc.dofs] = False
        return np.nonzero(~mask)[0], np.nonzero(mask)[0]

    def _dirichlet_state(self, problemType, b: torch.Tensor):
        """(known mask uint8, x with known values) on the device.

        Known values add up on duplicate DOFs (COO sum, _simu.py:1962-1966).
        Orphan-node DOFs get x = b there, which is what the reference's unit
        diagonal (_simu.py:1936-1946) produces."""
        n = self.Ndof(problemType)
        known = np.zeros(n, dtype=np.uint8)
        xk = np.zeros(n)
        for bc in self._dirichlet[problemType]:
            known[bc.dofs] = 1
            np.add.at(xk, bc.dofs, bc.values)
        orphans = np.asarray(self.mesh.orphanNodes, dtype=np.int64)
        od = np.zeros(0, dtype=np.int64)
        if orphans.size:
            od = self.Bc_dofs_nodes(orphans, self.Get_unknowns(problemType), problemType)
            od = od[known[od] == 0]
            known[od] = 1
        known_d = torch.as_tensor(known, device=_dev())
        x = torch.as_tensor(xk, device=_dev())
        if od.size:
            odd = torch.as_tensor(od, device=_dev())
            x[odd] = b[odd]
        return known_d, x

    def _solve_system(self, op: CsrOperator, b: torch.Tensor, problemType, x0: Optional[torch.Tensor] = None):
        known, x = self._dirichlet_state(problemType, b)
        if x0 is not None:
            x = torch.where(known.bool(), x, x0)
        coarse = self.coarse if op.dof_n > 1 else self.coarse_scalar
        ws = self._workspaces.setdefault(str(problemType), Workspace())
        info = pcg(op, b, x, known, rtol=self.rtol, precision="fp64" if self.precision == "fp64" else "mixed",
                   max_iters=self.max_iters, coarse=coarse, workspace=ws)
        self.last_solve = info
        return x

    def _solve_bounded(self, op: CsrOperator, b: torch.Tensor, problemType, lb: torch.Tensor, ub: torch.Tensor,
                       x0: Optional[torch.Tensor] = None, tol: float = 1e-12, max_outer: int = 100):
        """min ||A_uu x_u - (b_u - A_uk x_k)|| with lb <= x_u <= ub on the
        unknown DOFs u, the known ones x_k fixed: the reference's bounded
        least-squares damage solve (scipy.optimize.lsq_linear on the r1
        system, Solvers.py:376-383, bounds of _phasefield.py:148-163).

        Projected Newton on the strictly convex cost: the gradient
        g = A^T (A x - b) (A symmetric) fixes the binding set (at lb with
        g > 0, at ub with g < 0); the step on the other unknowns solves their
        least-squares problem by CGLS (two products with A per iteration);
        the step is projected on the box and halved until the cost decreases
        (Armijo); the loop ends when the projected gradient is below
        ``tol`` times its start value."""
        known, xk = self._dirichlet_state(problemType, b)
        unk = known == 0
        zero = torch.zeros_like(b)

        def A_u(v):  # rows and columns of the unknown DOFs
            return torch.where(unk, op.matvec(torch.where(unk, v, zero)), zero)

        bi = torch.where(unk, b - op.matvec(torch.where(unk, zero, xk)), zero)
        lo = torch.where(unk, lb, zero)
        hi = torch.where(unk, ub, zero)
        x = torch.where(unk, x0 if x0 is not None else zero, zero)
        x = torch.minimum(torch.maximum(x, lo), hi)
        g0 = None
        for _ in range(max_outer):
            r = A_u(x) - bi
            g = A_u(r)
            free = unk & ~(((x <= lo) & (g > 0)) | ((x >= hi) & (g < 0)))
            pg = float(torch.linalg.norm(torch.where(free, g, zero)))
            if g0 is None:
                g0 = max(float(torch.linalg.norm(A_u(bi))), 1e-300)
            if pg <= tol * g0:
                break
            # CGLS on the free unknowns: min ||A_F d + r||
            d = torch.zeros_like(b)
            rr = -r
            sv = torch.where(free, A_u(rr), zero)
            p = sv.clone()
            gam = float(sv @ sv)
            gam0 = gam
            for _k in range(20 * int(free.sum()) + 10):
                q = A_u(p)
                qq = float(q @ q)
                if qq <= 0:
                    break
                a = gam / qq
                d += a * p
                rr -= a * q
                sv = torch.where(free, A_u(rr), zero)
                gn = float(sv @ sv)
                if gn <= (1e-14) ** 2 * gam0:
                    break
                p = sv + (gn / gam) * p
                gam = gn
            f0 = 0.5 * float(r @ r)
            alpha = 1.0
            while True:
                xn = torch.minimum(torch.maximum(x + alpha * d, lo), hi)
                rn = A_u(xn) - bi
                fn = 0.5 * float(rn @ rn)
                if fn <= f0 + 1e-4 * float(g @ (xn - x)) or alpha < 1e-12:
                    break
                alpha *= 0.5
            x = xn
        return torch.where(unk, x, xk)

    # ---- iterations (_simu.py:288-471) ---------------------------------------
    def Save_Iter(self, iter: Optional[dict] = None) -> dict:
        """Store one iteration dict, in memory (folder == "") or as
        ``folder/Results/results{Niter}.pickle``: the reference's
        single-process layout and keys, so either side reads the other's."""
        it = {} if iter is None else dict(iter)
        it["indexMesh"] = 0
        if self.folder == "":
            self._results.append(it)
        else:
            import os
            import pickle

            d = os.path.join(self.folder, "Results")
            os.makedirs(d, exist_ok=True)
            path = os.path.join(d, f"results{self.Niter}.pickle")
            with open(path, "wb") as f:
                pickle.dump(it, f)
            self._results.append(path)
        return it

    @property
    def Niter(self) -> int:
        """Number of saved iterations."""
        return len(self._results)

    def Get_results(self, iter: int = -1) -> dict:
        """The iteration dict at index ``iter`` (read from its pickle in folder mode)."""
        iter = int(iter)
        if iter < 0:
            iter += self.Niter
        assert 0 <= iter < self.Niter, f"`iter` must be in [0, {self.Niter})"
        entry = self._results[iter]
        if isinstance(entry, str):
            import pickle

            with open(entry, "rb") as f:
                return pickle.load(f)
        return dict(entry)

    def Set_Iter(self, iter: int = -1, resetAll: bool = False) -> dict:
        raise NotImplementedError

    @property
    def results(self) -> list:
        return [self.Get_results(i) for i in range(self.Niter)]

    # ---- post-processing on the device (_simu.py:3067-3151) -------------------
    def Results_Available(self) -> list:
        return []

    def Result(self, result: str, nodeValues: bool = True):
        """The reference's Result(result, nodeValues): a host array (nodes or
        elements) or a float; computed on the device by Result_device."""
        v = self.Result_device(result, nodeValues)
        return v if isinstance(v, float) or v is None else v.cpu().numpy()

    def Result_device(self, result: str, nodeValues: bool = True):
        raise NotImplementedError

    def _check_result(self, result: str) -> None:
        if result not in self.Results_Available():
            raise ValueError(f"For a {self.problemType} problem result must be in: {self.Results_Available()}")

    def _reshape_values(self, values: torch.Tensor, nodeValues: bool) -> torch.Tensor:
        """Results_Reshape_values (_simu.py:3095-3151): element values to the
        nodes (node average) or node values to the elements (mean over each
        element's nodes); a node-sized array counts as node values first, as
        in the reference."""
        dm = self.dmesh
        Nn, Ne = dm.Nn, dm.main.Ne
        is1d = values.dim() == 1
        if nodeValues:
            if values.numel() % Nn == 0:
                return values.reshape(-1) if is1d else values.reshape(Nn, -1)
            vn = dm.node_values(values.reshape(Ne, -1))
            return vn.reshape(-1) if is1d else vn
        if values.numel() % Ne == 0:
            return values.reshape(-1) if is1d else values.reshape(Ne, -1)
        ve = values.reshape(Nn, -1)[dm.main.connect.long()].mean(1)
        return ve.reshape(-1) if is1d else ve

    def _element_fields(self, u: torch.Tensor, gauss: int = 0, coef: float = float(np.sqrt(2)), strain=False,
                        stress=False, vm=False, energy=False, psiP=False, sigma_n=None, pf=None, d=None,
                        H_old=None) -> dict:
        """One gfea_element_fields launch; returns the requested (Ne, ...) device tensors."""
        import ctypes

        dm = self.dmesh
        g = dm.main
        n = 3 if self.dim == 2 else 6
        out = {}

        def take(key, want, shape):
            if not want:
                return 0
            out[key] = torch.empty(shape, dtype=torch.float64, device=_dev())
            return _lib.ptr(out[key])

        f = _lib.Fields()
        f.version = _lib.ABI_VERSION
        f.gauss = gauss
        f.coef = coef
        f.thickness = self.model_thickness if self.dim == 2 else 1.0
        keep = []
        if pf is None:
            C, mode = self._C_device()
            keep.append(C)
            f.C = _lib.ptr(C)
            f.c_per_elem = int(mode)
        else:
            f.pf = ctypes.pointer(pf)
            f.d = _lib.ptr(d)
            f.H_old = _lib.ptr(H_old)
        if sigma_n is not None:
            sigma_n = sigma_n.contiguous()
            keep.append(sigma_n)
            f.sigma_n = _lib.ptr(sigma_n)
        f.strain_e = take("strain", strain, (g.Ne, n))
        f.stress_e = take("stress", stress, (g.Ne, n))
        f.vm_e = take("vm", vm, (g.Ne, 2))
        f.energy_e = take("energy", energy, (g.Ne,))
        f.psiP_e = take("psiP", psiP, (g.Ne,))
        _lib.check(_lib.load().gfea_element_fields(g.code, _lib.ptr(dm.coord), _lib.ptr(g.connect), g.Ne,
                                                   _lib.ptr(u), ctypes.byref(f), _lib.stream()), "element fields")
        return out

    def _displacement_result(self, u: torch.Tensor, result: str):
        Nn = self.mesh.Nn
        if result in ("ux", "uy", "uz"):
            return u.reshape(Nn, -1)[:, "xyz".index(result[1])]
        if result == "displacement":
            return u
        return torch.linalg.norm(u.reshape(Nn, -1), dim=1)  # displacement_norm

    def _strain_stress_result(self, result: str, fields) -> torch.Tensor:
        """The strain / stress branch of Result (_elastic.py:296-320,
        _phasefield.py:733-754); ``fields(strain, stress, vm)`` launches the
        element kernel."""
        isStrain = "E" in result or result == "Strain"
        isStress = "S" in result and result != "Strain"
        if not (isStrain or isStress):
            raise ValueError("Wrong option")
        res = result if result in ("Strain", "Stress") else result[-2:]
        if res == "vm":
            return fields(False, False, True)["vm"][:, 1 if isStress else 0]
        out = fields(not isStress, isStress, False)["stress" if isStress else "strain"]
        if res in ("Strain", "Stress"):
            return out
        names = ("xx", "yy", "xy") if self.dim == 2 else ("xx", "yy", "zz", "yz", "xz", "xy")
        return out[:, names.index(res)]


ctypes_int32 = __import__("ctypes").c_int32
ctypes_double = __import__("ctypes").c_double


class Elastic(_Simu):
    """Linear elasticity (EasyFEA/Simulations/_elastic.py)."""

    problemType = "elastic"

    def __init__(self, mesh: Mesh, model: _Elastic, folder: str = "", verbosity: bool = False):
        assert isinstance(model, _Elastic), "model must be an elastic model"
        assert model.dim == mesh.dim, "the material and the mesh must have the same dimension"
        self.__K = None
        self.__M = None
        self.__u = None
        super().__init__(mesh, model, verbosity)

    @property
    def material(self):
        return self.model

    @property
    def model_thickness(self) -> float:
        return self.model.thickness

    def Get_unknowns(self, problemType=None) -> list:
        return ["x", "y"] if self.dim == 2 else ["x", "y", "z"]

    def Get_dof_n(self, problemType=None) -> int:
        return self.dim

    def Need_Update(self, value: bool = True) -> None:
        super().Need_Update(value)
        if value:
            self.__M = None

    def _C_device(self):
        """(C tensor, mode) for gfea_assemble_elastic: an isotropic law as
        (lambda, mu) (3), or (lambda, mu) for E = 1 followed by the per-element
        moduli (4); other laws as the Kelvin-Mandel C, homogeneous (0) or per
        element (1)."""
        mat = self.material
        if getattr(mat, "isHeterogeneous", False) and isinstance(mat, ElasticModels.Isotropic):
            E = np.asarray(mat.E, dtype=np.float64).ravel()
            assert E.size == self.mesh.Ne, "per-element E must have one value per element"
            ref = ElasticModels.Isotropic(mat.dim, E=1.0, v=mat.v, planeStress=mat.planeStress).C
            lame = isotropic_lame(ref)
            if lame is not None:
                return torch.as_tensor(np.concatenate([lame, E]), device=_dev()), 4
            return torch.as_tensor(np.concatenate([ref.ravel(), E]), device=_dev()), 2
        C = np.ascontiguousarray(mat.C, dtype=np.float64)
        if C.ndim == 2:
            lame = isotropic_lame(C)
            if lame is not None:
                return torch.as_tensor(lame, device=_dev()), 3
        return torch.as_tensor(C, device=_dev()), 1 if C.ndim == 3 else 0

    def Assembly(self, problemType=None) -> CsrOperator:
        """K = sum_e K_e x thickness on the device (_elastic.py:123-152, _simu.py:1104-1144)."""
        dm = self.dmesh
        op = self.__K if self.__K is not None else CsrOperator(dm, self.dim, translation_invariant=True)
        C, per_elem = self._C_device()
        g = dm.main
        factor = self.material.thickness if self.dim == 2 else 1.0
        if self.assembly_schedule == "parts":
            import ctypes

            plan, _ = dm.part_plan(self.dim, _lib.F64)
            _lib.check(_lib.load().gfea_assemble_elastic_parts(g.code, _lib.ptr(dm.coord), _lib.ptr(g.connect), g.Ne,
                                                               _lib.ptr(dm.node_ptr), _lib.ptr(dm.rank), _lib.ptr(C),
                                                               int(per_elem), factor, _lib.F64, _lib.ptr(op.vals64),
                                                               ctypes.byref(plan), _lib.stream()), "assemble parts")
        else:
            _lib.check(_lib.load().gfea_assemble_elastic(g.code, _lib.ptr(dm.coord), _lib.ptr(g.connect), g.Ne,
                                                         _lib.ptr(dm.node_ptr), _lib.ptr(dm.rank), _lib.ptr(C),
                                                         int(per_elem), factor, _lib.F64, _lib.ptr(op.vals64),
                                                         op.nnz, 0, _lib.stream()), "assemble elastic")
        self.__K = op
        return op

    def _mass(self) -> CsrOperator:
        if self.__M is None:
            dm = self.dmesh
            op = CsrOperator(dm, self.dim)
            g = dm.main
            factor = self.material.thickness if self.dim == 2 else 1.0
            _lib.check(_lib.load().gfea_assemble_mass(g.code, _lib.ptr(dm.coord), _lib.ptr(g.connect), g.Ne,
                                                      _lib.ptr(dm.node_ptr), _lib.ptr(dm.rank), self.dim,
                                                      float(self.rho), factor, _lib.F64, _lib.ptr(op.vals64),
                                                      op.nnz, 0, _lib.stream()), "assemble mass")
            self.__M = op
        return self.__M

    @property
    def K_device(self) -> CsrOperator:
        if self.needUpdate or self.__K is None:
            self.Assembly()
            self.Need_Update(False)
        return self.__K

    def Get_K_C_M_F(self, problemType=None):
        """Host scipy copies (K, C, M, F) with the reference's CSR layout (_simu.py:161-175)."""
        import scipy.sparse as sp

        K = self.K_device.to_scipy()
        M = self._mass().to_scipy()
        C = sp.csr_matrix((np.zeros(K.nnz), K.indices, K.indptr), shape=K.shape)
        F = sp.csr_matrix((K.shape[0], 1))
        return K, C, M, F

    def Solve(self) -> np.ndarray:
        """Solve K u = b with the Dirichlet conditions; returns u (host copy)."""
        return self.Solve_device().cpu().numpy()

    def Solve_device(self) -> torch.Tensor:
        """Same as Solve, leaving u on the device (no host copy)."""
        op = self.K_device
        b = self._neumann_vec(self.problemType)
        self.__u = self._solve_system(op, b, self.problemType)
        return self.__u

    @property
    def u_device(self) -> Optional[torch.Tensor]:
        return self.__u

    def _Set_solutions(self, problemType, u) -> None:
        """Set the displacement (_simu.py:1517-1530)."""
        self._check_pt(problemType)
        self.__u = torch.as_tensor(np.ascontiguousarray(u, dtype=np.float64), device=_dev()).reshape(-1).clone()

    @property
    def displacement(self) -> np.ndarray:
        if self.__u is None:
            return np.zeros(self.Ndof())
        return self.__u.cpu().numpy()

    def Calc_Reaction(self, dofs=None, problemType=None) -> np.ndarray:
        """K[dofs] @ u (_simu.py:212-260)."""
        op = self.K_device
        u = self.__u if self.__u is not None else torch.zeros(self.Ndof(), dtype=torch.float64, device=_dev())
        _, _, Ku = reaction_energy(op, u, None)
        Ku = Ku.cpu().numpy()
        return Ku if dofs is None else Ku[np.asarray(dofs)]

    def Save_Iter(self, iter: Optional[dict] = None) -> dict:
        it = {} if iter is None else iter
        it["displacement"] = self.displacement
        return super().Save_Iter(it)

    def Set_Iter(self, iter: int = -1, resetAll: bool = False) -> dict:
        """Restore the displacement of a saved iteration (_elastic.py:178-205)."""
        results = self.Get_results(iter)
        self._Set_solutions(self.problemType, results["displacement"])
        return results

    # ---- results (_elastic.py:201-418) ---------------------------------------
    def Results_Available(self) -> list:
        comps = ["x", "y"] if self.dim == 2 else ["x", "y", "z"]
        tens = ["xx", "yy", "xy"] if self.dim == 2 else ["xx", "yy", "zz", "yz", "xz", "xy"]
        return (["displacement", "displacement_norm"] + [f"u{c}" for c in comps] + [f"S{t}" for t in tens] +
                [f"E{t}" for t in tens] + ["Svm", "Stress", "Evm", "Strain", "Wdef", "Wdef_e", "ZZ1", "ZZ1_e"])

    def Result_device(self, result: str, nodeValues: bool = True):
        """Elastic.Result on the device: displacement results, strain / stress
        components and von Mises (element means of the Gauss-point values),
        the strain energy and the ZZ1 error estimator."""
        self._check_result(result)
        u = self.__u if self.__u is not None else torch.zeros(self.Ndof(), dtype=torch.float64, device=_dev())
        if result in ("ux", "uy", "uz", "displacement", "displacement_norm"):
            values = self._displacement_result(u, result)
        elif result in ("Wdef", "Wdef_e"):
            W_e = self._element_fields(u, energy=True)["energy"]
            if result == "Wdef":
                return float(W_e.sum())
            values = W_e
        elif result in ("ZZ1", "ZZ1_e"):
            err, err_e = self._zz1(u)
            if result == "ZZ1":
                return err
            values = err_e
        else:
            values = self._strain_stress_result(
                result, lambda e, s, v: self._element_fields(u, strain=e, stress=s, vm=v))
        return self._reshape_values(values, nodeValues)

    def _zz1(self, u: torch.Tensor):
        """ZZ1 error (_elastic.py:397-418): the plain element energies, the
        Kelvin-Mandel element-mean stress averaged at the nodes, and the
        energies of that smoothed stress interpolated back with N."""
        first = self._element_fields(u, coef=1.0, stress=True, energy=True)
        sigma_n = self.dmesh.node_values(first["stress"])
        Ws_e = self._element_fields(u, energy=True, sigma_n=sigma_n)["energy"]
        W_e = first["energy"]
        Welas = W_e.sum()
        err = float(torch.abs(Welas - Ws_e.sum()) / Welas)
        return err, torch.abs(Ws_e - W_e) / Welas


class PhaseField(_Simu):
    """Staggered phase-field damage (EasyFEA/Simulations/_phasefield.py)."""

    problemType = "damage"

    class ProblemTypes:
        damage = "damage"
        elastic = "elastic"

    def __init__(self, mesh: Mesh, model: PhaseFieldModel, folder: str = "", verbosity: bool = False):
        assert isinstance(model, PhaseFieldModel), "model must be a phase field model"
        if model.split in ("Zhang", "Stress") or model.split.endswith(("_PM", "_MP", "_NoCross")):
            # Zhang: c+ = P+(sigma) C is not symmetric; Stress: c+ = C s+ C
            # with s+ = a P+ - b R+ IxI is not positive semi-definite, so the
            # degraded stiffness g c+ + c- can be indefinite; the PM / MP
            # anisotropic variants put one cross block (Cpm or Cmp, transposes
            # of each other) on each side, which is not symmetric, and NoCross
            # leaves C - (1 - g) Cpp, which can be indefinite.  The staggered
            # loop's PCG needs SPD systems (the reference factorises them with
            # a direct solver); these splits are available through
            # gfea_pf_split.  AnisotStrain / AnisotStress give g C + (1 - g) Cmm.
            raise NotImplementedError(f"the {model.split} split does not give an SPD degraded stiffness; the GPU "
                                      "staggered loop solves SPD systems")
        assert model.dim == mesh.dim, "the material and the mesh must have the same dimension"
        self.__u = None
        self.__d = None
        self.__Ku = None
        self.__Kd = None
        self.__Fd = None
        self.__psiP = None
        self.__psiP_old = None
        self.__updatedDamage = False
        self.__updatedDisplacement = False
        self.__Niter = 0
        self.__convIter = 0.0
        self.__timeIter = 0.0
        super().__init__(mesh, model, verbosity)

    @property
    def phaseFieldModel(self) -> PhaseFieldModel:
        return self.model

    @property
    def model_thickness(self) -> float:
        return self.model.thickness

    def Get_problemTypes(self) -> list:
        return ["damage", "elastic"]

    def Get_unknowns(self, problemType=None) -> list:
        if self._check_pt_raw(problemType) == "damage":
            return ["d"]
        return ["x", "y"] if self.dim == 2 else ["x", "y", "z"]

    @staticmethod
    def _check_pt_raw(problemType):
        return str(getattr(problemType, "value", problemType)) if problemType is not None else "damage"

    def Get_dof_n(self, problemType=None) -> int:
        return 1 if self._check_pt_raw(problemType) == "damage" else self.dim

    def Bc_dofs_nodes(self, nodes, unknowns, problemType="elastic") -> np.ndarray:
        return super().Bc_dofs_nodes(nodes, unknowns, problemType)

    def add_dirichlet(self, nodes, values, unknowns, problemType="elastic", description=""):
        return super().add_dirichlet(nodes, values, unknowns, problemType, description)

    def add_neumann(self, nodes, values, unknowns, problemType="elastic", description=""):
        return super().add_neumann(nodes, values, unknowns, problemType, description)

    def add_surfLoad(self, nodes, values, unknowns, problemType="elastic", description=""):
        return super().add_surfLoad(nodes, values, unknowns, problemType, description)

    def add_lineLoad(self, nodes, values, unknowns, problemType="elastic", description=""):
        return super().add_lineLoad(nodes, values, unknowns, problemType, description)

    def Need_Update(self, value: bool = True) -> None:
        super().Need_Update(value)
        self.__updatedDamage = not value
        self.__updatedDisplacement = not value

    # ---- state ---------------------------------------------------------------
    def _state(self):
        if self.__u is None:
            self.__u = torch.zeros(self.mesh.Nn * self.dim, dtype=torch.float64, device=_dev())
            self.__d = torch.zeros(self.mesh.Nn, dtype=torch.float64, device=_dev())
        return self.__u, self.__d

    @property
    def displacement(self) -> np.ndarray:
        return self._state()[0].cpu().numpy()

    @property
    def damage(self) -> np.ndarray:
        return self._state()[1].cpu().numpy()

    @property
    def u_device(self) -> torch.Tensor:
        return self._state()[0]

    @property
    def d_device(self) -> torch.Tensor:
        return self._state()[1]

    @property
    def psiP_device(self) -> Optional[torch.Tensor]:
        return self.__psiP

    def _Set_solutions(self, problemType, x) -> None:
        """Set the displacement or the damage (_simu.py:1517-1530); the
        operators that depend on it are re-assembled at their next use."""
        pt = self._check_pt_raw(problemType)
        u, d = self._state()
        (u if pt == "elastic" else d).copy_(torch.as_tensor(np.ascontiguousarray(x, dtype=np.float64)).reshape(-1))
        self.__updatedDamage = False
        self.__updatedDisplacement = False

    def set_history(self, H: Optional[np.ndarray]) -> None:
        """Replace the committed History field (psi+ at the mass Gauss points,
        (Ne, nPg) or flat); None clears it, as before the first Save_Iter.
        The damage system is re-assembled at its next use."""
        self.__updatedDamage = False
        if H is None:
            self.__psiP_old = None
            return
        h = torch.as_tensor(np.ascontiguousarray(H, dtype=np.float64).ravel(), device=_dev())
        if self.__psiP_old is not None and self.__psiP_old.numel() == h.numel():
            self.__psiP_old.copy_(h)
        else:
            self.__psiP_old = h.clone()

    def _params(self) -> _lib.PfParams:
        m = self.phaseFieldModel
        mat = m.material
        p = _lib.PfParams()
        p.version = _lib.ABI_VERSION
        p.split = _lib.SPLIT_CODE[m.split]
        p.regularization = _lib.REGU_CODE[m.regularization]
        p.dim = self.dim
        if isinstance(mat, ElasticModels.Isotropic):
            p.lambda_ = float(mat.get_lambda())
            p.mu = float(mat.get_mu())
        p.Gc = m.Gc
        p.l0 = m.l0
        p.thickness = m.thickness if self.dim == 2 else 1.0
        A = np.asarray(m.A, dtype=float).reshape(self.dim, self.dim)
        for i in range(self.dim * self.dim):
            p.A[i] = A.ravel()[i]
        C = mat.C.ravel()
        for i in range(C.size):
            p.C[i] = C[i]
        S = np.asarray(mat.S, dtype=float).ravel()
        for i in range(S.size):
            p.S[i] = S[i]
        p.k_res = 1e-12
        p.plane_stress = int(bool(getattr(mat, "planeStress", False)) and self.dim == 2)
        return p

    # ---- assembly ----------------------------------------------------------
    def _assemble_damage(self):
        """Kd, Fd and psi+ with the History max (_phasefield.py:494-573)."""
        dm = self.dmesh
        u, _ = self._state()
        g = dm.main
        from .mesh import NPG, MatrixType

        nPg = NPG[(g.elemType, MatrixType.mass)]
        if self.__Kd is None:
            self.__Kd = CsrOperator(dm, 1)
            self.__Fd = torch.zeros(self.mesh.Nn, dtype=torch.float64, device=_dev())
            self.__psiP = torch.zeros(g.Ne * nPg, dtype=torch.float64, device=_dev())
        self.__Kd.vals64.zero_()
        self.__Fd.zero_()
        p = self._params()
        H_old = self.__psiP_old
        _lib.check(_lib.load().gfea_pf_damage(g.code, _lib.ptr(dm.coord), _lib.ptr(g.connect), g.Ne,
                                              _lib.ptr(dm.node_ptr), _lib.ptr(dm.rank), _lib.ptr(u),
                                              __import__("ctypes").byref(p), _lib.ptr(H_old),
                                              _lib.ptr(self.__psiP), _lib.ptr(self.__Kd.vals64),
                                              _lib.ptr(self.__Fd), _lib.stream()), "phase-field damage")
        self.__updatedDamage = True

    def _assemble_elastic(self):
        """Degraded stiffness g(d) cP + cM (_phasefield.py:444-482)."""
        dm = self.dmesh
        u, d = self._state()
        g = dm.main
        if self.__Ku is None:
            self.__Ku = CsrOperator(dm, self.dim, translation_invariant=True)
        self.__Ku.vals64.zero_()
        p = self._params()
        _lib.check(_lib.load().gfea_pf_elastic(g.code, _lib.ptr(dm.coord), _lib.ptr(g.connect), g.Ne,
                                               _lib.ptr(dm.node_ptr), _lib.ptr(dm.rank), _lib.ptr(u), _lib.ptr(d),
                                               __import__("ctypes").byref(p), _lib.F64,
                                               _lib.ptr(self.__Ku.vals64), _lib.stream()), "phase-field elastic")
        self.__updatedDisplacement = True

    def Get_K_C_M_F(self, problemType=None):
        import scipy.sparse as sp

        pt = self._check_pt_raw(problemType) if problemType is not None else "elastic"
        if pt == "elastic":
            if not self.__updatedDisplacement or self.__Ku is None:
                self._assemble_elastic()
            K = self.__Ku.to_scipy()
            return K, sp.csr_matrix(K.shape), sp.csr_matrix(K.shape), sp.csr_matrix((K.shape[0], 1))
        if not self.__updatedDamage or self.__Kd is None:
            self._assemble_damage()
        K = self.__Kd.to_scipy()
        F = sp.csr_matrix(self.__Fd.cpu().numpy().reshape(-1, 1))
        return K, sp.csr_matrix(K.shape), sp.csr_matrix(K.shape), F

    # ---- staggered scheme (_phasefield.py:303-432) ----------------------------
    def _energy(self, op, x, dofs=None):
        return reaction_energy(op, x, None)[1]

    def Solve(self, tolConv: float = 1.0, maxIter: int = 500, convOption: int = 2):
        assert 0 < tolConv <= 1, "tolConv must be between 0 and 1."
        assert maxIter > 1, "Must be > 1."
        assert convOption in (0, 1, 2, 3), "convOption must be 0, 1, 2 or 3"
        import time

        tic = time.perf_counter()
        u, d = self._state()
        old_damage = d.clone()
        Niter = 0
        converged = False
        convIter = 0.0
        fu = self._neumann_vec("elastic")
        while not converged and Niter < maxIter:
            Niter += 1
            d_n = d.clone()
            u_n = u.clone()
            if convOption in (1, 2):
                E_n = self._psi_crack()
                if convOption == 2:
                    E_n += self._psi_elas() - self._psi_ext(fu)
            # damage
            self._assemble_damage()
            bd = self.__Fd + self._neumann_vec("damage")
            if self.phaseFieldModel.solver == "BoundConstrain":
                # d_n <= d <= 1 (1 - eps where d_n reached 1), _phasefield.py:148-163
                lb = torch.where(d >= 1, torch.full_like(d, 1 - np.finfo(float).eps), d)
                d_new = self._solve_bounded(self.__Kd, bd, "damage", lb, torch.ones_like(d), x0=d)
            else:
                d_new = self._solve_system(self.__Kd, bd, "damage", x0=d)
            d.copy_(d_new)
            self.__updatedDisplacement = False
            # displacement
            self._assemble_elastic()
            u_new = self._solve_system(self.__Ku, fu, "elastic", x0=u)
            u.copy_(u_new)
            self.__updatedDamage = False
            if convOption == 0:
                convIter = max_abs_diff(d, d_n)
            elif convOption in (1, 2):
                E_np1 = self._psi_crack()
                if convOption == 2:
                    E_np1 += self._psi_elas() - self._psi_ext(fu)
                convIter = abs(E_n - E_np1) if E_np1 == 0 else abs((E_n - E_np1) / E_np1)
            else:
                diffU = (u - u_n).abs()
                nz = u != 0
                diffU[nz] = diffU[nz] / u[nz].abs()
                diffD = (d - d_n).abs()
                nz = d != 0
                diffD[nz] = diffD[nz] / d[nz].abs()
                convU = float(diffU.sum())
                convD = float(diffD.sum())
                convIter = max(convD, convU)
            dmax = float(d.max())
            if tolConv == 1 or dmax == 0:
                converged = True
            elif convOption == 3:
                converged = (convD <= tolConv) and (convU <= tolConv * 0.999)
            else:
                converged = convIter <= tolConv
        if self.phaseFieldModel.solver == "HistoryDamage":
            torch.maximum(d, old_damage, out=d)
        self.__Niter = Niter
        self.__convIter = convIter
        self.__timeIter = time.perf_counter() - tic
        return u.cpu().numpy(), d.cpu().numpy(), converged

    def _psi_crack(self) -> float:
        if not self.__updatedDamage or self.__Kd is None:
            self._assemble_damage()
        return self._energy(self.__Kd, self._state()[1])

    def _psi_elas(self) -> float:
        if not self.__updatedDisplacement or self.__Ku is None:
            self._assemble_elastic()
        return self._energy(self.__Ku, self._state()[0])

    def _psi_ext(self, fu: torch.Tensor) -> float:
        return float(torch.dot(self._state()[0], fu))

    @property
    def staggered_iterations(self) -> int:
        """Staggered iterations of the last Solve (the "Niter" of its saved
        iteration dict)."""
        return self.__Niter

    def Save_Iter(self, iter: Optional[dict] = None) -> dict:
        """Commit the History field (_phasefield.py:613-630) and store u, d."""
        it = {} if iter is None else iter
        it["Niter"] = self.__Niter
        it["timeIter"] = self.__timeIter
        it["convIter"] = self.__convIter
        if self.phaseFieldModel.solver == "History" and self.__psiP is not None:
            if self.__psiP_old is None:
                self.__psiP_old = self.__psiP.clone()
            else:
                self.__psiP_old.copy_(self.__psiP)
        it["displacement"] = self.displacement
        it["damage"] = self.damage
        return super().Save_Iter(it)

    def Set_Iter(self, iter: int = -1, resetAll: bool = False) -> dict:
        """Restore u and d of a saved iteration (_phasefield.py:632-657); with
        resetAll the History field restarts from psi+ of that state."""
        results = self.Get_results(iter)
        self._Set_solutions("damage", results["damage"])
        self._Set_solutions("elastic", results["displacement"])
        if resetAll and self.phaseFieldModel.solver == "History":
            self.__psiP_old = None
            self._assemble_damage()
            self.__psiP_old = self.__psiP.clone()
            self.__updatedDamage = False
        return results

    def Calc_Reaction(self, dofs=None, problemType=None) -> np.ndarray:
        """Ku[dofs] @ u on the current degraded stiffness (_simu.py:212-260)."""
        pt = self._check_pt_raw(problemType) if problemType is not None else "damage"
        if pt == "damage":
            if self.__Kd is None:
                self._assemble_damage()
            op, x = self.__Kd, self._state()[1]
        else:
            if self.__Ku is None:
                self._assemble_elastic()
            op, x = self.__Ku, self._state()[0]
        _, _, Ax = reaction_energy(op, x, None)
        Ax = Ax.cpu().numpy()
        return Ax if dofs is None else Ax[np.asarray(dofs)]

    def reaction_sum(self, dofs: torch.Tensor) -> float:
        """sum Ku[dofs] @ u reduced on the device (no host copy of the vector)."""
        return reaction_energy(self.__Ku, self._state()[0], dofs)[0]

    # ---- results (_phasefield.py:659-760) ------------------------------------
    def Results_Available(self) -> list:
        comps = ["x", "y"] if self.dim == 2 else ["x", "y", "z"]
        tens = ["xx", "yy", "xy"] if self.dim == 2 else ["xx", "yy", "zz", "yz", "xz", "xy"]
        return (["displacement", "displacement_norm"] + [f"u{c}" for c in comps] + [f"S{t}" for t in tens] +
                [f"E{t}" for t in tens] + ["Svm", "Stress", "Evm", "Strain", "damage", "psiP", "Psi_Crack", "Wdef"])

    def Result_device(self, result: str, nodeValues: bool = True):
        """PhaseField.Result on the device: the degraded stress g(d) sig+ +
        sig- results, the strains, psiP (the History-max'ed psi+ at the mass
        Gauss points), the damage and the two energies."""
        self._check_result(result)
        u, d = self._state()
        if result == "Psi_Crack":
            return 0.0 if float(torch.linalg.norm(d)) == 0 else self._psi_crack()
        if result == "Wdef":
            return 0.0 if float(torch.linalg.norm(u)) == 0 else self._psi_elas()
        if result == "damage":
            values = d
        elif result in ("ux", "uy", "uz", "displacement", "displacement_norm"):
            values = self._displacement_result(u, result)
        elif result == "psiP":
            H = None
            if self.phaseFieldModel.solver == "History":
                from .mesh import NPG, MatrixType

                g = self.dmesh.main
                H = self.__psiP_old
                if H is None:  # nothing committed yet: the reference's zero history
                    H = torch.zeros(g.Ne * NPG[(g.elemType, MatrixType.mass)], dtype=torch.float64, device=_dev())
            values = self._element_fields(u, gauss=1, psiP=True, pf=self._params(), d=d, H_old=H)["psiP"]
        else:
            p = self._params()
            values = self._strain_stress_result(
                result, lambda e, s, v: self._element_fields(u, strain=e, stress=s, vm=v, pf=p, d=d))
        return self._reshape_values(values, nodeValues)
