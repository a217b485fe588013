"""Drop-in GPU subclasses of EasyFEA's own simulation classes.

``GpuElastic`` and ``GpuPhaseField`` derive from the reference's
``EasyFEA.Simulations.Elastic`` and ``EasyFEA.Simulations.PhaseField`` and
override the seams the reference documents for new simulations
(``docs/howto/new_simulation.md:92-130``): ``Assembly``
(``EasyFEA/Simulations/_simu.py:1104-1144``), ``_Solver_Solve_problemType``
(``_simu.py:1532-1550``) and, for the phase field, ``Solve`` and
``Get_K_C_M_F`` (``EasyFEA/Simulations/_phasefield.py:248-269, 303-432``);
``Result`` computes the strain, stress and energy results on the device.
Everything else -- meshes, materials, boundary conditions, the remaining
results -- is the reference's code, so an EasyFEA script switches by
replacing ``Simulations.Elastic(mesh, mat)`` with ``GpuElastic(mesh, mat)``.

What runs on the GPU:

* ``Assembly``: K (and M, for the reference's C = coefK K + coefM M) with
  ``gfea_assemble_elastic`` / ``gfea_assemble_mass``, returned as scipy CSR
  matrices with the reference's exact layout, so every reference path that
  reads ``Get_K_C_M_F`` (reactions, energies, time schemes) sees them.
* ``_Solver_Solve_problemType`` for linear problems without Lagrange
  conditions: the static solve (the reference's own Neumann and Dirichlet
  conditions, ``Bc_dofs_Neumann`` / ``Bc_values_Neumann`` summed as
  ``_Solver_Apply_Neumann`` sums them, and ``Bc_dofs_Dirichlet`` /
  ``Bc_values_Dirichlet``) and the time-stepping solves of the parabolic and
  hyperbolic schemes (Newmark, HHT, midpoint, Euler; ``_simu.py:1291-1456``,
  ``Solvers.py:69-182``: the operator coefK K + coefC C + coefM M formed on
  the device, the right-hand side from the reference's own
  ``_Solver_Apply_Neumann``), all with the library's PCG and the previous
  solution as the initial guess (``Get_x0``).  Newton and Lagrange
  multipliers go to the reference's solver with the GPU-assembled matrices.
* ``GpuPhaseField.Solve``: the staggered loop on the device (split, history,
  damage and degraded elastic systems, both solves), started from the
  reference's current u, d and committed history field and written back to
  it, so ``Save_Iter``, ``Set_Iter`` and ``Calc_Reaction`` keep their
  meaning.

Materials: isotropic elastic laws (homogeneous or with a per-element Young's
modulus), homogeneous transversely isotropic and anisotropic laws and, for the
phase field, a homogeneous material with the Bourdin / Amor / Miehe / He
(isotropic) and AnisotStrain / AnisotStress splits, AT1 / AT2 and the
History / HistoryDamage / BoundConstrain solvers; element groups of type
SEG2, SEG3, SEG4, SEG5, TRI3, TRI6, TRI10, TRI15, QUAD4, QUAD8, QUAD9, HEXA8,
HEXA20, HEXA27, TETRA4, TETRA10, PRISM6, PRISM15 and PRISM18.  Other models raise ``NotImplementedError`` at construction.

EasyFEA must be importable (it imports gmsh at start-up).
"""

from __future__ import annotations

import time
import numpy as np
import scipy.sparse as sp
import torch

import EasyFEA  # noqa: F401  (the reference package this module binds to)
from EasyFEA import Models as _RefModels
from EasyFEA import Simulations as _RefSimulations
from EasyFEA.Simulations.Solvers import AlgoType as _AlgoType

from . import mesh as _gmesh
from . import simulations as _engine
from .models import Elastic as _ElasticModels
from .models import PhaseField as _PhaseFieldModel

__all__ = ["GpuElastic", "GpuPhaseField", "to_gpu_mesh"]


def to_gpu_mesh(ref_mesh) -> _gmesh.Mesh:
    """The library's mesh for an EasyFEA ``Mesh``: same coordinates, same
    connectivity per element group (groups of types the GPU path does not
    handle, such as POINT, are left out; the main group must be handled)."""
    coord = np.ascontiguousarray(ref_mesh.coord, dtype=np.float64)
    groups = {}
    for g in ref_mesh.dict_groupElem.values():
        name = str(getattr(g.elemType, "value", g.elemType))
        try:
            et = _gmesh.ElemType(name)
        except ValueError:
            if g.dim == ref_mesh.dim:
                raise NotImplementedError(f"element type {name} is not handled by the GPU path")
            continue
        groups[et] = _gmesh.GroupElem(et, np.ascontiguousarray(g.connect, dtype=np.int64), coord)
    return _gmesh.Mesh(groups)


def _gpu_material(mat):
    """The library's law for an EasyFEA elastic material: isotropic
    (homogeneous or per-element E), transversely isotropic or anisotropic
    (homogeneous)."""
    thickness = float(getattr(mat, "thickness", 1.0))
    if isinstance(mat, _RefModels.Elastic.TransverselyIsotropic):
        if np.ndim(mat.El) or np.ndim(mat.Et) or np.ndim(mat.Gl):
            raise NotImplementedError("the GPU path takes a homogeneous transversely isotropic law")
        return _ElasticModels.TransverselyIsotropic(mat.dim, float(mat.El), float(mat.Et), float(mat.Gl),
                                                    float(mat.vl), float(mat.vt), axis_l=mat.axis_l,
                                                    axis_t=mat.axis_t, planeStress=bool(mat.planeStress),
                                                    thickness=thickness)
    if isinstance(mat, _RefModels.Elastic.Anisotropic):
        C = np.asarray(mat.C, dtype=np.float64)
        if C.ndim != 2:
            raise NotImplementedError("the GPU path takes a homogeneous anisotropic law")
        # the reference's C is already Kelvin-Mandel in x, y, z
        return _ElasticModels.Anisotropic(mat.dim, C, False, thickness=thickness)
    if not isinstance(mat, _RefModels.Elastic.Isotropic):
        raise NotImplementedError(f"the GPU path takes isotropic, transversely isotropic and anisotropic "
                                  f"elastic laws, not {type(mat).__name__}")
    E = mat.E
    E = float(E) if np.ndim(E) == 0 else np.asarray(E, dtype=np.float64)
    thickness = float(getattr(mat, "thickness", 1.0))
    return _ElasticModels.Isotropic(mat.dim, E=E, v=float(mat.v), planeStress=bool(mat.planeStress),
                                    thickness=thickness)


def _neumann(simu, problemType) -> np.ndarray:
    """The reference's Neumann vector (COO sum of its Neumann conditions,
    _simu.py:1750-1756) without the assembled F, which is zero for the
    elastic problem and added by the library for the damage problem (Fd);
    read directly so that no host copy of the matrices is made."""
    dofs = np.asarray(simu.Bc_dofs_Neumann(problemType), dtype=np.int64)
    vals = np.asarray(simu.Bc_values_Neumann(problemType), dtype=np.float64)
    n = simu.mesh.Nn * simu.Get_dof_n(problemType)
    return np.bincount(dofs, weights=vals, minlength=n) if dofs.size else np.zeros(n)


class _DirichletBC:
    """Dirichlet values of the reference handed to the library's solver."""

    def __init__(self, dofs, values):
        self.dofs = np.asarray(dofs, dtype=np.int64)
        self.values = np.asarray(values, dtype=np.float64)


class GpuElastic(_RefSimulations.Elastic):
    """``EasyFEA.Simulations.Elastic`` with assembly and static solves on the GPU.

    ``precision``: "fp64" (default) or "mixed" (FP32 iteration with FP64
    reliable updates); ``rtol``: relative residual of the PCG."""

    def __init__(self, mesh, model, folder: str = "", verbosity: bool = False, precision: str = "fp64",
                 rtol: float = 1e-10):
        self._gpu = None
        self._gpu_mesh_of = None
        self._gpu_dirty = True
        self.precision = precision
        self.rtol = rtol
        super().__init__(mesh, model, folder=folder, verbosity=verbosity)
        _gpu_material(model)  # reject unsupported laws now

    # -- engine ---------------------------------------------------------------
    def Need_Update(self, value: bool = True) -> None:
        super().Need_Update(value)
        if value:
            self._gpu_dirty = True

    def _engine(self) -> _engine.Elastic:
        """The library's simulation on the same mesh and material (rebuilt
        when the mesh or the material changed)."""
        if self._gpu is None or self._gpu_mesh_of is not self.mesh:
            self._gpu = _engine.Elastic(to_gpu_mesh(self.mesh), _gpu_material(self.material))
            self._gpu_mesh_of = self.mesh
            self._gpu_dirty = True
        if self._gpu_dirty:
            eng = self._gpu
            eng.model = _gpu_material(self.material)
            eng.precision = self.precision
            eng.rtol = self.rtol
            eng.Need_Update()
            self._gpu_dirty = False
        return self._gpu

    # -- seams ----------------------------------------------------------------
    def Assembly(self, problemType):
        """K, C = coefK K + coefM M, M and F (zero) as the reference assembles
        them (_elastic.py:123-152, _simu.py:1104-1144), computed on the GPU."""
        eng = self._engine()
        rho = self.rho
        if np.ndim(rho) != 0:
            raise NotImplementedError("the GPU mass matrix takes a homogeneous density")
        if float(rho) != eng.rho:
            eng.rho = float(rho)
            eng.Need_Update()
        K, _, M, F = eng.Get_K_C_M_F()
        coefK = getattr(self, "_Elastic__coefK", 0.0)
        coefM = getattr(self, "_Elastic__coefM", 0.0)
        C = sp.csr_matrix((coefK * K.data + coefM * M.data, K.indices, K.indptr), shape=K.shape)
        return K, C, M, F

    def _gpu_solvable(self, problemType) -> bool:
        return not self.isNonLinear and len(self.Bc_Lagrange) == 0

    def _time_operator(self, eng):
        """A = coefK K + coefC C + coefM M of the time scheme
        (_simu.py:1399-1456, Solvers.py:69-182) on the device, with the
        Rayleigh C = rK K + rM M: one linear combination of the K and M values,
        which share the CSR pattern."""
        from .device import CsrOperator

        cK, cC, cM = self._Solver_Get_K_C_M_coefs_for_time_scheme()
        rK = getattr(self, "_Elastic__coefK", 0.0)
        rM = getattr(self, "_Elastic__coefM", 0.0)
        a, m = cK + cC * rK, cM + cC * rM
        K, M = eng.K_device, eng._mass()
        if getattr(self, "_gpu_A", None) is None or self._gpu_A.dmesh is not K.dmesh:
            self._gpu_A = CsrOperator(K.dmesh, K.dof_n)
        A = self._gpu_A
        torch.mul(K.vals64, a, out=A.vals64)
        A.vals64.add_(M.vals64, alpha=m)
        # node block rows of A sum to zero only without the mass term
        A.translation_invariant = m == 0.0
        return A

    def _Solver_Solve_problemType(self, problemType):
        """The static and time-stepping linear solves on the GPU (elliptic,
        parabolic and every hyperbolic scheme): the right-hand side is the
        reference's own (_Solver_Apply_Neumann, which adds the scheme's
        history terms with the GPU-assembled matrices), the operator
        coefK K + coefC C + coefM M is formed on the device, the velocity and
        acceleration are updated by the reference's _Solver_Update_solutions."""
        if not self._gpu_solvable(problemType):
            return super()._Solver_Solve_problemType(problemType)
        eng = self._engine()
        dofs = self.Bc_dofs_Dirichlet(problemType)
        vals = self.Bc_values_Dirichlet(problemType)
        if self.algo == _AlgoType.elliptic:
            b_host = _neumann(self, problemType)
            op = eng.K_device
        else:
            b_host = np.asarray(self._Solver_Apply_Neumann(problemType).toarray(), dtype=np.float64).ravel()
            op = self._time_operator(eng)
            if self.algo == _AlgoType.euler_explicit:  # the unknown is a^n: zero on constrained DOFs
                vals = np.zeros_like(np.asarray(vals, dtype=np.float64))
        eng._dirichlet[eng.problemType] = [_DirichletBC(dofs, vals)]
        b = torch.as_tensor(b_host, device=_engine._dev())
        x0 = torch.as_tensor(np.ascontiguousarray(self.Get_x0(problemType), dtype=np.float64),
                             device=_engine._dev())
        u = eng._solve_system(op, b, eng.problemType, x0=x0).cpu().numpy()
        self.last_solve = eng.last_solve
        solutions = self._Solver_Update_solutions(problemType, u)
        self._Set_solutions(problemType, *solutions)
        return solutions[0]


    def Result(self, result: str, nodeValues: bool = True, iter=None):
        """Elastic.Result (_elastic.py:229-320) with the strain, stress, von
        Mises, energy and ZZ1 results computed on the device from the current
        displacement; the velocity, acceleration and displacement-matrix
        results are the reference's own."""
        if iter is not None:
            self.Set_Iter(iter)
        eng = self._engine()
        if result not in _DEVICE_RESULTS or result not in self.Results_Available():
            return super().Result(result, nodeValues)
        eng._Set_solutions(eng.problemType, self.displacement)
        return eng.Result(result, nodeValues)


# the results the device computes (the displacement ones stay on the host)
_DEVICE_RESULTS = frozenset(["Sxx", "Syy", "Szz", "Syz", "Sxz", "Sxy", "Exx", "Eyy", "Ezz", "Eyz", "Exz", "Exy",
                             "Svm", "Stress", "Evm", "Strain", "Wdef", "Wdef_e", "ZZ1", "ZZ1_e", "psiP",
                             "Psi_Crack"])


class GpuPhaseField(_RefSimulations.PhaseField):
    """``EasyFEA.Simulations.PhaseField`` with the staggered scheme on the GPU.

    ``precision``: "fp64" (default) or "mixed"; ``rtol``: relative residual
    of each PCG solve."""

    def __init__(self, mesh, model, folder: str = "", verbosity: bool = False, precision: str = "fp64",
                 rtol: float = 1e-12):
        self._gpu = None
        self._gpu_mesh_of = None
        self._gpu_state = None    # (u, d) the device holds, as host copies
        self._gpu_history = None  # committed history the device holds
        self.precision = precision
        self.rtol = rtol
        super().__init__(mesh, model, folder=folder, verbosity=verbosity)
        self._gpu_model(model)  # reject unsupported models now

    @staticmethod
    def _gpu_model(pfm):
        mat = pfm.material
        split = str(getattr(pfm.split, "value", pfm.split))
        regu = str(getattr(pfm.regularization, "value", pfm.regularization))
        solver = str(getattr(pfm.solver, "value", pfm.solver))
        if isinstance(mat, _RefModels.Elastic.Isotropic):
            if np.ndim(mat.E) != 0:
                raise NotImplementedError("the GPU phase field takes a homogeneous material")
            splits = ("Bourdin", "Amor", "Miehe", "He", "AnisotStrain", "AnisotStress")
        else:
            splits = ("Bourdin", "AnisotStrain", "AnisotStress")
        if split not in splits or regu not in ("AT1", "AT2") or solver not in ("History", "HistoryDamage", "BoundConstrain"):
            raise NotImplementedError(f"GPU phase field: {type(mat).__name__}, split {split}, {regu}, solver {solver}")
        A = getattr(pfm, "A", None)
        return _PhaseFieldModel(_gpu_material(mat), split, regu, float(pfm.Gc), float(pfm.l0), solver=solver,
                                A=None if A is None else np.asarray(A, dtype=np.float64))

    def Need_Update(self, value: bool = True) -> None:
        """The reference's flag (model or mesh changed); the device re-reads
        the model and re-assembles both systems at their next use."""
        super().Need_Update(value)
        if value and getattr(self, "_gpu", None) is not None:
            self._gpu_model_dirty = True

    def _engine(self) -> _engine.PhaseField:
        if self._gpu is None or self._gpu_mesh_of is not self.mesh:
            self._gpu = _engine.PhaseField(to_gpu_mesh(self.mesh), self._gpu_model(self.phaseFieldModel))
            self._gpu_mesh_of = self.mesh
            self._gpu_state = None
            self._gpu_history = None
            self._gpu_model_dirty = False
        eng = self._gpu
        if getattr(self, "_gpu_model_dirty", False):
            eng.model = self._gpu_model(self.phaseFieldModel)
            eng.Need_Update()
            self._gpu_model_dirty = False
        eng.precision = self.precision
        eng.rtol = self.rtol
        return eng

    def _push_state(self, eng):
        """The reference's boundary conditions to the device, and its u, d and
        committed history where they differ from the device's copies (the
        matrices the device caches stay valid otherwise, as the reference's
        cached ones do: the degraded stiffness of the last elastic solve was
        assembled from the previous displacement iterate)."""
        pts = self.ProblemTypes
        for pt, key in ((pts.elastic, "elastic"), (pts.damage, "damage")):
            eng._dirichlet[key] = [_DirichletBC(self.Bc_dofs_Dirichlet(pt), self.Bc_values_Dirichlet(pt))]
            eng._neumann_vec(key).copy_(torch.as_tensor(_neumann(self, pt)))
        u_ref = np.ascontiguousarray(self.displacement, dtype=np.float64)
        d_ref = np.ascontiguousarray(self.damage, dtype=np.float64)
        synced = getattr(self, "_gpu_state", None)
        if synced is None or not (np.array_equal(synced[0], u_ref) and np.array_equal(synced[1], d_ref)):
            u, d = eng._state()
            u.copy_(torch.as_tensor(u_ref))
            d.copy_(torch.as_tensor(d_ref))
            eng.Need_Update()
            self._gpu_state = (u_ref.copy(), d_ref.copy())
        H = getattr(self, "_PhaseField__old_psiP_e_pg", None)
        H = None if H is None or np.size(H) == 0 else np.asarray(H, dtype=np.float64)
        Hs = getattr(self, "_gpu_history", None)
        if (H is None) != (Hs is None) or (H is not None and not np.array_equal(H, Hs)):
            eng.set_history(H)
            self._gpu_history = None if H is None else H.copy()

    def Solve(self, tolConv=1.0, maxIter=500, convOption=2):
        """Staggered scheme (_phasefield.py:303-432) on the device; returns
        (u, d, converged) as the reference does."""
        assert tolConv > 0 and tolConv <= 1, "tolConv must be between 0 and 1."
        assert maxIter > 1, "Must be > 1."
        eng = self._engine()
        self._push_state(eng)
        t0 = time.perf_counter()
        u, d, converged = eng.Solve(tolConv, maxIter, convOption)
        pts = self.ProblemTypes
        self._Set_solutions(pts.elastic, u)
        self._Set_solutions(pts.damage, d)
        self._gpu_state = (np.array(u, dtype=np.float64), np.array(d, dtype=np.float64))
        # the reference's per-solve record, read by its Save_Iter
        self._PhaseField__Niter = eng.staggered_iterations
        self._PhaseField__convIter = eng._PhaseField__convIter
        self._PhaseField__timeIter = time.perf_counter() - t0
        self._PhaseField__tolConv = tolConv
        self._PhaseField__convOption = convOption
        self._PhaseField__maxIter = maxIter
        H = eng.psiP_device
        if H is not None:
            nPg = H.numel() // self.mesh.Ne
            self._PhaseField__psiP_e_pg = H.cpu().numpy().reshape(self.mesh.Ne, nPg)
        # the matrices the reference caches belong to the new state
        self._PhaseField__updatedDamage = False
        self._PhaseField__updatedDisplacement = False
        return u, d, converged

    def Result(self, result: str, nodeValues: bool = True, iter=None):
        """PhaseField.Result (_phasefield.py:682-760) with the degraded
        stress, strain, von Mises, psiP and energy results computed on the
        device from the reference's current u, d and committed history."""
        if iter is not None:
            self.Set_Iter(iter)
        if result not in _DEVICE_RESULTS or result not in self.Results_Available():
            return super().Result(result, nodeValues)
        eng = self._engine()
        self._push_state(eng)
        return eng.Result(result, nodeValues)

    def Get_K_C_M_F(self, problemType=None):
        """The damage system (Kd, Fd) or the degraded stiffness at the current
        state, assembled on the device (_phasefield.py:248-269)."""
        if problemType is None:
            problemType = self.ProblemTypes.elastic
        key = "elastic" if problemType == self.ProblemTypes.elastic else "damage"
        eng = self._engine()
        self._push_state(eng)
        return eng.Get_K_C_M_F(key)
