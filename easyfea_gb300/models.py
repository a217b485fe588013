"""Material models mirroring EasyFEA's ``Models`` API for the GPU path.

``Elastic.Isotropic`` follows EasyFEA/Models/Elastic/_laws.py:333-482 (Lame
constants, plane-stress lambda, Kelvin-Mandel stiffness) and accepts a scalar
or per-element Young's modulus (Models/_utils.py:69-108).  ``PhaseField``
follows EasyFEA/Models/_phasefield.py:38-251 (splits, regularisations,
irreversibility solver, diffusion tensor A).  Changing a parameter notifies the
simulations using the model so they re-assemble (the reference's
``Need_Update`` observers, EasyFEA/Utilities/_observers.py).
"""

from __future__ import annotations

from enum import Enum
from typing import Optional, Union

import numpy as np


class _Observable:
    def __init__(self):
        self._observers = []

    def _Add_observer(self, obs) -> None:
        if obs not in self._observers:
            self._observers.append(obs)

    def _Notify(self) -> None:
        for o in list(self._observers):
            o._Update(self)


def KelvinMandel_Matrix(dim: int, M: np.ndarray) -> np.ndarray:
    """Voigt -> Kelvin-Mandel scaling (EasyFEA/Models/_utils.py:111-152)."""
    r2 = np.sqrt(2)
    if dim == 2:
        T = np.array([[1, 1, r2], [1, 1, r2], [r2, r2, 2]])
    else:
        T = np.ones((6, 6))
        T[3:, :3] = r2
        T[:3, 3:] = r2
        T[3:, 3:] = 2
    return M * T


class _Elastic(_Observable):
    def __init__(self, dim: int, thickness: float, planeStress: bool):
        super().__init__()
        assert dim in (2, 3), "dim must be 2 or 3"
        assert thickness > 0, "thickness must be > 0"
        self.__dim = dim
        self.__thickness = float(thickness)
        self.__planeStress = bool(planeStress) if dim == 2 else False

    @property
    def dim(self) -> int:
        return self.__dim

    @property
    def thickness(self) -> float:
        return self.__thickness if self.__dim == 2 else 1.0

    @thickness.setter
    def thickness(self, value: float):
        assert value > 0
        self.__thickness = float(value)
        self._Notify()

    @property
    def planeStress(self) -> bool:
        return self.__planeStress

    @planeStress.setter
    def planeStress(self, value: bool):
        self.__planeStress = bool(value)
        self._Notify()

    @property
    def coef(self) -> float:
        return float(np.sqrt(2))


class Elastic:
    """Namespace mirroring ``EasyFEA.Models.Elastic``."""

    class Isotropic(_Elastic):
        """Isotropic linear elastic material (EasyFEA/Models/Elastic/_laws.py:333-482)."""

        def __init__(self, dim: int, E=210000.0, v=0.3, planeStress=True, thickness=1.0):
            super().__init__(dim, thickness, planeStress)
            self.E = E
            self.v = v

        @property
        def E(self):
            return self.__E

        @E.setter
        def E(self, value):
            arr = np.asarray(value, dtype=float)
            assert np.all(arr > 0), "E must be > 0"
            self.__E = arr.copy() if arr.ndim else float(arr)
            self._Notify()

        @property
        def v(self) -> float:
            return self.__v

        @v.setter
        def v(self, value):
            assert -1 < float(value) < 0.5, "v must be in ]-1, 0.5["
            self.__v = float(value)
            self._Notify()

        @property
        def isHeterogeneous(self) -> bool:
            return np.ndim(self.__E) > 0

        def get_lambda(self):
            E, v = self.E, self.v
            lmbda = E * v / ((1 + v) * (1 - 2 * v))
            if self.dim == 2 and self.planeStress:
                lmbda = E * v / (1 - v**2)
            return lmbda

        def get_mu(self):
            return self.E / (2 * (1 + self.v))

        def get_bulk(self):
            return self.get_lambda() + 2 * self.get_mu() / self.dim

        @property
        def C(self) -> np.ndarray:
            """Kelvin-Mandel stiffness, (n,n) or (Ne,n,n) for a per-element E."""
            lmbda = np.asarray(self.get_lambda(), dtype=float)
            mu = np.asarray(self.get_mu(), dtype=float)
            n = 3 if self.dim == 2 else 6
            c = np.zeros(lmbda.shape + (n, n))
            if self.dim == 2:
                c[..., 0, 0] = c[..., 1, 1] = lmbda + 2 * mu
                c[..., 0, 1] = c[..., 1, 0] = lmbda
                c[..., 2, 2] = mu
            else:
                for i in range(3):
                    for j in range(3):
                        c[..., i, j] = lmbda
                    c[..., i, i] = lmbda + 2 * mu
                for i in range(3, 6):
                    c[..., i, i] = mu
            return KelvinMandel_Matrix(self.dim, c)

        @property
        def S(self) -> np.ndarray:
            """Kelvin-Mandel compliance C^-1."""
            return np.linalg.inv(self.C)

        def __str__(self) -> str:
            return f"Isotropic: E = {self.E}, v = {self.v}, dim = {self.dim}"

    class TransverselyIsotropic(_Elastic):
        """Transversely isotropic law (EasyFEA/Models/Elastic/_laws.py:513-717):
        longitudinal axis ``axis_l``, transverse axis ``axis_t``; the
        Kelvin-Mandel compliance and stiffness in the material frame (L, T,
        R), turned to x, y, z, then reduced to 2D by plane stress (the 3x3
        block of the compliance, inverted) or plane strain (the 3x3 block of
        the stiffness)."""

        def __init__(self, dim: int, El: float, Et: float, Gl: float, vl: float, vt: float,
                     axis_l=(1, 0, 0), axis_t=(0, 1, 0), planeStress: bool = True, thickness: float = 1.0):
            super().__init__(dim, thickness, planeStress)
            assert El > 0 and Et > 0 and Gl > 0, "moduli must be > 0"
            assert -1 <= vl <= 0.5 and -1 <= vt <= 1, "Poisson ratios out of range"
            self.El, self.Et, self.Gl, self.vl, self.vt = float(El), float(Et), float(Gl), float(vl), float(vt)
            self.axis_l, self.axis_t = _unit_axes(axis_l, axis_t)

        @property
        def Gt(self) -> float:
            return self.Et / (2 * (1 + self.vt))

        @property
        def kt(self) -> float:
            El, Et, vt, vl = self.El, self.Et, self.vt, self.vl
            return El * Et / (2 * (1 - vt) * El - 4 * vl**2 * Et)

        @property
        def isHeterogeneous(self) -> bool:
            return False

        def _material_frame(self):
            El, Et, Gl, vl, vt, Gt, kt = self.El, self.Et, self.Gl, self.vl, self.vt, self.Gt, self.kt
            s = np.zeros((6, 6))
            s[0, :3] = [1 / El, -vl / El, -vl / El]
            s[1, :3] = [-vl / El, 1 / Et, -vt / Et]
            s[2, :3] = [-vl / El, -vt / Et, 1 / Et]
            s[3, 3] = 1 / (2 * Gt)
            s[4, 4] = s[5, 5] = 1 / (2 * Gl)
            c = np.zeros((6, 6))
            c[0, :3] = [El + 4 * vl**2 * kt, 2 * kt * vl, 2 * kt * vl]
            c[1, :3] = [2 * kt * vl, kt + Gt, kt - Gt]
            c[2, :3] = [2 * kt * vl, kt - Gt, kt + Gt]
            c[3, 3] = 2 * Gt
            c[4, 4] = c[5, 5] = 2 * Gl
            return c, s

        def _laws(self):
            c, s = self._material_frame()
            Q = km_rotation(self.axis_l, self.axis_t)
            c, s = Q @ c @ Q.T, Q @ s @ Q.T
            if self.dim == 3:
                return c, s
            x = [0, 1, 5]
            if self.planeStress:
                s2 = s[np.ix_(x, x)]
                return np.linalg.inv(s2), s2
            c2 = c[np.ix_(x, x)]
            return c2, np.linalg.inv(c2)

        @property
        def C(self) -> np.ndarray:
            return self._laws()[0]

        @property
        def S(self) -> np.ndarray:
            return self._laws()[1]

        def __str__(self) -> str:
            return f"TransverselyIsotropic: El = {self.El}, Et = {self.Et}, Gl = {self.Gl}, vl = {self.vl}, vt = {self.vt}"

    class Anisotropic(_Elastic):
        """Anisotropic law from its stiffness in the anisotropy basis
        (EasyFEA/Models/Elastic/_laws.py:1111-1270): Voigt or Kelvin-Mandel,
        (3, 3) in 2D or (6, 6), turned from (axis1, axis2) to x, y, z; 2D
        matrices are taken as the in-plane block of the 3D law."""

        def __init__(self, dim: int, C: np.ndarray, useVoigtNotation: bool, axis1=(1, 0, 0), axis2=(0, 1, 0),
                     thickness: float = 1.0):
            super().__init__(dim, thickness, False)
            self.axis1, self.axis2 = _unit_axes(axis1, axis2)
            self.Set_C(C, useVoigtNotation)

        def Set_C(self, C: np.ndarray, useVoigtNotation: bool = True) -> None:
            C = np.asarray(C, dtype=float)
            assert C.shape in ((3, 3), (6, 6)), "C must be a (3,3) or (6,6) matrix"
            assert np.linalg.norm(C - C.T) <= 1e-12 * np.linalg.norm(C), "The matrix is not symmetrical."
            d = 3 if C.shape[0] == 6 else 2
            Cm = KelvinMandel_Matrix(d, C) if useVoigtNotation else C.copy()
            x = [0, 1, 5]
            if d == 2:
                C6 = np.zeros((6, 6))
                C6[np.ix_(x, x)] = Cm
            else:
                # a (6, 6) matrix is turned as given, Voigt or not, as the
                # reference does (_laws.py:1239-1240)
                C6 = C.copy()
            Q = km_rotation(self.axis1, self.axis2)
            Cg = Q @ C6 @ Q.T
            self._C = Cg[np.ix_(x, x)] if self.dim == 2 else Cg
            self._Notify()

        @property
        def isHeterogeneous(self) -> bool:
            return False

        @property
        def C(self) -> np.ndarray:
            return self._C.copy()

        @property
        def S(self) -> np.ndarray:
            return np.linalg.inv(self._C)

        def __str__(self) -> str:
            return f"Anisotropic:\n{self._C}"


def _unit_axes(a1, a2):
    a1 = np.asarray(a1, dtype=float).reshape(3)
    a2 = np.asarray(a2, dtype=float).reshape(3)
    assert abs(a1 @ a2) <= 1e-12, "axis1 and axis2 must be perpendicular"
    return a1 / np.linalg.norm(a1), a2 / np.linalg.norm(a2)


# Kelvin-Mandel basis of symmetric 3x3 tensors: 11, 22, 33, sqrt2 23, sqrt2 13, sqrt2 12
_KM_PAIRS = ((0, 0), (1, 1), (2, 2), (1, 2), (0, 2), (0, 1))


def km_rotation(axis1, axis2) -> np.ndarray:
    """6x6 Kelvin-Mandel matrix Q of the change of basis from the material
    frame (axis1, axis2, axis1 x axis2) to x, y, z: a symmetric tensor's
    Kelvin-Mandel vector a maps to Q a, a stiffness or compliance M to
    Q M Q^T (Q is orthogonal).  Column I is the Kelvin-Mandel vector of
    R E_I R^T, E_I the unit tensor of component I and R the rotation whose
    columns are the material axes."""
    a1, a2 = _unit_axes(axis1, axis2)
    R = np.stack([a1, a2, np.cross(a1, a2)], axis=1)
    r2 = np.sqrt(2.0)
    Q = np.zeros((6, 6))
    for J, (k, l) in enumerate(_KM_PAIRS):
        E = np.zeros((3, 3))
        if k == l:
            E[k, k] = 1.0
        else:
            E[k, l] = E[l, k] = 1 / r2
        A = R @ E @ R.T
        for I, (i, j) in enumerate(_KM_PAIRS):
            Q[I, J] = A[i, j] if i == j else r2 * A[i, j]
    return Q


class PhaseField(_Observable):
    """Phase-field damage model (EasyFEA/Models/_phasefield.py:38-251)."""

    class ReguType(str, Enum):
        AT1 = "AT1"
        AT2 = "AT2"

    class SplitType(str, Enum):
        Bourdin = "Bourdin"
        Amor = "Amor"
        Miehe = "Miehe"
        Zhang = "Zhang"
        Stress = "Stress"
        He = "He"
        AnisotStrain = "AnisotStrain"
        AnisotStrain_PM = "AnisotStrain_PM"
        AnisotStrain_MP = "AnisotStrain_MP"
        AnisotStrain_NoCross = "AnisotStrain_NoCross"
        AnisotStress = "AnisotStress"
        AnisotStress_PM = "AnisotStress_PM"
        AnisotStress_MP = "AnisotStress_MP"
        AnisotStress_NoCross = "AnisotStress_NoCross"

    class SolverType(str, Enum):
        History = "History"
        HistoryDamage = "HistoryDamage"
        BoundConstrain = "BoundConstrain"

    def __init__(self, material: _Elastic, split: Union[str, SplitType], regularization: Union[str, ReguType],
                 Gc: float, l0: float, solver: Union[str, SolverType] = "History",
                 A: Optional[np.ndarray] = None):
        super().__init__()
        assert isinstance(material, _Elastic), "must be an elastic law"
        assert not material.isHeterogeneous, "the GPU phase field takes a homogeneous material"
        self.__material = material
        self.split = split
        if self.split in ("Amor", "Miehe", "Stress", "He"):
            # these splits are written for the isotropic law (Models/_phasefield.py:451-538, 599-631, 689-749)
            assert isinstance(material, Elastic.Isotropic), f"the {self.split} split needs an isotropic material"
        self.regularization = regularization
        self.Gc = Gc
        self.l0 = l0
        self.solver = solver
        self.A = np.eye(material.dim) if A is None else np.asarray(A, dtype=float)
        material._Add_observer(self)

    def _Update(self, observable) -> None:
        self._Notify()

    @property
    def material(self) -> _Elastic:
        return self.__material

    @property
    def dim(self) -> int:
        return self.__material.dim

    @property
    def thickness(self) -> float:
        return self.__material.thickness

    @property
    def split(self) -> str:
        return self.__split

    @split.setter
    def split(self, value):
        value = self.SplitType(value).value
        self.__split = value
        self._Notify()

    @property
    def regularization(self) -> str:
        return self.__regu

    @regularization.setter
    def regularization(self, value):
        self.__regu = self.ReguType(value).value
        self._Notify()

    @property
    def Gc(self) -> float:
        return self.__Gc

    @Gc.setter
    def Gc(self, value):
        assert float(value) > 0, "Gc must be > 0"
        self.__Gc = float(value)
        self._Notify()

    @property
    def l0(self) -> float:
        return self.__l0

    @l0.setter
    def l0(self, value):
        assert float(value) > 0, "l0 must be > 0"
        self.__l0 = float(value)
        self._Notify()

    @property
    def solver(self) -> str:
        return self.__solver

    @solver.setter
    def solver(self, value):
        self.__solver = self.SolverType(value).value
        self._Notify()

    @property
    def k(self) -> float:
        """Diffusion coefficient (EasyFEA/Models/_phasefield.py:237-251)."""
        return 3 / 4 * self.Gc * self.l0 if self.regularization == "AT1" else self.Gc * self.l0

    @property
    def c_w(self) -> float:
        return 8 / 3 if self.regularization == "AT1" else 2.0
