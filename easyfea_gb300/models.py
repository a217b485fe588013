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

        def __str__(self) -> str:
            return f"Isotropic: E = {self.E}, v = {self.v}, dim = {self.dim}"


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

    class SolverType(str, Enum):
        History = "History"
        HistoryDamage = "HistoryDamage"

    def __init__(self, material: _Elastic, split: Union[str, SplitType], regularization: Union[str, ReguType],
                 Gc: float, l0: float, solver: Union[str, SolverType] = "History",
                 A: Optional[np.ndarray] = None):
        super().__init__()
        assert isinstance(material, Elastic.Isotropic), "the GPU split supports isotropic materials"
        assert not material.isHeterogeneous, "the GPU phase field takes a homogeneous material"
        self.__material = material
        self.split = split
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
