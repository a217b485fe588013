"""easyfea_gb300 -- GB300 (sm_103a) implementation of EasyFEA's finite-element hot path.

Mirrors the reference's user API for that path:

    from easyfea_gb300 import Models, Simulations, mesh
    m = mesh.Mesh_Quad4_Rect(120, 13, 240, 26)
    mat = Models.Elastic.Isotropic(2, E=210000, v=0.3, planeStress=True, thickness=13)
    simu = Simulations.Elastic(m, mat)
    simu.add_dirichlet(m.Nodes_Conditions(lambda x, y, z: x == 0), [0, 0], ["x", "y"])
    simu.add_surfLoad(m.Nodes_Conditions(lambda x, y, z: x == 120), [-800 / 13**2], ["y"])
    u = simu.Solve()

Element operators, assembly, the phase-field split and the PCG solve run in
libgb300fea.so (C ABI: include/gfea.h); there is no CPU fallback.
"""

from . import mesh
from . import models as Models
from .mesh import ElemType, MatrixType, Mesh

__all__ = ["Models", "Simulations", "mesh", "Mesh", "ElemType", "MatrixType"]


def __getattr__(name):
    # Simulations imports torch; load it on first use
    if name == "Simulations":
        from . import simulations

        return simulations
    raise AttributeError(name)
