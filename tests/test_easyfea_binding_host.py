"""The EasyFEA subclasses (easyfea_gb300/easyfea_binding.py) on the host:
class hierarchy, mesh conversion and the models they reject (no GPU call).
Skipped when EasyFEA is not installed (EASYFEA_PATH, else baseline/_ref)."""

import os
import sys
import types

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def ref():
    path = os.environ.get("EASYFEA_PATH") or os.path.join(ROOT, "baseline", "_ref")
    if not os.path.isdir(os.path.join(path, "EasyFEA")):
        pytest.skip("EasyFEA is not installed")
    try:
        import gmsh  # noqa: F401
    except ImportError:
        sys.modules["gmsh"] = types.ModuleType("gmsh")
    if path not in sys.path:
        sys.path.insert(0, path)
    from EasyFEA import Models, Simulations
    from EasyFEA.FEM._group_elem import GroupElemFactory
    from EasyFEA.FEM._mesh import Mesh
    from EasyFEA.FEM._utils import ElemType

    from easyfea_gb300 import easyfea_binding

    return types.SimpleNamespace(Models=Models, Simulations=Simulations, GEF=GroupElemFactory, Mesh=Mesh,
                                 ElemType=ElemType, B=easyfea_binding)


def _mesh(R, g):
    from helpers import boundary_groups

    coord = np.asarray(g["coord"], float)
    groups = {getattr(R.ElemType, e): R.GEF.Create(getattr(R.ElemType, e), np.asarray(c, np.int64), coord.copy())
              for e, c in boundary_groups(g)}
    groups[getattr(R.ElemType, str(g["elem"]))] = R.GEF.Create(getattr(R.ElemType, str(g["elem"])),
                                                                g["connect"].astype(np.int64), coord.copy())
    return R.Mesh(groups)


def test_subclasses_and_mesh_conversion(ref, golden):
    R = ref
    assert issubclass(R.B.GpuElastic, R.Simulations.Elastic)
    assert issubclass(R.B.GpuPhaseField, R.Simulations.PhaseField)
    g = golden("el_quad4")
    mesh = _mesh(R, g)
    m = R.B.to_gpu_mesh(mesh)
    assert m.Nn == mesh.Nn and m.dim == 2
    assert {e.value for e in m.dict_groupElem} == {"SEG2", "QUAD4"}
    np.testing.assert_array_equal(m.groupElem.connect, mesh.groupElem.connect)
    simu = R.B.GpuElastic(mesh, R.Models.Elastic.Isotropic(2, E=210000.0, v=0.3, planeStress=True, thickness=13.0))
    assert simu.dim == 2 and simu.rho == 1.0


@pytest.mark.parametrize("case,groups", [("el_prism15", {"QUAD8", "TRI6", "PRISM15"}),
                                         ("el_prism6", {"QUAD4", "TRI3", "PRISM6"}),
                                         ("el_tri15", {"SEG5", "TRI15"})])
def test_higher_order_mesh_conversion(ref, golden, case, groups):
    """EasyFEA meshes of the higher-order triangles and of the prisms (two
    face groups) convert group by group, connectivity unchanged."""
    R = ref
    g = golden(case)
    mesh = _mesh(R, g)
    m = R.B.to_gpu_mesh(mesh)
    assert {e.value for e in m.dict_groupElem} == groups
    assert m.Nn == mesh.Nn and m.dim == mesh.dim
    np.testing.assert_array_equal(m.groupElem.connect, mesh.groupElem.connect)
    for gr in m.Get_list_groupElem(m.dim - 1):
        ref_group = mesh.dict_groupElem[getattr(R.ElemType, gr.elemType.value)]
        np.testing.assert_array_equal(gr.connect, ref_group.connect)


def test_unsupported_models_rejected(ref, golden):
    R = ref
    g = golden("el_quad4")
    mesh = _mesh(R, g)
    Ne = len(g["connect"])
    mat = R.Models.Elastic.TransverselyIsotropic(2, El=1e5 * np.ones(Ne), Et=1e4, Gl=1e4, vl=0.3, vt=0.2)
    with pytest.raises(NotImplementedError):
        R.B.GpuElastic(mesh, mat)  # a per-element transversely isotropic law
    iso = R.Models.Elastic.Isotropic(2, E=210000.0, v=0.3, planeStress=False)
    for split in ("Zhang", "AnisotStrain_PM", "AnisotStress_NoCross"):
        with pytest.raises(NotImplementedError):
            R.B.GpuPhaseField(mesh, R.Models.PhaseField(iso, split, "AT2", 2.7, 0.01))


def test_save_iter_pickles_read_both_ways(ref, golden, tmp_path):
    """Save_Iter in folder mode writes the reference's single-process layout
    (Results/results{i}.pickle holding the iteration dict): the library's
    simulation and the reference read each other's files (no GPU call)."""
    import pickle

    from easyfea_gb300 import Models
    from easyfea_gb300 import simulations as Simulations
    from easyfea_gb300.mesh import Mesh_Quad4_Rect

    R = ref
    g = golden("el_quad4")
    m = Mesh_Quad4_Rect(120.0, 13.0, 24, 4)
    ours = Simulations.Elastic(m, Models.Elastic.Isotropic(2, E=210000.0, v=0.3, planeStress=True, thickness=13.0))
    ours.folder = str(tmp_path / "ours")
    ours.Save_Iter()
    ours.Save_Iter()
    assert ours.Niter == 2
    assert sorted(os.listdir(tmp_path / "ours" / "Results")) == ["results0.pickle", "results1.pickle"]
    theirs = R.Simulations.Elastic(_mesh(R, g), R.Models.Elastic.Isotropic(2, E=210000.0, v=0.3, planeStress=True,
                                                                            thickness=13.0),
                                   folder=str(tmp_path / "theirs"))
    theirs._Set_solutions(theirs.problemType, g["u"])
    theirs.Save_Iter()
    with open(tmp_path / "theirs" / "Results" / "results0.pickle", "rb") as f:
        ref_iter = pickle.load(f)
    assert set(ref_iter) == set(ours.Get_results(0))
    # ours reads the reference's file, the reference reads ours
    ours._results.append(str(tmp_path / "theirs" / "Results" / "results0.pickle"))
    np.testing.assert_array_equal(ours.Get_results(-1)["displacement"], g["u"])
    theirs._Simu__list_results.append(str(tmp_path / "ours" / "Results" / "results0.pickle"))
    theirs._Simu__Niter += 1
    theirs.Set_Iter(-1)
    assert np.abs(theirs.displacement).max() == 0.0
