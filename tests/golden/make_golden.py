"""Generate the golden fixtures of ``tests/golden/`` by running the reference itself.

Run in a container where matnoel/EasyFEA's sources are importable::

    python tests/golden/make_golden.py <path to EasyFEA sources> [--only=name,...]

The path may instead come from the ``EASYFEA_REFERENCE`` environment variable.

gmsh (imported unconditionally by EasyFEA/FEM/_mesher.py:13) is replaced by an
empty stub module; meshes come from ``easyfea_gb300.mesh``'s organised
generators and are handed to the reference through
``GroupElemFactory.Create`` + ``Mesh`` (EasyFEA/FEM/_group_elem.py:2330-2355,
EasyFEA/FEM/_mesh.py:46-91).  The solver is pinned to ``scipy`` (SuperLU).

Each case is written as one compressed ``.npz`` holding its inputs (mesh
arrays, material, boundary conditions) and the reference's outputs.
"""

from __future__ import annotations

import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from easyfea_gb300 import mesh as gmesh  # noqa: E402

sys.path.insert(0, os.path.dirname(HERE))
from helpers import field_loads  # noqa: E402


def load_reference(path):
    sys.modules.setdefault("gmsh", types.ModuleType("gmsh"))
    sys.path.insert(0, path)
    import EasyFEA  # noqa: F401
    from EasyFEA import Models, Simulations
    from EasyFEA.FEM._group_elem import GroupElemFactory
    from EasyFEA.FEM._mesh import Mesh
    from EasyFEA.FEM._utils import ElemType
    from EasyFEA.Simulations.Solvers import SolverType
    return types.SimpleNamespace(Models=Models, Simulations=Simulations, GEF=GroupElemFactory,
                                 Mesh=Mesh, ElemType=ElemType, SolverType=SolverType)


def to_ref_mesh(R, m: gmesh.Mesh):
    groups = {}
    for g in m.dict_groupElem.values():
        et = getattr(R.ElemType, g.elemType.value)
        groups[et] = R.GEF.Create(et, np.array(g.connect, dtype=np.int64), m.coord.copy())
    return R.Mesh(groups)


def mesh_arrays(m: gmesh.Mesh):
    """The main group and the boundary groups (belem/bconnect, and for the
    prisms' second face type belem2/bconnect2)."""
    g = m.groupElem
    bs = m.Get_list_groupElem(m.dim - 1)
    d = dict(elem=g.elemType.value, coord=m.coord, connect=g.connect,
             belem=bs[0].elemType.value, bconnect=bs[0].connect)
    if len(bs) > 1:
        d.update(belem2=bs[1].elemType.value, bconnect2=bs[1].connect)
    return d


def csr_parts(prefix, A):
    A = A.tocsr()
    A.sort_indices()
    return {f"{prefix}_data": A.data, f"{prefix}_indices": A.indices.astype(np.int32),
            f"{prefix}_indptr": A.indptr.astype(np.int64)}


def elastic_case(R, name, m, E, v, planeStress, thickness, loadval, loaddir, out, law=None, load_axis=0):
    """``law``: None (isotropic E, v) or a dict of transversely isotropic
    parameters (El, Et, Gl, vl, vt, axis_l, axis_t).  The body is clamped
    at x = 0 and loaded on the face where coordinate ``load_axis`` is largest
    (stored as ``right``)."""
    dim = m.dim
    rm = to_ref_mesh(R, m)
    if law is None:
        mat = R.Models.Elastic.Isotropic(dim, E=E, v=v, planeStress=planeStress, thickness=thickness)
    else:
        mat = R.Models.Elastic.TransverselyIsotropic(dim, **law, planeStress=planeStress, thickness=thickness)
    simu = R.Simulations.Elastic(rm, mat)
    simu.solver = R.SolverType.scipy
    L = m.coord[:, 0].max()
    left = rm.Nodes_Conditions(lambda x, y, z: x == 0)
    Lmax = m.coord[:, load_axis].max()
    right = rm.Nodes_Conditions(lambda x, y, z: (x, y, z)[load_axis] == Lmax)
    unk = ["x", "y"] if dim == 2 else ["x", "y", "z"]
    simu.add_dirichlet(left, [0.0] * dim, unk)
    simu.add_surfLoad(right, [loadval], [loaddir])
    u = simu.Solve()
    K, C, M, F = simu.Get_K_C_M_F()
    b = np.asarray(simu._Solver_Apply_Neumann(simu.problemType).todense()).ravel()
    d = dict(mesh_arrays(m), E=np.asarray(E, float), v=v, planeStress=planeStress,
             thickness=thickness, loadval=loadval, loaddir=loaddir, u=u, b=b,
             left=left, right=right)
    if law is not None:
        d.update({f"ti_{k}": np.asarray(val, float) for k, val in law.items()}, C=mat.C, S=mat.S)
    d.update(csr_parts("K", K))
    d.update(csr_parts("M", M))
    np.savez_compressed(os.path.join(out, f"{name}.npz"), **d)
    print(name, "Ndof", u.size, "nnz", K.nnz, "|u|max", np.abs(u).max())


def split_case(R, out, seed=0):
    """cP, cM, psi+, psi- of the reference's PhaseField.Calc_C on seeded strains
    plus the degenerate cases of Models/_phasefield.py:793-805 and :861-906."""
    from EasyFEA.FEM._linalg import FeArray
    rng = np.random.default_rng(seed)
    res = {}
    for dim in (2, 3):
        n = 3 if dim == 2 else 6
        eps = rng.standard_normal((48, n)) * 1e-3
        special = [np.zeros(n)]
        e = np.zeros(n); e[0] = 1e-3; special.append(e)           # uniaxial
        e = np.zeros(n); e[:dim] = 1e-3; special.append(e)        # hydrostatic
        e = np.zeros(n); e[:dim] = -2e-3; special.append(e)
        e = np.zeros(n); e[0] = 1e-3; e[1] = 1e-3; special.append(e)  # two equal
        e = np.zeros(n); e[0] = -1e-3; e[1] = 2e-3; special.append(e)
        if dim == 3:
            e = np.zeros(n); e[0] = 1e-3; e[1] = 2e-3; e[2] = 2e-3; special.append(e)
            e = np.zeros(n); e[0] = 1e-3; e[1] = 1e-3; e[2] = 3e-3; special.append(e)
            e = np.zeros(n); e[5] = 1e-3; special.append(e)        # pure shear
        eps = np.concatenate([eps, np.array(special)], 0)[:, None, :]  # (Ne, 1, n)
        for planeStress in ((True, False) if dim == 2 else (False,)):
            mat = R.Models.Elastic.Isotropic(dim, E=210000.0, v=0.3, planeStress=planeStress)
            for split in ("Bourdin", "Amor", "Miehe", "Zhang", "Stress", "He"):
                pfm = R.Models.PhaseField(mat, split, "AT2", 2.7, 0.01)
                cP, cM = pfm.Calc_C(FeArray.asfearray(eps.copy()))
                psiP, psiM = pfm.Calc_psi_e_pg(FeArray.asfearray(eps.copy()))
                key = f"d{dim}_ps{int(planeStress)}_{split}"
                res[key + "_cP"] = np.asarray(cP)
                res[key + "_cM"] = np.asarray(cM)
                res[key + "_psiP"] = np.asarray(psiP)
                res[key + "_psiM"] = np.asarray(psiM)
        res[f"d{dim}_eps"] = eps
    np.savez_compressed(os.path.join(out, "split.npz"), **res)
    print("split", len(res))


def pf_case(R, name, m, split, regu, planeStress, E, v, Gc, l0, steps, dU, out, tol=1e-3, maxIter=100, law=None):
    dim = m.dim
    rm = to_ref_mesh(R, m)
    if law is None:
        mat = R.Models.Elastic.Isotropic(dim, E=E, v=v, planeStress=planeStress, thickness=1.0)
    else:
        mat = R.Models.Elastic.TransverselyIsotropic(dim, **law, planeStress=planeStress, thickness=1.0)
    pfm = R.Models.PhaseField(mat, split, regu, Gc, l0)
    simu = R.Simulations.PhaseField(rm, pfm)
    simu.solver = R.SolverType.scipy
    H = m.coord[:, 1].max()
    bottom = rm.Nodes_Conditions(lambda x, y, z: y == 0)
    top = rm.Nodes_Conditions(lambda x, y, z: y == H)
    notch = rm.Nodes_Conditions(lambda x, y, z: (np.abs(y - H / 2) < 1e-12) & (x <= 0.5 * m.coord[:, 0].max()))
    unk = ["x", "y"] if dim == 2 else ["x", "y", "z"]
    top_dofs = simu.Bc_dofs_nodes(top, ["y"])
    us, ds, Hs, Fs, its = [], [], [], [], []
    for k in range(1, steps + 1):
        simu.Bc_Init()
        simu.add_dirichlet(notch, [1.0], ["d"], problemType="damage")
        simu.add_dirichlet(bottom, [0.0] * dim, unk)
        simu.add_dirichlet(top, [0.0, k * dU] + ([0.0] if dim == 3 else []), unk)
        u, d, conv = simu.Solve(tol, maxIter, convOption=0)
        simu.Save_Iter()
        f = np.sum(simu.Calc_Reaction(top_dofs, simu.ProblemTypes.elastic))
        us.append(u.copy()); ds.append(d.copy()); Fs.append(f)
        Hs.append(np.asarray(simu._PhaseField__psiP_e_pg).copy())
        its.append(simu._PhaseField__Niter)
        print(name, "step", k, "F", f, "dmax", d.max(), "Niter", its[-1])
    Ku = simu.Get_K_C_M_F("elastic")[0]
    Kd, _, _, Fd = simu.Get_K_C_M_F("damage")
    extra = {} if law is None else {f"ti_{k}": np.asarray(val, float) for k, val in law.items()}
    res = dict(mesh_arrays(m), split=split, regu=regu, planeStress=planeStress, E=E, v=v,
               Gc=Gc, l0=l0, dU=dU, tol=tol, maxIter=maxIter, **extra,
               u=np.array(us), d=np.array(ds), H=np.array(Hs), F=np.array(Fs), Niter=np.array(its),
               bottom=bottom, top=top, notch=notch, top_dofs=top_dofs,
               Fd=np.asarray(Fd.todense()).ravel())
    res.update(csr_parts("Ku", Ku))
    res.update(csr_parts("Kd", Kd))
    np.savez_compressed(os.path.join(out, f"{name}.npz"), **res)


def field_load_case(R, name, m, E, v, planeStress, thickness, out):
    dim = m.dim
    rm = to_ref_mesh(R, m)
    mat = R.Models.Elastic.Isotropic(dim, E=E, v=v, planeStress=planeStress, thickness=thickness)
    simu = R.Simulations.Elastic(rm, mat)
    simu.solver = R.SolverType.scipy
    L = m.coord[:, 0].max()
    left = rm.Nodes_Conditions(lambda x, y, z: x == 0)
    Lmax = m.coord[:, load_axis].max()
    right = rm.Nodes_Conditions(lambda x, y, z: (x, y, z)[load_axis] == Lmax)
    unk = ["x", "y"] if dim == 2 else ["x", "y", "z"]
    simu.add_dirichlet(left, [0.0] * dim, unk)
    for nodes, vals, un in field_loads(dim, m.coord, right):
        simu.add_surfLoad(nodes, vals, un)
    u = simu.Solve()
    b = np.asarray(simu._Solver_Apply_Neumann(simu.problemType).todense()).ravel()
    d = dict(mesh_arrays(m), E=E, v=v, planeStress=planeStress, thickness=thickness, u=u, b=b,
             left=left, right=right)
    np.savez_compressed(os.path.join(out, f"{name}.npz"), **d)
    print(name, "Ndof", u.size, "|b|", np.abs(b).sum())


def _field_load_cases(R, out):
    field_load_case(R, "el_quad4_field_load", gmesh.Mesh_Quad4_Rect(120.0, 13.0, 24, 4), 210000.0, 0.3, True,
                    13.0, out)
    field_load_case(R, "el_hexa8_field_load", gmesh.Mesh_Hexa8_Box(60.0, 10.0, 10.0, 6, 2, 2), 210000.0, 0.3,
                    False, 1.0, out)


def pf_conv_case(R, name, m, convOption, steps, dU, out, tol=1e-3, maxIter=100):
    """Staggered loop of the reference with convergence criterion ``convOption``
    (1: crack energy, 2: total energy, 3: summed relative increments;
    Simulations/_phasefield.py:347-405) on a small notched TRI3 plate, through
    fracture: force, iterations, convergence measure, u and d per step."""
    dim = m.dim
    rm = to_ref_mesh(R, m)
    mat = R.Models.Elastic.Isotropic(dim, E=210000.0, v=0.3, planeStress=False, thickness=1.0)
    pfm = R.Models.PhaseField(mat, "Miehe", "AT2", 2.7, 0.1)
    simu = R.Simulations.PhaseField(rm, pfm)
    simu.solver = R.SolverType.scipy
    H = m.coord[:, 1].max()
    bottom = rm.Nodes_Conditions(lambda x, y, z: y == 0)
    top = rm.Nodes_Conditions(lambda x, y, z: y == H)
    notch = rm.Nodes_Conditions(lambda x, y, z: (np.abs(y - H / 2) < 1e-12) & (x <= 0.5 * m.coord[:, 0].max()))
    top_dofs = simu.Bc_dofs_nodes(top, ["y"])
    us, ds, Fs, its, convs = [], [], [], [], []
    for k in range(1, steps + 1):
        simu.Bc_Init()
        simu.add_dirichlet(notch, [1.0], ["d"], problemType="damage")
        simu.add_dirichlet(bottom, [0.0, 0.0], ["x", "y"])
        simu.add_dirichlet(top, [0.0, k * dU], ["x", "y"])
        u, d, conv = simu.Solve(tol, maxIter, convOption=convOption)
        simu.Save_Iter()
        f = np.sum(simu.Calc_Reaction(top_dofs, simu.ProblemTypes.elastic))
        us.append(u.copy()); ds.append(d.copy()); Fs.append(f)
        its.append(simu._PhaseField__Niter)
        convs.append(float(simu._PhaseField__convIter))
        print(name, "step", k, "F", f, "dmax", d.max(), "Niter", its[-1], "conv", convs[-1])
    res = dict(mesh_arrays(m), split="Miehe", regu="AT2", planeStress=False, E=210000.0, v=0.3,
               Gc=2.7, l0=0.1, dU=dU, tol=tol, maxIter=maxIter, convOption=convOption,
               u=np.array(us), d=np.array(ds), F=np.array(Fs), Niter=np.array(its),
               convIter=np.array(convs), bottom=bottom, top=top, notch=notch, top_dofs=top_dofs)
    np.savez_compressed(os.path.join(out, f"{name}.npz"), **res)


def _tetra4_cases(R, out):
    """TETRA4: the 3D cantilever box and a phase-field system at a prescribed state."""
    elastic_case(R, "el_tetra4", gmesh.Mesh_Tetra4_Box(60.0, 10.0, 10.0, 6, 2, 2), 210000.0, 0.3, False, 1.0,
                 -1.0, "z", out)
    pf_state_case(R, "pfsys_tetra4_miehe_at2", gmesh.Mesh_Tetra4_Box(1.0, 1.0, 0.5, 4, 4, 2), "Miehe", "AT2", out)


def _pf_split_cases(R, out):
    """Staggered loops with the stress-based and He splits on the 16x16 plate."""
    for split in ("Zhang", "Stress", "He"):
        pf_case(R, f"pf_tri3_{split.lower()}_at2", gmesh.Mesh_Tri3_Rect(1.0, 1.0, 16, 16), split, "AT2", False,
                210000.0, 0.3, 2.7, 0.1, 3, 4e-3, out)


def _pf_conv_cases(R, out):
    m = gmesh.Mesh_Tri3_Rect(1.0, 1.0, 16, 16)
    for opt in (1, 2, 3):
        pf_conv_case(R, f"pf_tri3_conv{opt}", m, opt, 4, 4e-3, out)


def pf_curve_case(R, out, steps=600, dU=1e-5, tol=1e-3, maxIter=500, keep_every=50):
    """The notched-plate benchmark through its whole load history: 200x200 squares
    of the unit plate split into 80,000 TRI3, AT2, Miehe split, E = 210000,
    nu = 0.3, Gc = 2.7, l0 = 0.01, plane strain, d = 1 imposed on the notch
    (y = 0.5, x <= 0.5), bottom clamped, top uy = k dU for k = 1..steps,
    ``Solve(tol, maxIter, convOption=0)`` and ``Save_Iter`` per step (the load
    loop of examples/PhaseField/Shear.py:182-220 with this plate's conditions).
    Stores per step the top reaction F, staggered iterations, convergence flag
    and max d, plus the damage field every ``keep_every`` steps, at the force
    peak and at the last step.  A partial file is rewritten every 10 steps."""
    name = "pf_curve_tri3_200x200"
    m = gmesh.Mesh_Tri3_Rect(1.0, 1.0, 200, 200)
    rm = to_ref_mesh(R, m)
    mat = R.Models.Elastic.Isotropic(2, E=210000.0, v=0.3, planeStress=False, thickness=1.0)
    pfm = R.Models.PhaseField(mat, "Miehe", "AT2", 2.7, 0.01)
    simu = R.Simulations.PhaseField(rm, pfm)
    simu.solver = R.SolverType.scipy
    bottom = rm.Nodes_Conditions(lambda x, y, z: y == 0)
    top = rm.Nodes_Conditions(lambda x, y, z: y == 1.0)
    notch = rm.Nodes_Conditions(lambda x, y, z: (np.abs(y - 0.5) < 1e-12) & (x <= 0.5))
    top_dofs = simu.Bc_dofs_nodes(top, ["y"])
    Fs, its, convd, dmax, secs = [], [], [], [], []
    kept = {}      # step -> damage field
    peak = None    # (step, damage) at the running force maximum
    import time
    t0 = time.perf_counter()
    for k in range(1, steps + 1):
        ts = time.perf_counter()
        simu.Bc_Init()
        simu.add_dirichlet(notch, [1.0], ["d"], problemType="damage")
        simu.add_dirichlet(bottom, [0.0, 0.0], ["x", "y"])
        simu.add_dirichlet(top, [0.0, k * dU], ["x", "y"])
        u, d, conv = simu.Solve(tol, maxIter, convOption=0)
        simu.Save_Iter()
        f = float(np.sum(simu.Calc_Reaction(top_dofs, simu.ProblemTypes.elastic)))
        if not Fs or f >= max(Fs):
            peak = (k, d.copy())
        Fs.append(f); its.append(simu._PhaseField__Niter); convd.append(bool(conv))
        dmax.append(float(d.max())); secs.append(time.perf_counter() - ts)
        if k % keep_every == 0 or k == steps:
            kept[k] = d.copy()
        print(name, "step", k, "F", f, "dmax", dmax[-1], "Niter", its[-1],
              f"{secs[-1]:.1f}s total {time.perf_counter() - t0:.0f}s", flush=True)
        if k % 10 == 0 or k == steps:
            allk = dict(kept)
            allk[peak[0]] = peak[1]
            ks = sorted(allk)
            res = dict(mesh_arrays(m), split="Miehe", regu="AT2", planeStress=False, E=210000.0,
                       v=0.3, Gc=2.7, l0=0.01, dU=dU, tol=tol, maxIter=maxIter, convOption=0,
                       F=np.array(Fs), Niter=np.array(its, np.int32), converged=np.array(convd),
                       dmax=np.array(dmax), ref_seconds=np.array(secs),
                       d_steps=np.array(ks, np.int32), d=np.array([allk[j] for j in ks]),
                       bottom=bottom, top=top, notch=notch, top_dofs=top_dofs)
            fn = f"{name}.npz" if k == steps else f"{name}.partial.npz"
            np.savez_compressed(os.path.join(out, fn), **res)


def pf_state_case(R, name, m, split, regu, out, seed=7):
    """Kd, Fd, Ku of the reference at a prescribed (u, d, committed history) state:
    pins r/f/k of both regularisations and the degraded stiffness without the
    staggered loop (PhaseField.Get_K_C_M_F, Simulations/_phasefield.py:248-269)."""
    dim = m.dim
    rng = np.random.default_rng(seed)
    rm = to_ref_mesh(R, m)
    mat = R.Models.Elastic.Isotropic(dim, E=210000.0, v=0.3, planeStress=False, thickness=1.0)
    pfm = R.Models.PhaseField(mat, split, regu, 2.7, 0.05)
    simu = R.Simulations.PhaseField(rm, pfm)
    x = m.coord
    # smooth displacement with tension and shear, damage in (0, 1)
    u = np.zeros((m.Nn, dim))
    u[:, 0] = 1e-3 * np.sin(2.0 * x[:, 1]) + 2e-4 * x[:, 0]
    u[:, 1] = 3e-3 * x[:, 1] ** 2 - 1e-3 * x[:, 0]
    if dim == 3:
        u[:, 2] = 5e-4 * x[:, 0] * x[:, 2]
    u = u.ravel()
    d = np.clip(0.5 + 0.4 * np.sin(3 * x[:, 0]) * np.cos(2 * x[:, 1]), 0, 1)
    simu._Set_solutions(simu.ProblemTypes.elastic, u)
    simu._Set_solutions(simu.ProblemTypes.damage, d)
    simu.Need_Update()
    Kd, _, _, Fd = simu.Get_K_C_M_F("damage")
    H1 = np.asarray(simu._PhaseField__psiP_e_pg).copy()
    Ku = simu.Get_K_C_M_F("elastic")[0]
    res = dict(mesh_arrays(m), split=split, regu=regu, E=210000.0, v=0.3, Gc=2.7, l0=0.05,
               u=u, d=d, H=H1, Fd=np.asarray(Fd.todense()).ravel())
    res.update(csr_parts("Ku", Ku))
    res.update(csr_parts("Kd", Kd))
    np.savez_compressed(os.path.join(out, f"{name}.npz"), **res)
    print(name, "Kd nnz", Kd.nnz, "Ku nnz", Ku.nnz)


ELASTIC_RESULTS = {2: ["ux", "uy", "displacement", "displacement_norm", "Sxx", "Syy", "Sxy", "Exx", "Eyy", "Exy"],
                   3: ["ux", "uy", "uz", "displacement", "displacement_norm", "Sxx", "Syy", "Szz", "Syz", "Sxz",
                       "Sxy", "Exx", "Eyy", "Ezz", "Eyz", "Exz", "Exy"]}
FIELD_RESULTS = ["Svm", "Stress", "Evm", "Strain"]


def _smooth_u(m, scale=1e-3):
    """A displacement field with strains that vary inside each element."""
    x = m.coord
    L = max(x[:, 0].max(), 1e-12)
    u = np.zeros((m.Nn, m.dim))
    u[:, 0] = scale * (np.sin(2.1 * x[:, 1] / L * 3) + 0.3 * (x[:, 0] / L) ** 2)
    u[:, 1] = scale * (0.7 * (x[:, 1] / L) ** 2 - 0.4 * x[:, 0] / L + 0.2 * np.cos(3 * x[:, 0] / L))
    if m.dim == 3:
        u[:, 2] = scale * (0.5 * x[:, 0] * x[:, 2] / L**2 + 0.1 * np.sin(4 * x[:, 1] / L))
    return u.ravel()


def results_case(R, name, m, E, v, planeStress, thickness, out):
    """Elastic.Result (Simulations/_elastic.py:229-320) on a prescribed
    displacement: every strain / stress / energy result at the nodes and on
    the elements."""
    rm = to_ref_mesh(R, m)
    mat = R.Models.Elastic.Isotropic(m.dim, E=E, v=v, planeStress=planeStress, thickness=thickness)
    simu = R.Simulations.Elastic(rm, mat)
    u = _smooth_u(m)
    simu._Set_solutions(simu.problemType, u)
    res = dict(mesh_arrays(m), E=np.asarray(E, float), v=v, planeStress=planeStress, thickness=thickness, u=u)
    names = ELASTIC_RESULTS[m.dim] + FIELD_RESULTS + ["Wdef_e", "ZZ1_e"]
    for r in names:
        res[f"{r}_n"] = np.asarray(simu.Result(r, nodeValues=True))
        res[f"{r}_e"] = np.asarray(simu.Result(r, nodeValues=False))
    for r in ("Wdef", "ZZ1"):
        res[r] = float(simu.Result(r))
    res["names"] = np.array(names)
    np.savez_compressed(os.path.join(out, f"{name}.npz"), **res)
    print(name, "Wdef", res["Wdef"], "ZZ1", res["ZZ1"])


def pf_results_case(R, name, m, split, regu, out, seed=11):
    """PhaseField.Result (Simulations/_phasefield.py:682-760) at a prescribed
    (u, d, committed History) state: the degraded stress results, psiP and the
    energies."""
    dim = m.dim
    rng = np.random.default_rng(seed)
    rm = to_ref_mesh(R, m)
    mat = R.Models.Elastic.Isotropic(dim, E=210000.0, v=0.3, planeStress=False, thickness=1.0)
    pfm = R.Models.PhaseField(mat, split, regu, 2.7, 0.05)
    simu = R.Simulations.PhaseField(rm, pfm)
    u = _smooth_u(m)
    x = m.coord
    d = np.clip(0.5 + 0.45 * np.sin(3 * x[:, 0]) * np.cos(2 * x[:, 1]), 0, 1)
    simu._Set_solutions(simu.ProblemTypes.elastic, u)
    simu._Set_solutions(simu.ProblemTypes.damage, d)
    simu.Need_Update()
    # a committed History field that is above psi+ at part of the Gauss points
    simu.Get_K_C_M_F("damage")
    psiP = np.asarray(simu._PhaseField__psiP_e_pg).copy()
    H_old = psiP * rng.uniform(0.5, 1.5, psiP.shape)
    from EasyFEA.FEM import FeArray
    simu._PhaseField__old_psiP_e_pg = FeArray.asfearray(H_old.copy())
    simu.Need_Update()
    res = dict(mesh_arrays(m), split=split, regu=regu, E=210000.0, v=0.3, Gc=2.7, l0=0.05, u=u, d=d, H_old=H_old)
    names = ELASTIC_RESULTS[dim][:2] + ELASTIC_RESULTS[dim][5:] + FIELD_RESULTS + ["damage", "psiP"]
    for r in names:
        res[f"{r}_n"] = np.asarray(simu.Result(r, nodeValues=True))
        res[f"{r}_e"] = np.asarray(simu.Result(r, nodeValues=False))
    for r in ("Wdef", "Psi_Crack"):
        res[r] = float(simu.Result(r))
    res["names"] = np.array(names)
    np.savez_compressed(os.path.join(out, f"{name}.npz"), **res)
    print(name, "Wdef", res["Wdef"], "Psi_Crack", res["Psi_Crack"])


def _results_cases(R, out):
    rng = np.random.default_rng(21)
    results_case(R, "res_quad4", gmesh.Mesh_Quad4_Rect(12.0, 3.0, 8, 3), 210000.0, 0.3, True, 13.0, out)
    mq = gmesh.Mesh_Quad4_Rect(12.0, 3.0, 7, 3)
    results_case(R, "res_quad4_hetero", mq, 210000.0 * np.exp(0.3 * rng.standard_normal(mq.Ne)), 0.3, True, 2.0,
                 out)
    results_case(R, "res_tri3", gmesh.Mesh_Tri3_Rect(12.0, 3.0, 6, 3), 210000.0, 0.25, False, 1.0, out)
    results_case(R, "res_quad9", gmesh.Mesh_Quad9_Rect(12.0, 3.0, 4, 2), 210000.0, 0.3, True, 1.0, out)
    results_case(R, "res_hexa8", gmesh.Mesh_Hexa8_Box(6.0, 2.0, 2.0, 4, 2, 2), 210000.0, 0.3, False, 1.0, out)
    results_case(R, "res_tetra4", gmesh.Mesh_Tetra4_Box(6.0, 2.0, 2.0, 3, 2, 2), 210000.0, 0.3, False, 1.0, out)
    pf_results_case(R, "res_pf_tri3_miehe", gmesh.Mesh_Tri3_Rect(1.0, 1.0, 6, 6), "Miehe", "AT2", out)
    pf_results_case(R, "res_pf_quad4_amor", gmesh.Mesh_Quad4_Rect(1.0, 1.0, 5, 5), "Amor", "AT1", out)
    pf_results_case(R, "res_pf_hexa8_miehe", gmesh.Mesh_Hexa8_Box(1.0, 1.0, 0.5, 3, 3, 2), "Miehe", "AT2", out)


# a transversely isotropic law (moduli of a wood-like fibre material), its
# fibre at 30 degrees in the plane, and a 3D orientation out of the axes
TI = dict(El=11580.0, Et=500.0, Gl=450.0, vl=0.02, vt=0.44)
TI_2D = dict(TI, axis_l=(np.cos(np.pi / 6), np.sin(np.pi / 6), 0.0), axis_t=(-np.sin(np.pi / 6), np.cos(np.pi / 6), 0.0))
TI_3D = dict(TI, axis_l=(1.0, 1.0, 1.0), axis_t=(1.0, -1.0, 0.0))
ANISOT_SPLITS = ("AnisotStrain", "AnisotStrain_PM", "AnisotStrain_MP", "AnisotStrain_NoCross", "AnisotStress",
                 "AnisotStress_PM", "AnisotStress_MP", "AnisotStress_NoCross")


def anisot_case(R, out, seed=3):
    """Transversely isotropic and anisotropic laws (Models/Elastic/_laws.py:
    513-717, 1111-1270): C and S; the anisotropic splits' cP, cM, psi+, psi-
    (Models/_phasefield.py:541-567, 646-676) on seeded strains."""
    from EasyFEA.FEM._linalg import FeArray
    rng = np.random.default_rng(seed)
    res = {}
    for dim, ps in ((2, True), (2, False), (3, False)):
        law = TI_2D if dim == 2 else TI_3D
        mat = R.Models.Elastic.TransverselyIsotropic(dim, **law, planeStress=ps)
        key = f"ti_d{dim}_ps{int(ps)}"
        res[key + "_C"], res[key + "_S"] = mat.C, mat.S
        n = 3 if dim == 2 else 6
        eps = rng.standard_normal((48, 1, n)) * 1e-3
        res[key + "_eps"] = eps
        for split in ANISOT_SPLITS:
            pfm = R.Models.PhaseField(mat, split, "AT2", 2.7, 0.01)
            cP, cM = pfm.Calc_C(FeArray.asfearray(eps.copy()))
            psiP, psiM = pfm.Calc_psi_e_pg(FeArray.asfearray(eps.copy()))
            res[f"{key}_{split}_cP"], res[f"{key}_{split}_cM"] = np.asarray(cP), np.asarray(cM)
            res[f"{key}_{split}_psiP"], res[f"{key}_{split}_psiM"] = np.asarray(psiP), np.asarray(psiM)
    for dim in (2, 3):
        n = 3 if dim == 2 else 6
        A = rng.standard_normal((n, n))
        Cin = A @ A.T + n * np.eye(n)
        res[f"an_d{dim}_Cin"] = Cin
        for voigt in (True, False):
            mat = R.Models.Elastic.Anisotropic(dim, Cin.copy(), voigt, axis1=(1.0, 2.0, 0.0), axis2=(-2.0, 1.0, 0.0))
            res[f"an_d{dim}_v{int(voigt)}_C"], res[f"an_d{dim}_v{int(voigt)}_S"] = mat.C, mat.S
    for k, val in TI.items():
        res["TI_" + k] = val
    for k in ("axis_l", "axis_t"):
        res["TI_2D_" + k] = np.asarray(TI_2D[k])
        res["TI_3D_" + k] = np.asarray(TI_3D[k])
    np.savez_compressed(os.path.join(out, "anisot.npz"), **res)
    print("anisot", len(res))
    elastic_case(R, "el_quad4_ti", gmesh.Mesh_Quad4_Rect(120.0, 13.0, 24, 4), 0.0, 0.0, True, 13.0, -8 / 13**2,
                 "y", out, law=TI_2D)
    elastic_case(R, "el_hexa8_ti", gmesh.Mesh_Hexa8_Box(60.0, 10.0, 10.0, 6, 2, 2), 0.0, 0.0, False, 1.0, -0.05, "z",
                 out, law=TI_3D)
    for split in ("AnisotStrain", "AnisotStress"):
        pf_case(R, f"pf_tri3_ti_{split.lower()}", gmesh.Mesh_Tri3_Rect(1.0, 1.0, 16, 16), split, "AT2", False,
                0.0, 0.0, 2.7, 0.1, 4, 1.6e-2, out, law=TI_2D)


def pf_solver_case(R, name, m, solver, steps, dU, out, tol=1e-3, maxIter=100):
    """The staggered loop with the HistoryDamage or BoundConstrain
    irreversibility solver (Simulations/_phasefield.py:148-163, 409-419;
    BoundConstrain solves the damage by scipy.optimize.lsq_linear with
    d_n <= d <= 1): the 16x16 TRI3 plate pulled at the top, no notch (the
    reference's bounds are full length, so no damage Dirichlet condition)."""
    rm = to_ref_mesh(R, m)
    mat = R.Models.Elastic.Isotropic(2, E=210000.0, v=0.3, planeStress=False, thickness=1.0)
    pfm = R.Models.PhaseField(mat, "Miehe", "AT2", 2.7, 0.1, solver=getattr(R.Models.PhaseField.SolverType, solver))
    simu = R.Simulations.PhaseField(rm, pfm)
    simu.solver = R.SolverType.scipy
    H = m.coord[:, 1].max()
    bottom = rm.Nodes_Conditions(lambda x, y, z: y == 0)
    top = rm.Nodes_Conditions(lambda x, y, z: y == H)
    top_dofs = simu.Bc_dofs_nodes(top, ["y"])
    us, ds, Fs, its = [], [], [], []
    for k in range(1, steps + 1):
        simu.Bc_Init()
        simu.add_dirichlet(bottom, [0.0, 0.0], ["x", "y"])
        simu.add_dirichlet(top, [0.0, k * dU], ["x", "y"])
        u, d, conv = simu.Solve(tol, maxIter, convOption=0)
        simu.Save_Iter()
        f = np.sum(simu.Calc_Reaction(top_dofs, simu.ProblemTypes.elastic))
        us.append(u.copy()); ds.append(d.copy()); Fs.append(f)
        its.append(simu._PhaseField__Niter)
        print(name, "step", k, "F", f, "dmax", d.max(), "Niter", its[-1])
    res = dict(mesh_arrays(m), split="Miehe", regu="AT2", solver=solver, planeStress=False, E=210000.0, v=0.3,
               Gc=2.7, l0=0.1, dU=dU, tol=tol, maxIter=maxIter, u=np.array(us), d=np.array(ds), F=np.array(Fs),
               Niter=np.array(its), bottom=bottom, top=top, top_dofs=top_dofs)
    np.savez_compressed(os.path.join(out, f"{name}.npz"), **res)


def _pf_solver_cases(R, out):
    pf_solver_case(R, "pf_tri3_boundconstrain", gmesh.Mesh_Tri3_Rect(1.0, 1.0, 16, 16), "BoundConstrain", 4, 4e-3,
                   out)
    # HistoryDamage: load steps small enough that the crack grows over several
    # steps (a larger step breaks the plate within one step in dozens of
    # staggered iterations, a path that rounding can change)
    pf_solver_case(R, "pf_tri3_historydamage", gmesh.Mesh_Tri3_Rect(1.0, 1.0, 16, 16), "HistoryDamage", 6,
                   1.5e-3, out)


def _quadratic_cases(R, out):
    """TRI6 / QUAD8 (SEG3 edges), TETRA10 (TRI6 faces), HEXA20 (QUAD8 faces) and
    HEXA27 (QUAD9 faces): elastic cantilevers,
    phase-field systems at a prescribed state and the post-processing
    results."""
    elastic_case(R, "el_tri6", gmesh.Mesh_Tri6_Rect(120.0, 13.0, 12, 3), 210000.0, 0.25, False, 1.0, -10.0, "y",
                 out)
    elastic_case(R, "el_quad8", gmesh.Mesh_Quad8_Rect(120.0, 13.0, 12, 3), 210000.0, 0.3, True, 13.0,
                 -800 / 13**2, "y", out)
    elastic_case(R, "el_tetra10", gmesh.Mesh_Tetra10_Box(60.0, 10.0, 10.0, 4, 2, 2), 210000.0, 0.3, False, 1.0,
                 -1.0, "z", out)
    pf_state_case(R, "pfsys_tri6_miehe_at2", gmesh.Mesh_Tri6_Rect(1.0, 1.0, 6, 6), "Miehe", "AT2", out)
    pf_state_case(R, "pfsys_quad8_amor_at1", gmesh.Mesh_Quad8_Rect(1.0, 1.0, 5, 5), "Amor", "AT1", out)
    pf_state_case(R, "pfsys_tetra10_miehe_at2", gmesh.Mesh_Tetra10_Box(1.0, 1.0, 0.5, 2, 2, 1), "Miehe", "AT2", out)
    elastic_case(R, "el_hexa20", gmesh.Mesh_Hexa20_Box(60.0, 10.0, 10.0, 4, 2, 2), 210000.0, 0.3, False, 1.0, -1.0,
                 "z", out)
    elastic_case(R, "el_hexa27", gmesh.Mesh_Hexa27_Box(60.0, 10.0, 10.0, 3, 1, 1), 210000.0, 0.3, False, 1.0, -1.0,
                 "z", out)
    pf_state_case(R, "pfsys_hexa20_miehe_at2", gmesh.Mesh_Hexa20_Box(1.0, 1.0, 0.5, 2, 2, 1), "Miehe", "AT2", out)
    results_case(R, "res_hexa27", gmesh.Mesh_Hexa27_Box(6.0, 2.0, 2.0, 2, 1, 1), 210000.0, 0.3, False, 1.0, out)
    results_case(R, "res_quad8", gmesh.Mesh_Quad8_Rect(12.0, 3.0, 6, 2), 210000.0, 0.3, True, 13.0, out)
    results_case(R, "res_tetra10", gmesh.Mesh_Tetra10_Box(6.0, 2.0, 2.0, 3, 1, 1), 210000.0, 0.3, False, 1.0, out)


def main():
    args = [a for a in sys.argv[1:] if not a.startswith("--only=")]
    only = [a.split("=", 1)[1].split(",") for a in sys.argv[1:] if a.startswith("--only=")]
    only = set(only[0]) if only else None
    ref = args[0] if args else os.environ.get("EASYFEA_REFERENCE")
    if not ref:
        sys.exit("usage: make_golden.py <path to EasyFEA sources> [--only=name,...] "
                 "(or set EASYFEA_REFERENCE)")
    R = load_reference(ref)
    if only is not None:  # regenerate the named fixtures only
        for name, fn in CASES.items():
            if name in only:
                fn(R, HERE)
        return
    out = HERE
    import scipy
    np.savez(os.path.join(out, "versions.npz"), numpy=np.__version__, scipy=scipy.__version__)

    elastic_case(R, "el_quad4", gmesh.Mesh_Quad4_Rect(120.0, 13.0, 24, 4), 210000.0, 0.3, True, 13.0,
                 -800 / 13**2, "y", out)
    elastic_case(R, "el_tri3", gmesh.Mesh_Tri3_Rect(120.0, 13.0, 12, 4), 210000.0, 0.25, False, 1.0,
                 -10.0, "y", out)
    elastic_case(R, "el_quad9", gmesh.Mesh_Quad9_Rect(120.0, 13.0, 6, 2), 210000.0, 0.3, True, 13.0,
                 -800 / 13**2, "y", out)
    elastic_case(R, "el_hexa8", gmesh.Mesh_Hexa8_Box(60.0, 10.0, 10.0, 6, 2, 2), 210000.0, 0.3, False, 1.0,
                 -1.0, "z", out)
    rng = np.random.default_rng(3)
    mq = gmesh.Mesh_Quad4_Rect(120.0, 13.0, 12, 3)
    Eh = 210000.0 * np.exp(0.3 * rng.standard_normal(mq.Ne))
    elastic_case(R, "el_quad4_hetero", mq, Eh, 0.3, True, 13.0, -800 / 13**2, "y", out)
    _el_hexa8_hetero(R, out)
    # full-size 2D cantilever: QUAD4 240x26, L=120, h=13, t=13
    elastic_case(R, "el_cantilever_240x26", gmesh.Mesh_Quad4_Rect(120.0, 13.0, 240, 26), 210000.0, 0.3,
                 True, 13.0, -800 / 13**2, "y", out)

    split_case(R, out)

    pf_case(R, "pf_tri3_miehe_at2", gmesh.Mesh_Tri3_Rect(1.0, 1.0, 16, 16), "Miehe", "AT2", False,
            210000.0, 0.3, 2.7, 0.1, 4, 4e-3, out)
    pf_case(R, "pf_quad4_amor_at2", gmesh.Mesh_Quad4_Rect(1.0, 1.0, 12, 12), "Amor", "AT2", True,
            210000.0, 0.3, 2.7, 0.1, 3, 6e-3, out)
    for split, regu, m in (("Amor", "AT1", gmesh.Mesh_Quad4_Rect(1.0, 1.0, 10, 10)),
                           ("Miehe", "AT1", gmesh.Mesh_Tri3_Rect(1.0, 1.0, 10, 10)),
                           ("Miehe", "AT2", gmesh.Mesh_Hexa8_Box(1.0, 1.0, 0.5, 4, 4, 2))):
        pf_state_case(R, f"pfsys_{m.elemType.value.lower()}_{split.lower()}_{regu.lower()}", m, split, regu, out)
    pf_case(R, "pf_hexa8_miehe_at2", gmesh.Mesh_Hexa8_Box(1.0, 1.0, 0.25, 6, 6, 1), "Miehe", "AT2", False,
            210000.0, 0.3, 2.7, 0.2, 2, 4e-3, out)
    _results_cases(R, out)


def _el_hexa8_hetero(R, out):
    rng = np.random.default_rng(5)
    mh = gmesh.Mesh_Hexa8_Box(60.0, 10.0, 10.0, 6, 2, 2)
    Eh = 210000.0 * np.exp(0.3 * rng.standard_normal(mh.Ne))
    elastic_case(R, "el_hexa8_hetero", mh, Eh, 0.3, False, 1.0, -1.0, "z", out)


def _higher_order_cases(R, out):
    """TRI10 (SEG4 edges), TRI15 (SEG5 edges) and the prisms PRISM6 (QUAD4 and
    TRI3 faces), PRISM15 (QUAD8, TRI6) and PRISM18 (QUAD9, TRI6): elastic
    cantilevers (the prisms loaded on an end face z = Lz, whose TRI faces
    share the mesh with the QUAD side faces, or on x = L), phase-field
    systems at a prescribed state and the post-processing results."""
    elastic_case(R, "el_tri10", gmesh.Mesh_Tri10_Rect(120.0, 13.0, 8, 2), 210000.0, 0.25, True, 2.0, -10.0, "y",
                 out)
    elastic_case(R, "el_tri15", gmesh.Mesh_Tri15_Rect(120.0, 13.0, 6, 2), 210000.0, 0.3, False, 1.0, -10.0, "y",
                 out)
    elastic_case(R, "el_prism6", gmesh.Mesh_Prism6_Box(60.0, 10.0, 10.0, 6, 2, 2), 210000.0, 0.3, False, 1.0, -1.0,
                 "z", out, load_axis=2)
    elastic_case(R, "el_prism15", gmesh.Mesh_Prism15_Box(60.0, 10.0, 10.0, 4, 2, 2), 210000.0, 0.3, False, 1.0,
                 -1.0, "z", out)
    elastic_case(R, "el_prism18", gmesh.Mesh_Prism18_Box(60.0, 10.0, 10.0, 3, 1, 1), 210000.0, 0.3, False, 1.0,
                 -1.0, "z", out, load_axis=2)
    pf_state_case(R, "pfsys_tri10_miehe_at2", gmesh.Mesh_Tri10_Rect(1.0, 1.0, 4, 4), "Miehe", "AT2", out)
    pf_state_case(R, "pfsys_tri15_amor_at1", gmesh.Mesh_Tri15_Rect(1.0, 1.0, 3, 3), "Amor", "AT1", out)
    pf_state_case(R, "pfsys_prism6_miehe_at2", gmesh.Mesh_Prism6_Box(1.0, 1.0, 0.5, 3, 3, 2), "Miehe", "AT2", out)
    pf_state_case(R, "pfsys_prism15_amor_at2", gmesh.Mesh_Prism15_Box(1.0, 1.0, 0.5, 2, 2, 1), "Amor", "AT2", out)
    pf_state_case(R, "pfsys_prism18_miehe_at1", gmesh.Mesh_Prism18_Box(1.0, 1.0, 0.5, 2, 2, 1), "Miehe", "AT1",
                  out)
    results_case(R, "res_tri10", gmesh.Mesh_Tri10_Rect(12.0, 3.0, 6, 2), 210000.0, 0.3, True, 13.0, out)
    results_case(R, "res_tri15", gmesh.Mesh_Tri15_Rect(12.0, 3.0, 4, 2), 210000.0, 0.3, False, 1.0, out)
    results_case(R, "res_prism6", gmesh.Mesh_Prism6_Box(6.0, 2.0, 2.0, 3, 1, 2), 210000.0, 0.3, False, 1.0, out)
    results_case(R, "res_prism15", gmesh.Mesh_Prism15_Box(6.0, 2.0, 2.0, 2, 1, 1), 210000.0, 0.3, False, 1.0, out)
    results_case(R, "res_prism18", gmesh.Mesh_Prism18_Box(6.0, 2.0, 2.0, 2, 1, 1), 210000.0, 0.3, False, 1.0, out)


# fixtures that can be regenerated alone (--only=name,...)
CASES = {"el_hexa8_hetero": _el_hexa8_hetero, "pf_conv": _pf_conv_cases, "field_load": _field_load_cases,
         "split": split_case, "pf_splits": _pf_split_cases, "tetra4": _tetra4_cases,
         "pf_curve_tri3_200x200": pf_curve_case, "results": _results_cases, "anisot": anisot_case,
         "pf_solvers": _pf_solver_cases, "quadratic": _quadratic_cases, "higher_order": _higher_order_cases}


if __name__ == "__main__":
    main()
