"""CPU oracle drivers: elastic solve and phase-field staggered scheme -- TEST
INFRASTRUCTURE ONLY (the checker, never the product path).

Restates the reference's simulation-level algorithms on plain arrays:
``Simulations.Elastic`` (EasyFEA/Simulations/_elastic.py:123-152, _simu.py:1104-1144,
:1735-1968, Solvers.py:502-553) and ``Simulations.PhaseField``
(EasyFEA/Simulations/_phasefield.py:303-573, :613-630).  Solves use scipy
``spsolve`` exactly as the reference's default solver does (Solvers.py:361-362).
"""

from __future__ import annotations

import numpy as np
import scipy.sparse as sp

from . import fem


class OracleMesh:
    """Plain-array mesh: main group (elem, connect) + boundary groups."""

    def __init__(self, elem, coord, connect, boundary=()):
        self.elem = elem
        self.coord = np.asarray(coord, float)
        self.connect = np.asarray(connect, np.int64)
        self.boundary = [(e, np.asarray(c, np.int64)) for e, c in boundary]
        self.dim = fem.ELEM_DIM[elem]
        used = np.zeros(self.coord.shape[0], bool)
        used[self.connect.ravel()] = True
        for _, c in self.boundary:
            used[c.ravel()] = True
        self.orphans = np.nonzero(~used)[0]

    @property
    def Nn(self):
        return self.coord.shape[0]

    @classmethod
    def from_mesh(cls, mesh):
        """From an ``easyfea_gb300.mesh.Mesh`` (array access only)."""
        g = mesh.groupElem
        bnd = [(b.elemType.value, b.connect) for b in mesh.Get_list_groupElem(mesh.dim - 1)]
        return cls(g.elemType.value, mesh.coord, g.connect, bnd)


def neumann(mesh: OracleMesh, loads, dof_n, thickness):
    """b from the Neumann list -- _simu.py:1750-1756 (COO sum of duplicate dofs)."""
    Ndof = mesh.Nn * dof_n
    avail = fem.UNKNOWNS[dof_n]
    dofs_all, vals_all = [np.zeros(0, np.int64)], [np.zeros(0)]
    for nodes, values, unknowns in loads:
        for belem, bcon in mesh.boundary:
            d, v = fem.surf_load(belem, mesh.coord, bcon, nodes, values, unknowns, avail,
                                 thickness if mesh.dim == 2 else 1.0)
            dofs_all.append(d)
            vals_all.append(v)
    dofs = np.concatenate(dofs_all)
    vals = np.concatenate(vals_all)
    return np.bincount(dofs, weights=vals, minlength=Ndof)


def dirichlet(mesh: OracleMesh, conds, dof_n):
    """(dofs, values) COO lists -- _simu.py:2400-2469 (values summed on duplicates)."""
    avail = fem.UNKNOWNS[dof_n]
    dofs, vals = [np.zeros(0, np.int64)], [np.zeros(0)]
    for nodes, values, unknowns in conds:
        nodes = np.asarray(nodes, np.int64)
        v = np.zeros((nodes.size, len(unknowns)))
        for i, val in enumerate(values):
            if callable(val):
                x, y, z = mesh.coord[nodes].T
                v[:, i] = val(x, y, z)
            else:
                v[:, i] = val
        dofs.append(fem.dofs_nodes(nodes, unknowns, avail))
        vals.append(v.ravel())
    return np.concatenate(dofs), np.concatenate(vals)


def elastic_system(mesh: OracleMesh, E, v, planeStress=True, thickness=1.0, rho=1.0, C=None):
    """K, M (CSR) -- _elastic.py:123-152 (K_e, M_e x thickness in 2D) + assembly.
    ``C``: a Kelvin-Mandel law in place of the isotropic (E, v) one."""
    dim = mesh.dim
    C = fem.isotropic_C(E, v, dim, planeStress) if C is None else np.asarray(C, float)
    geo = fem.Geometry(mesh.elem, mesh.coord, mesh.connect, "rigi")
    K_e = fem.K_elastic_e(geo, C)
    geom = fem.Geometry(mesh.elem, mesh.coord, mesh.connect, "mass")
    M_e = fem.UV_e(geom, rho, dof_n=dim)
    if dim == 2:
        K_e = K_e * thickness
        M_e = M_e * thickness
    Ndof = mesh.Nn * dim
    inv, ind, ptr, nnz = fem.csr_map(mesh.connect, dim, Ndof)
    K = fem.assemble_csr(K_e, inv, ind, ptr, nnz, Ndof)
    M = fem.assemble_csr(M_e, inv, ind, ptr, nnz, Ndof)
    return K, M


def elastic_solve(mesh: OracleMesh, E, v, planeStress, thickness, dir_conds, loads, C=None):
    """Simulations.Elastic.Solve() restated: returns (u, K, b)."""
    dim = mesh.dim
    K, _ = elastic_system(mesh, E, v, planeStress, thickness, C=C)
    b = neumann(mesh, loads, dim, thickness)
    dk, dv = dirichlet(mesh, dir_conds, dim)
    orphan = fem.dofs_nodes(mesh.orphans, fem.UNKNOWNS[dim], fem.UNKNOWNS[dim])
    u = fem.solve_r1(K, b, dk, dv, orphan)
    return u, K, b


def bounded_lsq_exact(A, b, lb, ub, tol=1e-14, max_outer=200):
    """The minimiser of ||A x - b|| over lb <= x <= ub (A nonsingular, so the
    cost is strictly convex): projected Newton -- the binding set from the
    gradient A^T (A x - b), a least-squares step (LSQR) on the other
    unknowns, projection on the box and step halving until the cost drops --
    until the projected gradient is below tol times its start value."""
    import scipy.sparse.linalg as sla

    x = np.clip(np.asarray(lb, float), lb, ub)
    g0 = max(np.linalg.norm(A.T @ b), 1e-300)
    for _ in range(max_outer):
        r = A @ x - b
        g = A.T @ r
        free = ~(((x <= lb) & (g > 0)) | ((x >= ub) & (g < 0)))
        if np.linalg.norm(g[free]) <= tol * g0:
            break
        dx = np.zeros_like(x)
        dx[free] = sla.lsqr(A[:, free], -r, atol=1e-15, btol=1e-15, iter_lim=100000)[0]
        f0, a = 0.5 * r @ r, 1.0
        while True:
            xn = np.clip(x + a * dx, lb, ub)
            rn = A @ xn - b
            if 0.5 * rn @ rn <= f0 + 1e-4 * g @ (xn - x) or a < 1e-12:
                break
            a *= 0.5
        x = xn
    return x


class PhaseFieldOracle:
    """Staggered phase-field scheme (Simulations/_phasefield.py:303-432) with the
    History solver (psi+ max against the committed field, :494-538, committed in
    Save_Iter :613-630)."""

    def __init__(self, mesh: OracleMesh, E, v, planeStress, thickness, split, regu, Gc, l0, A=None, C=None, S=None):
        """``C``, ``S``: a Kelvin-Mandel law and its compliance in place of the
        isotropic (E, v) one (the Bourdin and anisotropic splits)."""
        self.mesh = mesh
        self.dim = dim = mesh.dim
        self.E, self.v = E, v
        self.planeStress = planeStress
        self.thickness = thickness if dim == 2 else 1.0
        self.split, self.regu, self.Gc, self.l0 = split, regu, Gc, l0
        self.A = np.eye(dim) if A is None else np.asarray(A, float)
        self.lmbda, self.mu = fem.lame(E, v, dim, planeStress) if C is None else (0.0, 0.0)
        self.C = fem.isotropic_C(E, v, dim, planeStress) if C is None else np.asarray(C, float)
        self.S = None if S is None else np.asarray(S, float)
        self.u = np.zeros(mesh.Nn * dim)
        self.d = np.zeros(mesh.Nn)
        self.H_old = None
        self.psiP = None
        self.solver = "History"  # History, HistoryDamage or BoundConstrain (_phasefield.py:105-110)
        # BoundConstrain: "lsq_linear" (the reference's scipy call, which stops
        # at a 1e-10 relative change of the cost: about 1e-5 from the
        # minimiser where bounds are active) or "exact" (the minimiser itself)
        self.bounded_solver = "lsq_linear"
        self.geo_r = fem.Geometry(mesh.elem, mesh.coord, mesh.connect, "rigi")
        self.geo_m = fem.Geometry(mesh.elem, mesh.coord, mesh.connect, "mass")
        self.map_u = fem.csr_map(mesh.connect, dim, mesh.Nn * dim)
        self.map_d = fem.csr_map(mesh.connect, 1, mesh.Nn)
        self.dir_u = []
        self.dir_d = []
        self.Ku = None
        self.Kd = None
        self.Fd = None

    def strain(self, geo):
        """Calc_Epsilon_e_pg, Elastic/_laws.py:127-157."""
        u_e = self.u[fem.assembly_e(self.mesh.connect, self.dim)]
        return np.einsum("epij,ej->epi", fem.B_e_pg(geo.dNx), u_e)

    def damage_system(self):
        """__Construct_Damage_Matrix, _phasefield.py:540-573."""
        eps = self.strain(self.geo_m)
        cP, cM = fem.split_C(eps, self.split, self.lmbda, self.mu, self.dim, self.C, E=self.E, v=self.v, S=self.S,
                              planeStress=self.planeStress)
        psiP, _ = fem.psi_split(eps, cP, cM)
        if self.H_old is not None and self.H_old.shape == psiP.shape:
            psiP = np.where(psiP - self.H_old < 0, self.H_old, psiP)
        self.psiP = psiP
        r, f, k = fem.pf_r_f_k(psiP, self.regu, self.Gc, self.l0)
        R_e = fem.UV_e(self.geo_m, r)
        D_e = fem.GradU_A_GradV_e(self.geo_r, self.A, k)
        F_e = fem.V_e(self.geo_m, f)
        K_e = (R_e + D_e) * self.thickness
        F_e = F_e * self.thickness
        inv, ind, ptr, nnz = self.map_d
        self.Kd = fem.assemble_csr(K_e, inv, ind, ptr, nnz, self.mesh.Nn)
        self.Fd = fem.assemble_vec(F_e, self.mesh.connect, 1, self.mesh.Nn)
        return self.Kd, self.Fd

    def elastic_system(self):
        """__Construct_Elastic_Matrix, _phasefield.py:444-482 (g = (1-d)^2 + 1e-12)."""
        eps = self.strain(self.geo_r)
        cP, cM = fem.split_C(eps, self.split, self.lmbda, self.mu, self.dim, self.C, E=self.E, v=self.v, S=self.S,
                              planeStress=self.planeStress)
        d_e = self.d[self.mesh.connect]
        d_pg = np.einsum("pn,en->ep", self.geo_r.N, d_e)
        g = (1 - d_pg) ** 2 + 1e-12
        c = g[..., None, None] * cP + cM
        K_e = fem.K_elastic_e(self.geo_r, c) * self.thickness
        inv, ind, ptr, nnz = self.map_u
        self.Ku = fem.assemble_csr(K_e, inv, ind, ptr, nnz, self.mesh.Nn * self.dim)
        return self.Ku

    # The reference assembles lazily: Get_K_C_M_F re-assembles a system only
    # when its flag says the other field changed (_phasefield.py:248-269); the
    # damage solve clears the displacement flag and the elastic solve the
    # damage flag (:366-374).  The energy criteria (convOption 1, 2) read the
    # systems through the same flags, which decides which displacement the
    # History field is computed from when Save_Iter commits it.
    def _kd(self):
        if not getattr(self, "_upd_d", False) or self.Kd is None:
            self.damage_system()
            self._upd_d = True
        return self.Kd

    def _ku(self):
        if not getattr(self, "_upd_u", False) or self.Ku is None:
            self.elastic_system()
            self._upd_u = True
        return self.Ku

    def solve_damage(self):
        Kd, Fd = self._kd(), self.Fd
        dk, dv = dirichlet(self.mesh, self.dir_d, 1)
        if self.solver == "BoundConstrain":
            # scipy.optimize.lsq_linear on the r1 system with d_n <= d <= 1
            # (Solvers.py:376-383, _phasefield.py:148-163; the reference takes
            # these full-length bounds, so its damage problem has no Dirichlet DOF)
            from scipy import optimize

            assert len(dk) == 0, "bounded damage solve without damage Dirichlet conditions"
            lb = self.d.copy()
            lb[lb >= 1] = 1 - np.finfo(float).eps
            ub = np.ones(lb.shape)
            if self.bounded_solver == "lsq_linear":
                self.d = optimize.lsq_linear(Kd.tocsr(), Fd, bounds=(lb, ub), tol=1e-10, method="trf", verbose=0)["x"]
            else:
                self.d = bounded_lsq_exact(Kd.tocsr(), Fd, lb, ub)
        else:
            self.d = fem.solve_r1(Kd, Fd, dk, dv)
        return self.d

    def solve_elastic(self):
        Ku = self._ku()
        b = np.zeros(self.mesh.Nn * self.dim)
        dk, dv = dirichlet(self.mesh, self.dir_u, self.dim)
        self.u = fem.solve_r1(Ku, b, dk, dv)
        return self.u

    def psi_crack(self):
        """_Calc_Psi_Crack, _phasefield.py:799-817: 1/2 d.Kd d."""
        Kd = self._kd()
        return 0.0 if np.linalg.norm(self.d) == 0 else 0.5 * self.d @ (Kd @ self.d)

    def psi_elas(self):
        """_Calc_Psi_Elas, _phasefield.py:775-797: 1/2 u.Ku u."""
        Ku = self._ku()
        return 0.0 if np.linalg.norm(self.u) == 0 else 0.5 * self.u @ (Ku @ self.u)

    def solve(self, tolConv=1.0, maxIter=500, convOption=0):
        """Staggered loop, _phasefield.py:303-432 (no external forces: the work
        of f_u in convOption 2 is zero)."""
        assert convOption in (0, 1, 2, 3)
        old_damage = self.d.copy()
        Niter = 0
        converged = False
        convIter = 0.0
        while not converged and Niter < maxIter:
            Niter += 1
            d_n = self.d.copy()
            u_n = self.u.copy()
            if convOption == 1:
                E_n = self.psi_crack()
            elif convOption == 2:
                E_n = self.psi_crack() + self.psi_elas()
            d_np1 = self.solve_damage()
            self._upd_u = False
            u_np1 = self.solve_elastic()
            self._upd_d = False
            if convOption == 0:
                convIter = np.max(np.abs(d_np1 - d_n))
            elif convOption in (1, 2):
                E_np1 = self.psi_crack()
                if convOption == 2:
                    E_np1 += self.psi_elas()
                convIter = abs(E_n - E_np1) if E_np1 == 0 else abs((E_n - E_np1) / E_np1)
            else:
                diffU = np.abs(u_np1 - u_n)
                diffU[u_np1 != 0] *= 1 / np.abs(u_np1[u_np1 != 0])
                diffD = np.abs(d_np1 - d_n)
                diffD[d_np1 != 0] *= 1 / np.abs(d_np1[d_np1 != 0])
                convU, convD = np.sum(diffU), np.sum(diffD)
                convIter = max(convD, convU)
            if tolConv == 1 or d_np1.max() == 0:
                converged = True
            elif convOption == 3:
                converged = (convD <= tolConv) and (convU <= tolConv * 0.999)
            else:
                converged = convIter <= tolConv
        if self.solver == "HistoryDamage":  # _phasefield.py:412-416
            self.d = np.maximum(self.d, old_damage)
        self.Niter = Niter
        self.convIter = convIter
        return self.u, self.d, converged

    def save_iter(self):
        if self.solver == "History":
            self.H_old = self.psiP

    def reaction(self, dofs):
        """Calc_Reaction, _simu.py:212-260: Ku[dofs] @ u."""
        return self._ku()[dofs] @ self.u
