"""Batched cluster-resident PCG (gfea_batch_pcg) against single solves and the oracle."""

import numpy as np
import pytest

from easyfea_gb300 import mesh as gmesh

pytestmark = pytest.mark.gpu


def elastic_system(m, E, v=0.3, thickness=13.0, load=-800 / 13**2, rtol=1e-10):
    from easyfea_gb300 import Models
    from easyfea_gb300 import simulations as Simulations
    from easyfea_gb300.batching import BatchSystem

    dim = m.dim
    mat = Models.Elastic.Isotropic(dim, E=E, v=v, planeStress=True, thickness=thickness)
    simu = Simulations.Elastic(m, mat)
    L = m.coord[:, 0].max()
    left = m.Nodes_Conditions(lambda x, y, z: x == 0)
    right = m.Nodes_Conditions(lambda x, y, z: x == L)
    unk = ["x", "y"] if dim == 2 else ["x", "y", "z"]
    simu.add_dirichlet(left, [0.0] * dim, unk)
    simu.add_surfLoad(right, [load], ["y" if dim == 2 else "z"])
    op = simu.K_device
    b = simu._neumann_vec("elastic")
    known, x = simu._dirichlet_state("elastic", b)
    return simu, BatchSystem(op, b, x, known, rtol=rtol), (left, right)


def mixed_batch():
    ms = [gmesh.Mesh_Quad4_Rect(120.0, 13.0, 48, 6), gmesh.Mesh_Tri3_Rect(120.0, 13.0, 30, 5),
          gmesh.Mesh_Quad9_Rect(120.0, 13.0, 12, 3), gmesh.Mesh_Hexa8_Box(60.0, 10.0, 10.0, 12, 2, 2),
          gmesh.Mesh_Quad4_Rect(120.0, 13.0, 120, 13)]
    return [elastic_system(m, 210000.0)[1] for m in ms]


@pytest.mark.parametrize("coarse", [0, -1])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batch_matches_single_solves(precision, coarse):
    """Block-Jacobi (coarse 0) and two-level (coarse -1) batched PCG."""
    from easyfea_gb300.batching import solve_batch
    from easyfea_gb300.device import pcg

    systems = mixed_batch()
    x0 = [s.x.clone() for s in systems]
    infos = solve_batch(systems, precision=precision, coarse=coarse)
    for s, x_init, info in zip(systems, x0, infos):
        assert info.status == 0
        assert info.rel_residual <= max(1e-10, info.floor_rel)
        xs = x_init.clone()
        pcg(s.op, s.b, xs, s.known, rtol=1e-12, precision="fp64")
        ref = xs.cpu().numpy()
        err = np.abs(s.x.cpu().numpy() - ref).max() / np.abs(ref).max()
        assert err <= 1e-7, f"relative difference {err:.3e}"


@pytest.mark.parametrize("coarse", [0, -1])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_result_identical_alone_and_in_the_mix(precision, coarse):
    """A system's solution does not depend on the other systems of the batch:
    bit for bit with block-Jacobi; with the coarse level within 1e-8 (its
    coarse matrix is summed with FP64 atomics when it is rebuilt)."""
    from easyfea_gb300.batching import solve_batch

    systems = mixed_batch()
    x0 = [s.x.clone() for s in systems]
    solve_batch(systems, precision=precision, coarse=coarse)
    mixed = [s.x.clone() for s in systems]
    for k in (0, 3, 4):
        s = systems[k]
        s.x.copy_(x0[k])
        solve_batch([s], precision=precision, coarse=coarse)
        a, b = s.x.cpu().numpy(), mixed[k].cpu().numpy()
        if coarse == 0:
            assert np.array_equal(a, b), f"system {k} differs alone / in the mix"
        else:
            assert np.abs(a - b).max() <= 1e-8 * np.abs(b).max(), f"system {k} differs alone / in the mix"


def test_two_level_batch_cuts_iterations():
    """The coarse level inside the persistent kernel: same answer as
    block-Jacobi with several times fewer iterations on the slender bars."""
    from easyfea_gb300.batching import solve_batch

    systems = mixed_batch()
    x0 = [s.x.clone() for s in systems]
    bj = solve_batch(systems, precision="mixed", coarse=0)
    u_bj = [s.x.clone() for s in systems]
    for s, x in zip(systems, x0):
        s.x.copy_(x)
    tl = solve_batch(systems, precision="mixed", coarse=-1)
    for s, ub, i0, i1 in zip(systems, u_bj, bj, tl):
        ref = ub.cpu().numpy()
        assert np.abs(s.x.cpu().numpy() - ref).max() <= 1e-7 * np.abs(ref).max()
    big = 4  # the 120 x 13 QUAD4 bar
    assert tl[big].iterations * 3 < bj[big].iterations, (tl[big].iterations, bj[big].iterations)


def test_random_material_batch_matches_oracle():
    """Per-element E from a random Fourier field (the batched random-material
    workload), against the oracle's SuperLU solves."""
    from easyfea_gb300.batching import random_material_cantilevers, solve_batch
    from oracle.simulate import OracleMesh, elastic_solve

    inst = random_material_cantilevers(n=6, seed=100, dof_min=300, dof_max=3000)
    sims = [elastic_system(m, E) for m, E in inst]
    infos = solve_batch([s[1] for s in sims], precision="mixed")
    for (m, E), (simu, sys_, (left, right)), info in zip(inst, sims, infos):
        assert info.status == 0
        u_ref, K_ref, _ = elastic_solve(OracleMesh.from_mesh(m), E, 0.3, True, 13.0,
                                        [(left, [0.0, 0.0], ["x", "y"])], [(right, [-800 / 13**2], ["y"])])
        K = simu.Get_K_C_M_F()[0]
        assert abs(K - K_ref).max() <= 1e-12 * abs(K_ref).max()
        u = sys_.x.cpu().numpy()
        assert np.abs(u - u_ref).max() <= 1e-8 * np.abs(u_ref).max()


@pytest.mark.parametrize("coarse", [0, -1])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_graph_captured_batch_replays(precision, coarse):
    """Re-assembly of every operator, the coarse matrices and inverses, the
    reset of x and the persistent solve captured as one CUDA graph: each
    replay gives the direct batch's result (bit for bit with block-Jacobi,
    within 1e-8 with the coarse level, whose matrix is summed with atomics)."""
    import torch

    from easyfea_gb300.batching import GraphBatch, solve_batch

    systems = mixed_batch()
    x0 = [s.x.clone() for s in systems]
    solve_batch(systems, precision=precision, coarse=coarse)
    direct = [s.x.clone() for s in systems]
    for s, x in zip(systems, x0):
        s.x.copy_(x)
    vals = [s.op.vals64.clone() for s in systems]

    def pre():  # stand-in for re-assembly: rewrite the values in place
        for s, v in zip(systems, vals):
            s.op.vals64.copy_(v)
            if s.op.vals32 is not None:
                s.op.vals32.copy_(v)

    gb = GraphBatch(systems, precision=precision, pre=pre, coarse=coarse)
    for _ in range(2):
        for s in systems:
            s.x.zero_()
        gb.replay()
        infos = gb.results()
        assert all(i.status == 0 for i in infos)
        for s, d in zip(systems, direct):
            if coarse == 0:
                assert torch.equal(s.x, d)
            else:
                assert (s.x - d).abs().max() <= 1e-8 * d.abs().max()


def test_random_material_256_in_one_graph_launch_matches_oracle(golden):
    """The batched random-material workload as specified: 256 cantilevers of
    2k-200k DOF with per-element E, assembled (element kernels), given their
    coarse levels and solved (one persistent launch) inside one CUDA graph,
    replayed twice; every instance against the oracle's SuperLU solution
    through its checksums (2-norm, largest magnitude, seeded weighted sum)
    within 1e-8."""
    from easyfea_gb300.batching import RandomMaterialBatch, random_material_cantilevers

    g = golden("batch_random_material_256")
    inst = random_material_cantilevers(n=256, seed=int(g["seed"]))
    rb = RandomMaterialBatch(inst, precision="mixed", rtol=1e-10)
    for _ in range(2):
        for s in rb.systems:
            s.x.fill_(1.0)  # garbage: the graph resets x itself
        rb.replay()
        infos = rb.results()
        assert all(i.status == 0 for i in infos), [i.status for i in infos if i.status]
        for i, s in enumerate(rb.systems):
            u = s.x.cpu().numpy()
            assert u.size == g["ndof"][i]
            w = np.random.default_rng(1000 + i).uniform(-1.0, 1.0, u.size)
            assert abs(np.linalg.norm(u) - g["norm"][i]) <= 1e-8 * g["norm"][i], i
            assert abs(np.abs(u).max() - g["absmax"][i]) <= 1e-8 * g["absmax"][i], i
            assert abs(w @ u - g["wdot"][i]) <= 1e-8 * np.linalg.norm(w) * g["norm"][i], i
