"""Checksums of the 256-instance random-material batch, from the CPU oracle.

The batched workload (``easyfea_gb300.batching.random_material_cantilevers(n=256,
seed=0)``: plane-stress cantilevers of 2k-200k DOF with per-element moduli)
is too large to store solutions for.  For every instance this script solves
it with the oracle (``oracle.simulate.elastic_solve``: the reference's
element matrices, bincount assembly and SuperLU, pinned against the
reference's own fixtures by tests/test_oracle_golden.py) and stores
size-independent checksums of the displacement: its 2-norm, its largest
magnitude and its dot product with a seeded weight vector (uniform in
[-1, 1], seed 1000 + instance).  Run::

    python tests/golden/make_batch_golden.py [processes]
"""

from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

N_INSTANCES = 256
SEED = 0


def weights(i: int, n: int) -> np.ndarray:
    return np.random.default_rng(1000 + i).uniform(-1.0, 1.0, n)


def _solve(i):
    os.environ["OMP_NUM_THREADS"] = "1"
    from easyfea_gb300.batching import random_material_cantilevers
    from oracle.simulate import OracleMesh, elastic_solve

    (m, E), = random_material_cantilevers(n=1, seed=SEED + i)
    x = m.coord
    left = np.where(x[:, 0] == 0)[0]
    right = np.where(x[:, 0] == x[:, 0].max())[0]
    u, _, _ = elastic_solve(OracleMesh.from_mesh(m), E, 0.3, True, 13.0, [(left, [0.0, 0.0], ["x", "y"])],
                            [(right, [-800 / 13**2], ["y"])])
    return i, u.size, float(np.linalg.norm(u)), float(np.abs(u).max()), float(weights(i, u.size) @ u)


def main():
    import multiprocessing as mp

    procs = int(sys.argv[1]) if len(sys.argv) > 1 else (os.cpu_count() or 1)
    out = np.zeros((N_INSTANCES, 4))
    with mp.get_context("spawn").Pool(procs) as pool:
        for i, n, nrm, amax, wdot in pool.imap_unordered(_solve, range(N_INSTANCES)):
            out[i] = (n, nrm, amax, wdot)
            print(i, n, nrm, flush=True)
    np.savez_compressed(os.path.join(HERE, "batch_random_material_256.npz"), ndof=out[:, 0].astype(np.int64),
                        norm=out[:, 1], absmax=out[:, 2], wdot=out[:, 3], seed=SEED)


if __name__ == "__main__":
    main()
