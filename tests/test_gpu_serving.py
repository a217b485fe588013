"""Solve service on the GPU: concurrent (continuous-batching) results against
one-at-a-time FP64 solves, and each result the same alone and in the mix."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def small_stream(n=16, seed=5):
    from easyfea_gb300 import serving

    mix = serving.StreamMix(quad_dof=(1e3, 2e4), hexa_dof=(1e4, 3e4), pf_elems=(800, 3200), classes=3)
    return serving.poisson_stream(2000.0, n, seed=seed, mix=mix)


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def test_served_mixed_matches_plain_fp64():
    from easyfea_gb300 import serving

    cache = serving.MeshCache()
    t, reqs, sessions = small_stream()
    with serving.Server(workers=4, precision="mixed", cache=cache) as srv:
        served = serving.run_stream(srv, t, reqs)
    assert all(r.error is None for r in served), [r.error for r in served if r.error]
    # the same requests, fresh phase-field sessions, one at a time in FP64
    t2, reqs2, _ = small_stream()
    plain = serving.run_plain(reqs2, cache, precision="fp64")
    for a, b in zip(served, plain):
        assert a.kind == b.kind
        if a.kind == "elastic":
            assert a.status == 0
            assert rel(a.u, b.u) <= 1e-8, (a.rid, rel(a.u, b.u))
        else:
            assert np.abs(a.d - b.d).max() <= 1e-6
            assert rel(a.u, b.u) <= 1e-6


def test_result_same_alone_and_in_the_mix():
    from easyfea_gb300 import serving

    cache = serving.MeshCache()
    t, reqs, _ = small_stream(n=12, seed=9)
    reqs = [r for r in reqs if r.kind == "elastic"]
    with serving.Server(workers=6, precision="mixed", cache=cache) as srv:
        mixed = serving.run_stream(srv, np.zeros(len(reqs)), reqs)
    for r, m in zip(reqs, mixed):
        with serving.Server(workers=1, precision="mixed", cache=cache) as srv:
            srv.submit(r)
            srv.drain()
            alone = srv.results[r.rid]
        assert alone.status == 0 and m.status == 0
        # same operator, same solver, same stopping test: only the order of
        # floating-point atomics in the coarse restriction differs
        assert rel(m.u, alone.u) <= 1e-8


def test_batched_random_material_instances():
    """Random-material cantilevers (per-element E) through the service in
    largest-first order, against single FP64 solves."""
    from easyfea_gb300 import serving
    from easyfea_gb300.batching import random_material_cantilevers

    inst = random_material_cantilevers(n=8, seed=1, dof_min=500, dof_max=20000)
    cache = serving.MeshCache()
    reqs = []
    for i, (m, E) in enumerate(inst):
        spec = serving.MeshSpec("quad4", *_nx_ny(m))
        reqs.append(serving.ElasticRequest(spec, E=E, rid=i))
    order = sorted(reqs, key=lambda r: -r.spec.dof)
    with serving.Server(workers=4, precision="mixed", cache=cache) as srv:
        for r in order:
            srv.submit(r)
        srv.drain()
        res = srv.results
    plain = serving.run_plain(reqs, cache, precision="fp64")
    for r, p in zip(reqs, plain):
        assert res[r.rid].status == 0
        assert rel(res[r.rid].u, p.u) <= 1e-8


def _nx_ny(m):
    x = m.coord
    nx = len(np.unique(x[:, 0])) - 1
    ny = len(np.unique(x[:, 1])) - 1
    return nx, ny


@pytest.mark.parametrize("batch_max_dof", [40_000])
def test_batched_small_requests(batch_max_dof):
    """Small elastic requests served through the batcher (one persistent
    batched two-level PCG launch per batch, per-system convergence): every
    result against one-at-a-time FP64 solves within 1e-8, the same alone (a
    batch of one) and in the mix within 1e-8, and the large requests and
    phase-field steps still served by the workers."""
    from easyfea_gb300 import serving

    cache = serving.MeshCache()
    t, reqs, _ = small_stream(n=24, seed=13)
    with serving.Server(workers=4, precision="mixed", cache=cache, batch_max_dof=batch_max_dof,
                        batch_window_s=0.005) as srv:
        served = serving.run_stream(srv, np.zeros(len(reqs)), reqs)
        assert srv.batcher.batches >= 1
    assert all(r.error is None for r in served), [r.error for r in served if r.error]
    n_small = sum(1 for r in reqs if r.kind == "elastic" and r.spec.dof <= batch_max_dof)
    assert n_small >= 4
    t2, reqs2, _ = small_stream(n=24, seed=13)
    plain = serving.run_plain(reqs2, cache, precision="fp64")
    for r, a, b in zip(reqs, served, plain):
        if a.kind == "elastic":
            assert a.status == 0
            assert rel(a.u, b.u) <= 1e-8, (a.rid, a.dof, rel(a.u, b.u))
    for r, m in zip(reqs, served):
        if r.kind != "elastic" or r.spec.dof > batch_max_dof:
            continue
        with serving.Server(workers=1, precision="mixed", cache=cache, batch_max_dof=batch_max_dof) as srv:
            srv.submit(r)
            srv.drain()
            alone = srv.results[r.rid]
        assert alone.status == 0
        assert rel(m.u, alone.u) <= 1e-8, (r.rid, rel(m.u, alone.u))
