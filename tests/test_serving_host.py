"""Host logic of the solve service: admission by HBM footprint, bypass limit,
request streams (no GPU: the executor is a stand-in that sleeps)."""

import threading
import time

import numpy as np
import pytest

from easyfea_gb300 import serving


class FakeReq:
    kind = "elastic"

    def __init__(self, rid, fp, dur):
        self.rid = rid
        self.fp = fp
        self.dur = dur
        self.spec = serving.MeshSpec("quad4", 4, 2)
        self.keep_solution = False

    def footprint(self, precision):
        return self.fp


def make_server(budget, workers, log):
    lock = threading.Lock()
    running = {"fp": 0, "n": 0}

    def execute(req, res):
        with lock:
            running["fp"] += req.fp
            running["n"] += 1
            log.append((running["fp"], running["n"]))
        time.sleep(req.dur)
        with lock:
            running["fp"] -= req.fp
            running["n"] -= 1

    return serving.Server(workers=workers, hbm_budget=budget, executor=execute, max_bypass=3)


def test_admission_respects_budget_and_workers():
    log = []
    rng = np.random.default_rng(0)
    reqs = [FakeReq(i, int(rng.integers(1, 60)), float(rng.uniform(0.001, 0.01))) for i in range(60)]
    with make_server(100, 4, log) as srv:
        for r in reqs:
            srv.submit(r)
        assert srv.drain(timeout=30)
        assert all(srv.results[r.rid].error is None for r in reqs)
        assert len(srv.results) == len(reqs)
        assert srv.peak_in_use <= 100
    assert max(fp for fp, _ in log) <= 100
    assert max(n for _, n in log) <= 4


def test_requests_run_concurrently():
    log = []
    reqs = [FakeReq(i, 1, 0.05) for i in range(8)]
    with make_server(100, 8, log) as srv:
        t0 = time.perf_counter()
        for r in reqs:
            srv.submit(r)
        srv.drain(timeout=30)
        dt = time.perf_counter() - t0
    assert dt < 0.3, dt  # 8 x 50 ms sequentially would be 0.4 s
    assert max(n for _, n in log) >= 4


def test_large_request_is_not_starved():
    """A request that needs the whole budget runs after at most max_bypass
    smaller ones have passed it."""
    log = []
    with make_server(100, 4, log) as srv:
        srv.submit(FakeReq(0, 60, 0.05))  # occupies 60
        time.sleep(0.01)
        srv.submit(FakeReq(1, 100, 0.01))  # must wait for the whole budget
        for i in range(2, 40):
            srv.submit(FakeReq(i, 10, 0.02))
        srv.drain(timeout=30)
        order = sorted(srv.results.values(), key=lambda r: r.start)
        pos = [r.rid for r in order].index(1)
    assert pos <= 1 + 3 + 4, pos  # started after at most max_bypass admissions (+ those already running)


def test_request_over_budget_is_refused():
    with make_server(100, 2, []) as srv:
        with pytest.raises(ValueError):
            srv.submit(FakeReq(0, 101, 0.0))


def test_failed_request_is_reported_and_server_continues():
    def execute(req, res):
        if req.rid == 1:
            raise RuntimeError("boom")

    with serving.Server(workers=2, hbm_budget=100, executor=execute) as srv:
        for i in range(4):
            srv.submit(FakeReq(i, 1, 0.0))
        srv.drain(timeout=10)
        assert srv.results[1].error is not None and "boom" in srv.results[1].error
        assert all(srv.results[i].error is None for i in (0, 2, 3))


def test_poisson_stream_is_seeded_and_in_range():
    t1, r1, _ = serving.poisson_stream(100.0, 400, seed=3)
    t2, r2, _ = serving.poisson_stream(100.0, 400, seed=3)
    assert np.array_equal(t1, t2)
    assert [type(a).__name__ for a in r1] == [type(b).__name__ for b in r2]
    gaps = np.diff(t1)
    assert abs(gaps.mean() - 0.01) < 0.002
    for r in r1:
        if r.kind == "elastic":
            lo, hi = (1e3, 5e5) if r.spec.kind != "hexa8" else (1e4, 2e6)
            assert 0.5 * lo <= r.spec.dof <= 1.5 * hi, (r.spec, r.spec.dof)
        else:
            assert 0.5 * 20000 <= r.spec.n_elems <= 1.5 * 320000


@pytest.mark.parametrize("spec", [serving.MeshSpec("quad4", 12, 3), serving.MeshSpec("quad9", 6, 2),
                                  serving.MeshSpec("hexa8", 6, 2, 3), serving.MeshSpec("tri3_sen", 4, 4)])
def test_mesh_spec_counts(spec):
    m = spec.build()
    assert m.Nn == spec.n_nodes
    assert m.Ne == spec.n_elems
