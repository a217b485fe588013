"""Replica path with two ranks on CPU (gloo): each rank serves its own
request stream with no data-path collective; the measurement takes the
slowest rank's time and reports the whole job's throughput on every rank."""

import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), LOCAL_RANK=str(rank),
                      WORLD_SIZE=str(world))
    from easyfea_gb300 import replicas, serving

    replicas.init("gloo")
    offsets, reqs, _ = serving.poisson_stream(1000.0, 20, seed=3)
    served = []

    def execute(req, res):  # host stand-in for the GPU solve
        served.append(req.rid)

    with serving.Server(workers=2, hbm_budget=1 << 40, executor=execute) as srv:
        for r in reqs:
            srv.submit(r)
        srv.drain(timeout=30)
    replicas.barrier()
    value, t = replicas.job_throughput(len(reqs), 0.1 * (rank + 1))
    q.put((rank, sorted(served), value, t))
    replicas.finish()


@pytest.mark.timeout(120)
def test_two_replicas_throughput():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=90) for _ in procs]
    for p in procs:
        p.join(timeout=30)
        assert p.exitcode == 0
    out.sort()
    for rank, served, value, t in out:
        assert served == list(range(20))  # each replica served its whole stream
        assert t == pytest.approx(0.2)  # the slowest rank's time
        assert value == pytest.approx(2 * 20 / 0.2)


def test_single_process_is_its_own_job():
    from easyfea_gb300 import replicas

    value, t = replicas.job_throughput(30, 0.5)
    assert (value, t) == (60.0, 0.5)
