"""The multi-rank timing of bench.py --gpus N (replicas: one process per GPU,
no collective on the data path) on CPU ranks with the gloo backend: barrier
and synchronisation around the timed region, the time of the slowest rank,
and the whole-job rate."""
import multiprocessing as mp
import os
import socket
import time

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, q):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    from hyperdeal_gb300.replicas import Replicas, time_steps, whole_job_rate
    rep = Replicas("gloo")
    calls = {"n": 0}

    def step():
        calls["n"] += 1
        time.sleep(0.02 * (rank + 1))  # rank 1 is the slow one

    ms = time_steps(rep, step, steps=4, warmup=2, sync=lambda: None)
    rate = whole_job_rate(1000.0, rep.world, ms)
    q.put((rank, ms, rate, calls["n"], rep.world))
    rep.close()


def test_two_gloo_ranks_report_the_slowest():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    out.sort()
    (r0, ms0, rate0, n0, w0), (r1, ms1, rate1, n1, w1) = out
    assert w0 == w1 == 2 and n0 == n1 == 6
    # both ranks report the maximum over ranks: the slow rank's ~40 ms per step
    assert ms0 == ms1
    assert 38.0 <= ms0 <= 80.0
    assert rate0 == pytest.approx(1000.0 * 2 / (ms0 / 1e3))


def test_single_process_needs_no_process_group():
    from hyperdeal_gb300.replicas import Replicas, time_steps
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        os.environ.pop(k, None)
    rep = Replicas("gloo")
    assert rep.world == 1 and rep.dist is None
    ms = time_steps(rep, lambda: time.sleep(0.005), steps=3, warmup=1, sync=lambda: None)
    assert 4.0 <= ms <= 50.0
