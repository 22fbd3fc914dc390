"""Multi-GPU host logic (replicas only: no exchange on the geometry path) as
two CPU ranks over gloo: the slowest rank's time, the whole-job rate, and a
rank that leaves before the collective."""
import multiprocessing as mp
import os
import socket

import pytest

pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, port, mode, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE="2",
                      LOCAL_RANK=str(rank))
    from voxplat_gb300 import replicas
    try:
        r, ws, dist = replicas.init("gloo", timeout_s=5)
        if mode == "leave" and r == 1:
            q.put((r, "left"))  # leaves without joining the collective
            return
        t = replicas.max_over_ranks(10.0 + 5.0 * r, dist)
        rate = replicas.whole_job_rate(4096, ws, t)
        replicas.finish(dist)
        q.put((r, (ws, t, rate)))
    except Exception as e:  # the surviving rank reports the failed collective
        q.put((rank, "error: %s" % type(e).__name__))


def _run(mode):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, port, mode, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = dict(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        if p.is_alive():
            p.kill()
    return out


def test_two_ranks_report_the_slowest_time_and_the_job_rate():
    out = _run("ok")
    for r in (0, 1):
        ws, t, rate = out[r]
        assert ws == 2 and t == 15.0
        assert rate == pytest.approx(2 * 4096 / 0.015)


def test_a_rank_that_leaves_fails_the_other_ranks_collective():
    out = _run("leave")
    assert out[1] == "left"
    assert isinstance(out[0], str) and out[0].startswith("error")


def test_single_process_needs_no_group():
    from voxplat_gb300 import replicas
    assert replicas.init("gloo")[:2] == (0, 1) or os.environ.get("WORLD_SIZE", "1") != "1"
    assert replicas.max_over_ranks(3.0, None) == 3.0
    assert replicas.whole_job_rate(100, 1, 1000.0) == 100.0
