"""The N > 1 path of bench.py on the CPU: two ranks on the gloo backend
(127.0.0.1), the barrier and the max over ranks that the timed region uses,
the whole-job value (all ranks' simulated days over the slowest rank's
time), and the reference arm's rank rule (rank 0 alone runs and prints)."""
import multiprocessing as mp
import os
import socket

from conftest import ROOT


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import sys

    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench

    r, w, local = bench.dist_env()
    d = bench.Dist(w)
    d.barrier()
    slowest = d.max(10.0 + 5.0 * r)  # rank r "took" 10 + 5 r ms
    d.barrier()
    d.close()
    q.put((r, w, local, slowest))


def test_two_ranks_gloo_barrier_and_max():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert out == [(0, 2, 0, 15.0), (1, 2, 1, 15.0)]


def test_whole_job_value_and_reference_rank_rule(capsys):
    import bench

    # 2 ranks x 40 steps of 45 s in 73 ms (the slowest rank): 3600 simulated s
    v = bench.job_value(2, 40, 45.0, 73.0)
    assert abs(v - 2 * 40 * 45.0 / 86400.0 / 0.073) < 1e-12
    assert bench.job_value(1, 40, 45.0, 73.0) * 2 == v

    class Args:
        pass

    # rank 1 of 2 leaves the reference arm at once, without work or output
    assert bench.run_reference(Args(), 1, 2) is None
    assert capsys.readouterr().out == ""
