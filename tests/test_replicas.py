"""The multi-GPU replica logic of bench.py (scalar reductions and barriers
only), run as two gloo ranks on the CPU."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    from research_codes_gb300 import replicas
    assert replicas.init("gloo") == world
    replicas.barrier()
    # rank r processed 100 (r + 1) units per step in 10 (r + 1) ms over 5 steps
    rate, worst = replicas.aggregate_rate(100.0 * (rank + 1), 10.0 * (rank + 1), 5)
    q.put((rank, rate, worst, replicas.replica_seed(7, rank)))
    replicas.finalize()


def test_replica_reductions_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    for rank, rate, worst, seed in out:
        assert worst == 20.0
        assert rate == pytest.approx((100.0 + 200.0) * 5 / 20e-3)
        assert seed == 7 + rank


def test_single_rank_defaults():
    from research_codes_gb300 import replicas
    os.environ.pop("WORLD_SIZE", None)
    assert replicas.rank_info()[0] == 1
    assert replicas.aggregate_rate(10.0, 2.0, 3) == (10.0 * 3 / 2e-3, 2.0)
