"""The multi-GPU path of bench.py is replicas: every rank solves its own copy
and the ranks only meet at the timing barrier and the max-over-ranks
reduction.  That host logic runs here as two gloo ranks on the CPU."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    d = bench.Dist(use_cuda=False)
    d.barrier()
    got = d.max(float(10 * (rank + 1)))        # per-rank elapsed times -> the job's time
    d.barrier()
    d.close()
    q.put((rank, d.rank, d.world, got))


def test_two_replicas_barrier_and_max():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
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
    assert [o[1] for o in out] == [0, 1] and all(o[2] == 2 for o in out)
    assert all(o[3] == 20.0 for o in out)     # both ranks see the slower rank's time


def test_reference_arm_other_ranks_exit_quietly(monkeypatch, capsys):
    """Under torchrun only rank 0 of the reference arm works and prints."""
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setattr(sys, "argv", ["bench.py", "--impl", "reference", "--gpus", "2"])
    assert bench.main() == 0
    assert capsys.readouterr().out == ""
