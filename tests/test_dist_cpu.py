"""The replicas-only multi-GPU path of bench.py on the CPU: two gloo ranks
take the barrier and the max over ranks the timing uses (no GPU, no
collective in the data path)."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _rank(rank, ws, port, q):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "WORLD_SIZE": str(ws),
                       "RANK": str(rank), "LOCAL_RANK": str(rank)})
    import bench
    D = bench.Dist(ws)
    D.barrier()
    got = D.max(10.0 + rank)       # per-rank step time: the job takes the slowest
    ws_, rank_, local_ = bench.dist_info()
    D.close()
    q.put((rank, got, ws_, rank_, local_))


def test_two_gloo_ranks_barrier_and_max():
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.SimpleQueue()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    out = sorted(q.get() for _ in range(2))
    assert [o[1] for o in out] == [11.0, 11.0]
    assert [(o[2], o[3], o[4]) for o in out] == [(2, 0, 0), (2, 1, 1)]


def test_gpus_flag_must_match_world_size(monkeypatch):
    import bench
    monkeypatch.setenv("WORLD_SIZE", "1")
    with pytest.raises(SystemExit):
        bench.main(["--gpus", "2"])
