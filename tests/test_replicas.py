"""The N>1 benchmark path (one replica per GPU, no collective on the data
path): two gloo ranks on CPU check the barrier, the slowest-rank time and the
whole-job throughput."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import time

    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank)})
    from heavyrt_gb300 import replicas

    r = replicas.from_env()
    assert (r.rank, r.world, r.local) == (rank, world, rank)
    replicas.init(r, "gloo")
    local_ms = [3.0, 5.5][rank]  # rank 1 is the slow replica
    if rank == 1:
        time.sleep(0.3)  # arrives late: the barrier must hold rank 0
    t0 = time.perf_counter()
    replicas.barrier(r)
    waited = time.perf_counter() - t0
    ms = replicas.max_over_ranks(r, local_ms)
    value = replicas.job_throughput(r, 1000.0, ms)
    with open(os.path.join(out_dir, f"rank{rank}.txt"), "w") as f:
        f.write(f"{ms} {value} {waited}\n")
    replicas.finish(r)


def test_two_gloo_replicas(tmp_path):
    pytest.importorskip("torch")
    import torch.multiprocessing as mp

    mp.start_processes(_rank_main, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    rows = [list(map(float, (tmp_path / f"rank{k}.txt").read_text().split())) for k in range(2)]
    for ms, value, _ in rows:
        assert ms == 5.5  # every rank sees the slowest replica's time
        assert value == pytest.approx(2 * 1000.0 / 5.5e-3)  # both replicas' work over the slowest time
    assert rows[0][2] > 0.1  # rank 0 waited at the barrier for the late rank


def test_single_process_defaults(monkeypatch):
    from heavyrt_gb300 import replicas

    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    r = replicas.from_env()
    assert (r.rank, r.world, r.local, r.leader) == (0, 1, 0, True)
    replicas.init(r)  # no process group for one rank
    replicas.barrier(r)
    assert replicas.max_over_ranks(r, 4.25) == 4.25
    assert replicas.job_throughput(r, 500.0, 2.0) == pytest.approx(250000.0)
