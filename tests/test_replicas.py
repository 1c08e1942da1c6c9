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


def test_partition_covers_in_order():
    from heavyrt_gb300 import replicas

    for n in (0, 1, 7, 1000, 2073600):
        for world in (1, 2, 3, 8):
            for align in (1, 16, 15360):
                shares = [replicas.partition(n, replicas.Rank(k, world, k), align) for k in range(world)]
                assert shares[0][0] == 0 and shares[-1][1] == n
                for (a0, a1), (b0, b1) in zip(shares, shares[1:]):
                    assert a1 == b0 and a0 <= a1
                for k, (a0, a1) in enumerate(shares):
                    assert (a0 % align == 0 or a0 == n) and (a1 % align == 0 or a1 == n)
                blocks = [-(-(a1 - a0) // align) for a0, a1 in shares]
                assert max(blocks) - min(blocks) <= 1


def _split_main(rank, world, port, out_dir):
    import numpy as np

    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank)})
    from heavyrt_gb300 import replicas

    r = replicas.from_env()
    replicas.init(r, "gloo")
    grp = replicas.host_group(r)
    n, width = 1003, 17
    rays = np.arange(n * 8, dtype=np.float32).reshape(n, 8)
    a0, a1 = replicas.partition(n, r, align=width)
    # a stand-in for the traced result of each ray: records derived from it
    hits = (rays[a0:a1, :4].view(np.uint32) ^ np.uint32(0x5A5A5A5A)).copy()
    flags = (np.arange(a0, a1) % 3 == 0).astype(np.uint8)
    got = replicas.gather_rows(r, hits, grp)
    got_flags = replicas.gather_rows(r, flags, grp)
    if r.leader:
        want = rays[:, :4].view(np.uint32) ^ np.uint32(0x5A5A5A5A)
        ok = np.array_equal(got, want) and np.array_equal(got_flags, (np.arange(n) % 3 == 0).astype(np.uint8))
        (open(os.path.join(out_dir, "split.txt"), "w")).write("ok" if ok else "mismatch")
    else:
        assert got is None
    replicas.finish(r)


def test_split_batch_gathers_in_order(tmp_path):
    """Three gloo ranks each take their share of one ray batch; rank 0 gets
    every rank's result rows back in ray order."""
    pytest.importorskip("torch")
    import torch.multiprocessing as mp

    mp.start_processes(_split_main, args=(3, _free_port(), str(tmp_path)), nprocs=3, join=True, start_method="spawn")
    assert (tmp_path / "split.txt").read_text() == "ok"
