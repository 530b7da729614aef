"""The multi-process path of bench.py on the CPU (gloo, world size 2): a J
build does not shard, so `bench.py --gpus N` runs one replica per rank. Rank
0 builds the representation and caches it, the other ranks wait at the
barrier and load it; every rank times its own builds, the job time is the
maximum over ranks, and the value counts the builds of all ranks."""
import json
import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, ws, port, cache, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws))
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    import bench
    import h2eri_gb300 as hg
    from h2eri_gb300 import molecules
    bench.CACHE_DIR = cache
    bench.WORKLOAD = dict(bench.WORKLOADS["c10"], molecule="C2H6", n_carbon=2)
    h, setup_s = bench.representation(hg, molecules, rank, ws, dist.barrier)
    ms = bench.max_over_ranks(10.0 + 5.0 * rank, dist, "cpu")
    value = bench.replica_value(ws, 5, ms)
    with open(os.path.join(out, f"rank{rank}.json"), "w") as f:
        json.dump({"num_bf": h.num_bf, "krnl": h.krnl_mat_size, "built": setup_s is not None,
                   "ms": ms, "value": value}, f)
    h.destroy()
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_share_the_cached_representation(tmp_path):
    import torch.multiprocessing as mp
    cache, out = tmp_path / "cache", tmp_path / "out"
    cache.mkdir()
    out.mkdir()
    mp.start_processes(_worker, args=(2, _free_port(), str(cache), str(out)), nprocs=2, start_method="spawn")
    r = [json.load(open(out / f"rank{i}.json")) for i in range(2)]
    assert r[0]["built"] and not r[1]["built"]          # rank 0 built it, rank 1 loaded the cache
    assert r[0]["num_bf"] == r[1]["num_bf"] > 0
    assert r[0]["krnl"] == r[1]["krnl"] > 0
    assert r[0]["ms"] == r[1]["ms"] == 15.0              # the slowest rank's time on every rank
    assert r[0]["value"] == pytest.approx(2 * 5 / 0.015)  # builds of both ranks over that time


def test_single_process_helpers():
    import bench
    assert bench.max_over_ranks(3.5, None, "cpu") == 3.5
    assert bench.replica_value(1, 10, 5.0) == pytest.approx(2000.0)
