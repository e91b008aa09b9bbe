"""Replica bookkeeping across ranks, on CPU with two gloo processes.

The multiply path has no exchange step, so N GPUs run N independent replicas.
What crosses ranks is host-side: the share of units each rank takes, the
barrier around the timed region and the max over ranks of the step time (the
job's time for weak scaling). This covers that logic without a GPU.
"""
import json
import os
import socket

import pytest
import torch.multiprocessing as mp

from cuyashe_gb300 import replicas


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, out_dir):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank)})
    rep = replicas.from_env("gloo")
    units = list(range(1001))  # e.g. ciphertext pairs of one submission
    mine = replicas.shard_items(units, rep)
    replicas.barrier(rep)
    slowest = replicas.max_over_ranks(rep, 10.0 + rank)  # per-rank step time in ms
    total = replicas.sum_over_ranks(rep, len(mine))
    with open(os.path.join(out_dir, "rank%d.json" % rank), "w") as f:
        json.dump({"mine": mine, "slowest": slowest, "total": total, "root": rep.is_root}, f)
    replicas.close(rep)


@pytest.mark.parametrize("world", [2])
def test_two_gloo_ranks_shard_and_reduce(tmp_path, world):
    mp.start_processes(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True,
                       start_method="spawn")
    res = [json.load(open(tmp_path / ("rank%d.json" % r))) for r in range(world)]
    assert sorted(sum((r["mine"] for r in res), [])) == list(range(1001))
    assert all(r["slowest"] == 10.0 + world - 1 for r in res)
    assert all(r["total"] == 1001 for r in res)
    assert [r["root"] for r in res] == [True] + [False] * (world - 1)


def test_shard_is_a_partition():
    for total in (0, 1, 7, 64, 4096, 4097):
        for world in (1, 2, 3, 8):
            spans = [replicas.shard(total, r, world) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == total
            assert all(spans[i][1] == spans[i + 1][0] for i in range(world - 1))
            sizes = [b - a for a, b in spans]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        replicas.shard(10, 2, 2)


def test_single_process_needs_no_group(monkeypatch):
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    rep = replicas.from_env("gloo")
    assert rep.world == 1 and rep.group is None and rep.is_root
    assert replicas.max_over_ranks(rep, 3.5) == 3.5
    replicas.close(rep)


def test_bench_gpus_2_launches_two_ranks_on_cpu():
    """`bench.py --gpus 2` outside a launcher starts two ranks itself
    (torch.distributed.run); with --cpu-dry-run they use gloo and no CUDA, and
    rank 0 prints one line for the whole job with n_gpus = 2 and both shares."""
    import subprocess
    import sys

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = {k: v for k, v in os.environ.items() if k not in ("WORLD_SIZE", "RANK", "LOCAL_RANK", "MASTER_PORT")}
    proc = subprocess.run([sys.executable, "bench.py", "--gpus", "2", "--cpu-dry-run", "--steps", "3",
                           "--warmup", "3", "--batch", "1000"], cwd=root, env=env, capture_output=True, text=True,
                          timeout=300)
    assert proc.returncode == 0, proc.stderr[-3000:]
    lines = [l for l in proc.stdout.splitlines() if l.strip().startswith("{")]
    assert len(lines) == 1, proc.stdout
    d = json.loads(lines[0])
    assert d["n_gpus"] == 2 and d["dry_run"] is True
    assert d["shards"] == [[0, 1000], [1000, 2000]] and d["pairs_per_step"] == 2000
