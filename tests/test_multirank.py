"""The N>1 path of bench.py on CPU: two gloo ranks (replicas, reads sharded by
rank, no data-path collective) -- disjoint seeded shards, max/sum reductions of
the timing scalars, and the reference arm's non-zero ranks exiting without work."""
from __future__ import annotations

import hashlib
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out_dir: str) -> None:
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, str(ROOT))
    sys.path.insert(0, str(ROOT / "hpg-libs_gb300"))
    import bench
    from hpgbwt import synth
    d = bench.Dist(world, backend="gloo")
    assert (d.rank, d.world) == (rank, world)
    g = synth.genome("repeats", 200_000, 1)  # every rank builds the same genome (same seed)
    reads = synth.reads_fast(g, 2000, bench.read_seed(rank), 100, "per_base_capped")
    shard = hashlib.sha256(reads.seq.tobytes()).hexdigest()
    import torch.distributed as dist
    shards = [None] * world
    dist.all_gather_object(shards, shard)
    genomes = [None] * world
    dist.all_gather_object(genomes, hashlib.sha256(g.tobytes()).hexdigest())
    d.barrier()
    t = 1.5 + 2.5 * rank
    res = {"max": d.max(t), "sum": d.sum(float(len(reads))), "shards": shards, "genomes": genomes}
    d.close()
    Path(out_dir, f"rank{rank}.txt").write_text(repr(res))


def test_two_gloo_ranks(tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    port = _free_port()
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, start_method="spawn", join=True)
    res = [eval((tmp_path / f"rank{r}.txt").read_text()) for r in range(2)]
    for r in res:
        assert r["max"] == 4.0 and r["sum"] == 4000.0
        assert r["shards"][0] != r["shards"][1]      # each rank maps its own reads
        assert r["genomes"][0] == r["genomes"][1]    # against the same index
    assert res[0]["shards"] == res[1]["shards"]


def test_reference_arm_other_ranks_exit_quietly():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1", MASTER_ADDR="127.0.0.1")
    p = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--gpus", "2"],
                       capture_output=True, text=True, env=env, timeout=120)
    assert p.returncode == 0 and p.stdout.strip() == ""
