"""Sharding over ranks (gloo, world size 2, CPU): the summed shards equal the
unsharded run.  The per-rank runner here is the CPU oracle on the engine's
Philox streams, standing in for one GPU per rank."""
import os
import socket
import sys
from pathlib import Path

import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parent.parent


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    sys.path.insert(0, str(ROOT))
    sys.path.insert(0, str(ROOT / "oracle"))
    import torch.distributed as dist
    import oracle_io
    from mytrim_gb300 import shard
    from mytrim_gb300 import workloads as W
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sim = W.cu_self_ion(n_primaries=61, E=3e3)

    def run(s):
        return oracle_io.run(s, seed=5, philox=True, first=s.first_primary, n=s.n_primaries)

    # the oracle indexes primaries globally: give it the whole count and a subset
    def run_subset(s):
        full = W.cu_self_ion(n_primaries=sim.n_primaries, E=3e3)
        return oracle_io.run(full, seed=5, philox=True, first=s.first_primary, n=s.n_primaries)

    tot = shard.run_sharded(run_subset, sim, rank, world, dist)
    if rank == 0:
        q.put({k: (list(v) if hasattr(v, "__len__") else v) for k, v in tot.items() if k != "records"})
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_shards_sum_to_the_whole(oracle_built):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    got = q.get(timeout=120)
    for p in ps:
        p.join(timeout=120)
        assert p.exitcode == 0
    from mytrim_gb300 import workloads as W
    whole = oracle_built.run(W.cu_self_ion(n_primaries=61, E=3e3), seed=5, philox=True)
    for k in ("primaries", "members", "collisions", "vacancies", "replacements", "interstitials", "range_n"):
        assert got[k] == whole[k], k
    for k in ("Eel", "Enuc", "sx", "sxx"):
        assert abs(got[k] - whole[k]) <= 1e-9 * max(1.0, abs(whole[k])), k
    assert list(got["hist_range"]) == whole["hist_range"]


def test_shard_ranges_partition():
    from mytrim_gb300.shard import shard_range
    for n in (0, 1, 7, 1000, 12345):
        for world in (1, 2, 3, 8):
            parts = [shard_range(n, r, world) for r in range(world)]
            assert sum(c for _, c in parts) == n
            pos = 0
            for first, c in parts:
                assert first == pos
                pos += c
