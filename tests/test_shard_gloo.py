"""Data-parallel sharding of chains, exercised with world_size-2 gloo on the CPU.

Each rank takes its length-balanced shard, runs the oracle on it (the kinematics
of a chain never depends on another chain), and the gathered shards equal the
full-batch result."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from torchproteinlibrary_gb300.sharding import partition_chains


def test_partition_is_exact_and_balanced():
    rng = np.random.default_rng(0)
    lengths = rng.integers(20, 701, 1024)
    for ws in (1, 2, 3, 8):
        parts = partition_chains(lengths, ws)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(lengths)))
        loads = [int(lengths[p].sum()) for p in parts]
        assert max(loads) - min(loads) <= int(lengths.max())


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out_dir):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import oracle
    rng = np.random.default_rng(42)
    B, L = 12, 30
    ang = rng.uniform(-np.pi, np.pi, (B, 3, L))
    lengths = rng.integers(1, L + 1, B).astype(np.int32)
    mine = partition_chains(lengths, world)[rank]
    c, _ = oracle.a2b_forward(ang[mine], lengths[mine])
    full = torch.zeros(B, 9 * L, dtype=torch.float64)
    full[mine] = torch.from_numpy(c)
    dist.all_reduce(full)  # shards are disjoint: the sum is the gathered batch
    ref, _ = oracle.a2b_forward(ang, lengths)
    ok = torch.tensor([float(np.array_equal(full.numpy(), ref))])
    dist.all_reduce(ok, op=dist.ReduceOp.MIN)
    if rank == 0:
        with open(os.path.join(out_dir, "ok"), "w") as f:
            f.write(str(int(ok.item())))
    dist.barrier()
    dist.destroy_process_group()


def test_gloo_world2_shards_match_full_batch(tmp_path, oracle_lib):
    port = _free_port()
    mp.start_processes(_worker, args=(2, port, str(tmp_path)), nprocs=2, start_method="spawn")
    assert (tmp_path / "ok").read_text() == "1"
