"""Host-side logic: argument validation, operand generation, and the replica
sharding of the multi-GPU bench (gloo ranks on CPU)."""
import os

import numpy as np
import pytest

import nttanafis_gb300 as ntt
from nttanafis_gb300.operands import from_int, operand, sparse_operand, to_int


def test_operand_is_splitmix64():
    # first outputs of SplitMix64 from seed 0 (Steele et al. 2014 test vector)
    v = operand(3, 0)
    assert [hex(int(x)) for x in v] == ["0xe220a8397b1dcdaf", "0x6e789e6aa1b965f4", "0x6c45d188009454f"]


def test_int_round_trip():
    x = operand(10, 5)
    assert np.array_equal(from_int(to_int(x), 10), x)


def test_sparse_operand_density():
    s = sparse_operand(100000)
    frac = np.count_nonzero(s) / s.size
    assert 0.005 < frac < 0.02


def test_host_arrays_are_validated():
    ws = object.__new__(ntt.GpuMulWorkspace)  # no device needed for argument checks
    ws._lib, ws._ws = ntt.library(), None
    with pytest.raises(TypeError):
        ws.mul(np.zeros(4, dtype=np.int64), np.zeros(2, dtype=np.uint64), np.zeros(2, dtype=np.uint64))
    with pytest.raises(TypeError):
        ws.mul(np.zeros(4, dtype=np.uint64), np.zeros((2, 1), dtype=np.uint64), np.zeros(2, dtype=np.uint64))


def _replica_worker(rank, world, port, q):
    import torch
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    units = list(bench.shard_units(10, rank, world))
    t = bench.max_over_ranks(float(rank + 1), world, torch.device("cpu"))
    gathered = [None] * world
    dist.all_gather_object(gathered, units)
    dist.destroy_process_group()
    q.put((rank, t, gathered))


def test_replica_sharding_with_gloo_ranks():
    import multiprocessing as mp
    import socket

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_replica_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    results = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, t, gathered in results:
        assert t == 2.0  # max over ranks
        flat = sorted(u for part in gathered for u in part)
        assert flat == list(range(10))  # every unit exactly once, no overlap
