"""Batch sharding across ranks (host logic, CPU): the partition of the cloud
list and the gather to rank 0, with world size 2 over gloo.  The CPU oracle
stands in for the per-rank GPU solve, so the test checks the plumbing: every
cloud's result arrives at rank 0, in order, equal to a one-rank run."""
import os
import socket

import numpy as np
import pytest

import emst_shard as S


def test_partition_covers_and_balances():
    rng = np.random.default_rng(1)
    sizes = rng.integers(0, 1000, 97)
    for world in (1, 2, 3, 8, 200):
        parts = S.partition(sizes, world)
        assert len(parts) == world and parts[0][0] == 0 and parts[-1][1] == len(sizes)
        assert all(a <= b for a, b in parts) and all(parts[r][1] == parts[r + 1][0] for r in range(world - 1))
        if world <= 8:
            loads = [int(sizes[a:b].sum()) for a, b in parts]
            assert max(loads) - min(loads) <= 2 * int(sizes.max()) + 1


def _clouds():
    from families import family
    rng = np.random.default_rng(2)
    out = []
    for i in range(11):
        n = int(rng.choice([0, 1, 2, 40, 150, 400]))
        dim = int(rng.choice([2, 3]))
        out.append(family("uniform", n, dim, 10 + i) if n else np.zeros((0, dim), np.float32))
    return out


def _oracle_solve(clouds):
    import pyoracle as O
    uvs, lens = [], []
    for c in clouds:
        if len(c) < 2:
            uvs.append(np.zeros((0, 2), np.int32))
            lens.append(0.0)
            continue
        sp, _, _, _ = O.rescale(c)
        r = O.emst(sp, "exact")
        uvs.append(np.sort(np.asarray(r.edges, np.int32).reshape(-1, 2), axis=1))
        lens.append(float(len(r.edges)))
    return uvs, np.asarray(lens)


def _worker(rank, world, port, q):
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    for p in (here, os.path.join(here, "..", "oracle"),
              os.path.join(here, "..", "component-based-2d-3d-nns-to-gpu-parallel-2d-3d-emst_gb300")):
        sys.path.insert(0, p)
    import torch.distributed as dist
    import emst_shard
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    uvs, lens = emst_shard.solve_sharded(_clouds(), rank, world, _oracle_solve, dist)
    if rank == 0:
        q.put(([u.tolist() for u in uvs], lens.tolist()))
    dist.barrier()
    dist.destroy_process_group()


def test_sharded_batch_equals_one_rank():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = q.get(timeout=120)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    ref_uv, ref_len = _oracle_solve(_clouds())
    assert len(got[0]) == len(ref_uv)
    for u, r in zip(got[0], ref_uv):
        assert np.array_equal(np.asarray(u, np.int32).reshape(-1, 2), r)
    assert np.allclose(got[1], ref_len)
