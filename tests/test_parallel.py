"""Replica parallelism on CPU: shard balance, and a world_size-2 gloo run of
the shard + all-reduce gather (the reference's MPI_ALLREDUCE of disjoint
entries) with a stand-in solver, so no GPU is needed."""
import os
import socket

import numpy as np
import pytest

from phinfortran_gb300.parallel import shard_indices, shard_points


def test_shard_points_cover_and_balance():
    for npts in (0, 1, 7, 1024, 1025):
        for world in (1, 2, 3, 8):
            cuts = [shard_points(npts, world, r) for r in range(world)]
            assert cuts[0][0] == 0 and cuts[-1][1] == npts
            for (a, b), (c, d) in zip(cuts, cuts[1:]):
                assert b == c
            sizes = [b - a for a, b in cuts]
            assert max(sizes) - min(sizes) <= 1
    cost = np.r_[np.full(10, 10.0), np.ones(90)]       # expensive first points
    lo, hi = shard_points(100, 2, 0, cost)
    assert 0 < hi < 60


def test_strided_shards_spread_a_cost_ramp():
    """Without a cost estimate the points are dealt out strided: every point
    once, and a cost that rises along the energy grid (the decimation count
    near a band edge) is split evenly, unlike contiguous chunks."""
    for npts, world in ((0, 2), (13, 2), (1024, 8), (7, 3)):
        idx = [shard_indices(npts, world, r) for r in range(world)]
        assert np.array_equal(np.sort(np.concatenate(idx)), np.arange(npts))
    ramp = np.linspace(10.0, 40.0, 1024)                  # iterations rising along the grid
    strided = [ramp[shard_indices(1024, 8, r)].sum() for r in range(8)]
    chunks = [ramp[slice(*shard_points(1024, 8, r))].sum() for r in range(8)]
    assert max(strided) / min(strided) < 1.02
    assert max(chunks) / min(chunks) > 2.0
    assert np.array_equal(shard_indices(100, 2, 0, np.ones(100)), np.arange(50))


def fake_solve(E, blocks, qidx=None, zero_flag=None, scale=1.0):
    T = scale * np.asarray(E) ** 2 + (0 if qidx is None else np.asarray(qidx))
    if zero_flag is not None:
        T = np.where(np.asarray(zero_flag) != 0, 0.0, T)
    return dict(transl=T, status=np.zeros(T.size, np.int32))


def _worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from phinfortran_gb300.parallel import transport_tdb_replicas
    E = np.linspace(0.1, 3.0, 13)
    q = np.arange(13) % 3
    zf = (np.arange(13) == 0).astype(np.int32)
    r = transport_tdb_replicas(E, None, solve=fake_solve, qidx=q, zero_flag=zf, scale=2.0)
    np.save(os.path.join(out, f"r{rank}.npy"), r["transl"])
    np.save(os.path.join(out, f"s{rank}.npy"), np.array(r["shard"]))
    dist.destroy_process_group()


def test_two_rank_gather(tmp_path):
    torch_mp = pytest.importorskip("torch.multiprocessing")
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    torch_mp.spawn(_worker, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    E = np.linspace(0.1, 3.0, 13)
    want = fake_solve(E, None, qidx=np.arange(13) % 3, zero_flag=(np.arange(13) == 0).astype(np.int32),
                      scale=2.0)["transl"]
    for rank in (0, 1):
        np.testing.assert_array_equal(np.load(tmp_path / f"r{rank}.npy"), want)
    s0, s1 = np.load(tmp_path / "s0.npy"), np.load(tmp_path / "s1.npy")
    assert np.array_equal(s0, np.arange(0, 13, 2)) and np.array_equal(s1, np.arange(1, 13, 2))
