"""Sharded normals over two CPU ranks (gloo): Morton-range partition, halo
exchange by widened boxes, halo raw-normal exchange.  Each rank's normals,
adaptive rounds and interpolated normals equal the single-process result bit
for bit.  The per-rank compute is the oracle (this test needs no GPU)."""
import os
import socket

import numpy as np
import pytest

KN, KI = 5, 10
K_MAX = 32 * KN  # the largest k lvr2's adaptive rounds can use


def cloud():
    from lvr2_gb300 import synthetic
    return synthetic.spheres_tori(24_000, seed=13)


def flip_of(P):
    return ((P.min(0) + P.max(0)) / 2).astype(np.float32)


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def rank_main(rank, world, port, out_dir):
    import torch.distributed as dist

    from lvr2_gb300 import shard
    from oracle import oracle as O
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    try:
        P = cloud()
        ids = shard.morton_partition(P, world)[rank]
        own = P[ids]
        _, d, _ = O.OracleSurface(own, threads=2).knn(own, min(K_MAX, len(own)))
        kth = d[:, -1] if len(own) >= K_MAX else np.full(len(own), np.inf, np.float32)
        Pl, Il, owned = shard.halo_exchange(own, ids, kth)
        o = O.OracleSurface(Pl, threads=2)
        raw, k = o.normals(KN, nem=3, adaptive=True, flip=flip_of(P), with_k=True)
        raw = shard.share_halo_values(Il, raw, owned)
        interp = o.interpolate(raw, KI)
        np.savez(os.path.join(out_dir, "rank%d.npz" % rank), ids=Il[owned], raw=raw[owned], k=k[owned],
                 interp=interp[owned], halo=int((~owned).sum()))
    finally:
        dist.destroy_process_group()


def test_sharded_normals_equal_single_process(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    from oracle import oracle as O
    O.build()
    world = 2
    mp.start_processes(rank_main, args=(world, free_port(), str(tmp_path)), nprocs=world, start_method="spawn")
    P = cloud()
    o = O.OracleSurface(P, threads=4)
    raw, k = o.normals(KN, nem=3, adaptive=True, flip=flip_of(P), with_k=True)
    interp = o.interpolate(raw, KI)
    seen = np.zeros(len(P), bool)
    for r in range(world):
        z = np.load(tmp_path / ("rank%d.npz" % r))
        ids = z["ids"]
        assert not seen[ids].any()
        seen[ids] = True
        assert 0 < int(z["halo"]) < len(P) // 2  # a halo, not the whole cloud
        assert np.array_equal(z["k"], k[ids])
        assert np.array_equal(z["raw"], raw[ids], equal_nan=True)
        assert np.array_equal(z["interp"], interp[ids], equal_nan=True)
    assert seen.all()


def test_partition_is_spatial():
    from lvr2_gb300 import shard
    P = cloud()
    parts = shard.morton_partition(P, 4)
    assert sorted(np.concatenate(parts).tolist()) == list(range(len(P)))
    assert max(len(p) for p in parts) - min(len(p) for p in parts) <= 1
    # Morton ranges are compact: each part's box is much smaller than the cloud's
    vol = np.prod(P.max(0) - P.min(0))
    assert all(np.prod(P[p].max(0) - P[p].min(0)) < 0.75 * vol for p in parts)


def gpu_rank_main(rank, world, port, out_dir):
    import torch.distributed as dist

    from lvr2_gb300 import shard
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    try:
        P = cloud()
        ids = shard.morton_partition(P, world)[rank]
        final, raw, k = shard.sharded_normals(P[ids], ids, kn=KN, ki=KI, nem=3, flip_point=flip_of(P))
        np.savez(os.path.join(out_dir, "gpu%d.npz" % rank), ids=ids, final=final, raw=raw, k=k)
    finally:
        dist.destroy_process_group()


@pytest.mark.gpu
def test_sharded_gpu_normals_equal_one_surface(lib, tmp_path):
    """Two ranks on one GPU (their kernels are independent; the halo goes
    through gloo on the host): sharded normals equal one surface's."""
    import torch.multiprocessing as mp

    import lvr2_gb300
    world = 2
    mp.start_processes(gpu_rank_main, args=(world, free_port(), str(tmp_path)), nprocs=world, start_method="spawn")
    P = cloud()
    with lvr2_gb300.Surface(P, kn=KN, ki=KI, nem=3, flip_point=flip_of(P)) as s:
        s.calculate_normals()
        final = s.normals()
        raw, k = s.raw_normals()
    for r in range(world):
        z = np.load(tmp_path / ("gpu%d.npz" % r))
        ids = z["ids"]
        assert np.array_equal(z["k"], k[ids])
        assert np.array_equal(z["raw"], raw[ids], equal_nan=True)
        assert np.array_equal(z["final"], final[ids], equal_nan=True)
