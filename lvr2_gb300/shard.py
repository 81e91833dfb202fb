"""Spatial sharding of one point cloud over ranks, with halo exchange.

lvr2 distributes large reconstructions as chunks over MPI workers
(LargeScaleReconstruction.tcc:915-1347); here a cloud is split into Morton
ranges, one per rank, and each rank computes the normals of its own points
exactly as one process would over the whole cloud:

1. partition: the points sorted by 63-bit Morton code (21 bits per axis over
   the cloud's bounding cube) and cut into `world` contiguous ranges;
2. bound: each rank's k-th-neighbour distance over its own points only is an
   upper bound of the true one (fewer candidates can only be farther);
3. halo: each rank's box, widened per point by that bound, goes to every
   rank (all_gather); every rank sends the points of its range that fall in
   another rank's widened box (point-to-point, sizes first);
4. the owned + halo points, ordered by global index (so that ties of the
   (d2, index) order break as in the whole cloud), give exact kNN, normals
   and adaptive-k rounds for the owned points;
5. a second exchange sends the raw normals of the halo points, so the ki
   interpolation of owned points is exact too.

The per-rank compute steps are callables, so the same logic runs over the
GPU surface (torch.distributed with NCCL or gloo) or over any other
implementation of the same operations.
"""
import numpy as np


def morton63(points, lo, scale):
    """63-bit Morton codes of float32 points in the frame (p - lo) * scale."""
    c = np.clip(((points.astype(np.float32) - lo) * scale), 0, 2 ** 21 - 1).astype(np.uint64)
    out = np.zeros(len(points), np.uint64)
    for b in range(21):
        for a in range(3):
            out |= ((c[:, a] >> np.uint64(b)) & np.uint64(1)) << np.uint64(3 * b + a)
    return out


def morton_partition(points, world):
    """Global indices of the points of each rank: contiguous Morton ranges of
    equal size (the last takes the remainder)."""
    p = np.asarray(points, np.float32)
    if len(p) == 0:
        return [np.zeros(0, np.int64) for _ in range(world)]
    lo = p.min(0)
    ext = float((p.max(0) - lo).max())
    scale = np.float32(2 ** 21 / ext) if ext > 0 else np.float32(0)
    order = np.argsort(morton63(p, lo, scale), kind="stable")
    bounds = [len(p) * r // world for r in range(world + 1)]
    return [np.sort(order[bounds[r]:bounds[r + 1]]).astype(np.int64) for r in range(world)]


def widened_box(points, radius):
    """Box of the points, each widened by its own radius (6 floats); a
    relative margin of 1e-5 covers the float32 rounding of the distances."""
    if len(points) == 0:
        return np.array([np.inf] * 3 + [-np.inf] * 3, np.float64)
    p = np.asarray(points, np.float64)
    r = np.asarray(radius, np.float64)[:, None] * (1.0 + 1e-5) + 1e-30
    return np.concatenate([(p - r).min(0), (p + r).max(0)])


def in_box(points, box):
    p = np.asarray(points, np.float64)
    return np.all((p >= box[:3]) & (p <= box[3:]), axis=1)


def _exchange(send, dtype, width, group=None):
    """send[r]: array (m_r, width) for rank r (own entry ignored); returns the
    arrays received from every other rank, by rank."""
    import torch
    import torch.distributed as dist
    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    counts = torch.tensor([len(a) if r != rank else 0 for r, a in enumerate(send)], dtype=torch.int64)
    table = [torch.zeros_like(counts) for _ in range(world)]
    dist.all_gather(table, counts, group=group)
    reqs, recv = [], {}
    for r in range(world):
        if r == rank:
            continue
        buf = torch.empty((int(table[r][rank]), width), dtype=dtype)
        recv[r] = buf
        if buf.numel():
            reqs.append(dist.irecv(buf, src=r, group=group))
        out = torch.from_numpy(np.ascontiguousarray(send[r]).reshape(-1, width)).to(dtype)
        if out.numel():
            reqs.append(dist.isend(out, dst=r, group=group))
    for q in reqs:
        q.wait()
    return {r: b.numpy() for r, b in recv.items()}


def halo_exchange(points, ids, kth_dist, group=None):
    """Owned points (float32 (m, 3)) with their global ids and local k-th
    neighbour distances -> (points, ids) of owned + halo points, sorted by
    global id, and the mask of owned entries."""
    import torch
    import torch.distributed as dist
    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    box = torch.from_numpy(widened_box(points, kth_dist))
    boxes = [torch.zeros_like(box) for _ in range(world)]
    dist.all_gather(boxes, box, group=group)
    sel = [in_box(points, boxes[r].numpy()) if r != rank else np.zeros(len(points), bool) for r in range(world)]
    got_p = _exchange([np.asarray(points, np.float32)[m] for m in sel], torch.float32, 3, group)
    got_i = _exchange([np.asarray(ids, np.int64)[m] for m in sel], torch.int64, 1, group)
    all_p = [np.asarray(points, np.float32)] + [got_p[r] for r in sorted(got_p)]
    all_i = [np.asarray(ids, np.int64)] + [got_i[r].reshape(-1) for r in sorted(got_i)]
    P = np.concatenate(all_p)
    I = np.concatenate(all_i)
    order = np.argsort(I, kind="stable")
    owned = np.zeros(len(I), bool)
    owned[:len(ids)] = True
    return P[order], I[order], owned[order]


def share_halo_values(ids, values, owned, group=None):
    """values: per entry of the local (owned + halo) arrays, sorted by global
    id, valid for the owned entries; returns them with the halo entries set
    to their owners' values."""
    import torch
    import torch.distributed as dist
    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    values = np.array(values, np.float32, copy=True)
    width = values.shape[1]
    need = ids[~owned]
    empty_i = np.zeros(0, np.int64)
    wanted = _exchange([need if r != rank else empty_i for r in range(world)], torch.int64, 1, group)
    own_ids = ids[owned]
    own_vals = values[owned]
    send_ids, send_vals = [], []
    for r in range(world):
        if r == rank:
            send_ids.append(empty_i)
            send_vals.append(np.zeros((0, width), np.float32))
            continue
        w = wanted[r].reshape(-1)
        hit = w[np.isin(w, own_ids)]
        send_ids.append(hit)
        send_vals.append(own_vals[np.searchsorted(own_ids, hit)])
    got_ids = _exchange(send_ids, torch.int64, 1, group)
    got_vals = _exchange(send_vals, torch.float32, width, group)
    for r in got_ids:
        values[np.searchsorted(ids, got_ids[r].reshape(-1))] = got_vals[r]
    return values


def sharded_normals(points, ids, kn=10, ki=10, nem=3, flip_point=(0.0, 0.0, 0.0), adaptive=True, group=None,
                    device=0):
    """Normals of this rank's points (float32 (m, 3), global ids `ids`,
    ascending) on the GPU, equal to those of one surface over the whole
    cloud: returns (normals after interpolation, raw normals, k used), rows
    in `ids` order.  Needs an initialised torch.distributed process group."""
    from .surface import Surface
    own = np.ascontiguousarray(points, np.float32)
    k_halo = (32 if adaptive else 2) * kn  # the largest k a normal search uses
    k_halo = max(k_halo, ki)
    if len(own) >= k_halo:
        with Surface(own, kn=kn, ki=0, nem=nem, flip_point=flip_point, adaptive=adaptive, device=device) as s:
            _, d, _ = s.knn(own, k_halo)
        kth = d[:, -1]
    else:
        kth = np.full(len(own), np.inf, np.float32)
    P, I, owned = halo_exchange(own, np.asarray(ids, np.int64), kth, group)
    with Surface(P, kn=kn, ki=0, nem=nem, flip_point=flip_point, adaptive=adaptive, device=device) as s:
        s.calculate_normals()
        raw, k = s.raw_normals()
        raw = share_halo_values(I, raw, owned, group)
        final = raw
        if ki > 0:
            s.set_k(ki=ki)
            s.set_normals(raw)
            s.interpolate_normals()
            final = s.normals()
    return final[owned], raw[owned], k[owned]
