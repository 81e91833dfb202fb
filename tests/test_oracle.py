"""The CPU oracle against brute force, float64 PCA and its frozen outputs."""
from pathlib import Path

import numpy as np
import pytest

from tests.helpers import angle_deg, canonical_mesh, fp64_pca_normals

ROOT = Path(__file__).resolve().parent.parent
GOLD = np.load(ROOT / "tests/golden/oracle_small.npz")


def brute_knn(P, Q, k):
    d = Q[:, None, :].astype(np.float32) - P[None, :, :].astype(np.float32)
    sq = d * d
    d2 = (sq[..., 0] + sq[..., 1]) + sq[..., 2]
    idx = np.broadcast_to(np.arange(len(P)), d2.shape)
    order = np.lexsort((idx, d2), axis=1)[:, :k]
    return order.astype(np.uint32), np.sqrt(np.take_along_axis(d2, order, 1))


REF_LBVH = np.load(ROOT / "tests/golden/ref_lbvh.npz")


@pytest.mark.parametrize("name", ["sphere", "scan", "spheres_tori"])
def test_oracle_against_lvr2_lbvh_outputs(oracle_mod, name):
    """The oracle pinned to outputs of lvr2's own code: what LBVHIndex::kSearch
    and LBVHIndex::knn_normals (src/liblvr2/reconstruction/cuda/LBVHIndex.cu,
    run unmodified on a GB300 by tests/golden/make_ref_lbvh.py) returned.
    - kNN: the same neighbour set for every query; lvr2's squared distances
      (NVRTC contracts them into FMAs) within 2 ulp of the float32 ones, the
      oracle's Euclidean distances within 2 ulp of their square roots.
    - nem 4 (the comparator's FP64 plane fit): bit-equal normals."""
    g = REF_LBVH
    K = int(g["K"])
    P, Q = g[name + "_points"], g[name + "_queries"]
    ridx, rd2 = g[name + "_idx"], g[name + "_dist"]
    o = oracle_mod.OracleSurface(P)
    oi, od, oc = o.knn(Q, K)
    assert (oc == K).all() and (g[name + "_cnt"] == K).all()
    assert all(set(a) == set(b) for a, b in zip(oi.tolist(), ridx.tolist()))
    d = P[ridx.astype(np.int64)] - Q[:, None, :]
    d2 = (d[..., 0] * d[..., 0] + d[..., 1] * d[..., 1]) + d[..., 2] * d[..., 2]

    def ulps(a, b):
        a = np.asarray(a, np.float32)
        b = np.asarray(b, np.float32)
        return np.abs(a.astype(np.float64) - b) / np.spacing(np.maximum(np.abs(a), np.abs(b)))

    assert ulps(d2, rd2).max() <= 2
    ref_d = np.sqrt(np.sort(rd2, 1).astype(np.float64)).astype(np.float32)
    assert ulps(np.sort(od, 1), ref_d).max() <= 2
    n4 = oracle_mod.lbvh_knn_normals(o, K, flip=(1e6, 1e6, 1e6))
    assert np.array_equal(n4, g[name + "_normals"])


@pytest.mark.parametrize("kind", ["uniform", "lattice", "duplicates"])
def test_canonical_knn_is_exact(oracle_mod, kind):
    rng = np.random.Generator(np.random.PCG64(5))
    if kind == "uniform":
        P = rng.uniform(-1, 1, (3000, 3)).astype(np.float32)
    elif kind == "lattice":
        g = np.stack(np.meshgrid(*[np.arange(14)] * 3, indexing="ij"), -1).reshape(-1, 3)
        P = (g * 0.25).astype(np.float32)
    else:
        P = rng.uniform(0, 1, (1000, 3)).astype(np.float32)
        P = np.concatenate([P, P[:300], P[:50]])
    Q = np.concatenate([P[::11], rng.uniform(-1.5, 1.5, (50, 3)).astype(np.float32)])
    s = oracle_mod.OracleSurface(P, threads=2)
    for k in (1, 7, 20):
        idx, dist, cnt = s.knn(Q, k)
        bi, bd = brute_knn(P, Q, k)
        assert (idx == bi).all()
        assert (dist == bd).all()
        assert (cnt == k).all()


def test_knn_fewer_points_than_k(oracle_mod):
    P = np.array([[0, 0, 0], [1, 0, 0], [0, 2, 0]], np.float32)
    s = oracle_mod.OracleSurface(P)
    idx, dist, cnt = s.knn(np.zeros((1, 3), np.float32), 5)
    assert cnt[0] == 3
    assert list(idx[0, :3]) == [0, 1, 2] and (idx[0, 3:] == 0xFFFFFFFF).all()
    assert np.isinf(dist[0, 3:]).all()


def test_reference_order_agrees_except_near_ties(oracle_mod):
    """The reference kd-tree ranks by double d2; the canonical order by float32
    d2 and index.  Sets may differ only where float32 d2 ties at the k-th."""
    rng = np.random.Generator(np.random.PCG64(6))
    P = rng.uniform(0, 1, (20000, 3)).astype(np.float32)
    s = oracle_mod.OracleSurface(P, threads=2)
    Q = P[::13]
    a, da, _ = s.knn(Q, 10, canonical=True)
    b, db, _ = s.knn(Q, 10, canonical=False)
    same = np.array([set(x) == set(y) for x, y in zip(a, b)])
    assert same.mean() > 0.999
    for r in np.nonzero(~same)[0]:
        assert abs(float(da[r, -1]) - float(db[r, -1])) <= 1e-6 * float(da[r, -1])


def test_ipca_normals_match_fp64_pca(oracle_mod):
    pts = GOLD["sphere/points"]
    s = oracle_mod.OracleSurface(pts)
    flip = np.array([0.5, 0.5, 0.5], np.float32)
    n, k = s.normals(5, nem=3, adaptive=True, flip=flip, with_k=True)
    sel = np.arange(0, len(pts), 5)
    nb = np.concatenate([s.knn(pts[i:i + 1], int(k[i]))[0] for i in sel])
    ref = fp64_pca_normals(pts, sel, nb, flip)
    assert np.percentile(angle_deg(n[sel], ref), 99.9) < 0.05


def test_oracle_reproduces_frozen_outputs(oracle_mod):
    for name in ("sphere", "scan", "lattice"):
        pts = GOLD[name + "/points"]
        s = oracle_mod.OracleSurface(pts, threads=2)
        idx, dist, _ = s.knn(pts[::7], 8)
        assert (idx == GOLD[name + "/knn_idx"]).all() and (dist == GOLD[name + "/knn_dist"]).all()
        flip = np.array([0.5, 0.5, 0.5], np.float32) if name == "sphere" else np.zeros(3, np.float32)
        for nem in (0, 1, 2, 3):
            n, k = s.normals(5, nem=nem, adaptive=True, flip=flip, with_k=True)
            assert (k == GOLD["%s/kused_nem%d" % (name, nem)]).all()
            assert np.array_equal(n, GOLD["%s/normals_nem%d" % (name, nem)], equal_nan=True)
        inter = s.interpolate(GOLD[name + "/normals_nem3"], 6)
        assert np.array_equal(inter, GOLD[name + "/interp"], equal_nan=True)
        proj, eucl = s.distance(inter, 4, GOLD[name + "/dist_q"])
        assert np.array_equal(proj, GOLD[name + "/dist_proj"], equal_nan=True)
        vs = float(GOLD[name + "/voxelsize"])
        r = s.reconstruct(inter, voxelsize=vs, kd=4, decomposition="PMC")
        for key in ("cells_all", "cells_valid", "qp_lattice", "qp_pos", "qp_dist", "qp_invalid"):
            assert np.array_equal(r[key], GOLD["%s/PMC/%s" % (name, key)], equal_nan=True), key
        a = canonical_mesh(r["vkeys"], r["vpos"], r["faces"])
        b = canonical_mesh(GOLD[name + "/PMC/vkeys"], GOLD[name + "/PMC/vpos"], GOLD[name + "/PMC/faces"])
        for x, y in zip(a, b):
            assert np.array_equal(x, y)


def test_mesh_is_closed_on_a_sphere(oracle_mod):
    """Marching cubes on a closed surface gives a mesh in which no edge is
    shared by more than two faces and almost every edge by exactly two (the
    rest border the few holes left by culled cells)."""
    pts = GOLD["sphere/points"]
    s = oracle_mod.OracleSurface(pts)
    flip = np.array([0.5, 0.5, 0.5], np.float32)
    n = s.interpolate(s.normals(5, nem=3, flip=flip), 6)
    r = s.reconstruct(n, voxelsize=0.05, kd=4, decomposition="MC")
    f = r["faces"].astype(np.int64)
    e = np.sort(np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]]), axis=1)
    _, counts = np.unique(e, axis=0, return_counts=True)
    assert len(f) > 100
    assert counts.max() == 2
    assert (counts == 2).mean() > 0.98


def test_grid_invalid_rule_and_culling(oracle_mod):
    pts = GOLD["scan/points"]
    vs = float(GOLD["scan/voxelsize"])
    s = oracle_mod.OracleSurface(pts)
    r = s.reconstruct(GOLD["scan/interp"], voxelsize=vs, kd=4)
    # culled cells are exactly the cells with an invalid corner
    lat = {tuple(x): bool(i) for x, i in zip(r["qp_lattice"], r["qp_invalid"])}
    corner = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]])
    valid = {tuple(c) for c in r["cells_valid"]}
    for c in r["cells_all"]:
        ok = not any(lat[tuple(c + o)] for o in corner)
        assert ok == (tuple(c) in valid)


def test_unsupported_method(oracle_mod):
    s = oracle_mod.OracleSurface(GOLD["sphere/points"])
    with pytest.raises(ValueError):
        s.normals(5, nem=5)


def test_lbvh_comparator_fit_restatement(oracle_mod):
    """The restated LBVHIndex::knn_normals fit (nem 4): close to FP64 PCA of
    the same neighbours (slot 0 left out) on a dense noisy sphere, flipped
    toward the flip point, zero for collinear neighbourhoods and for fewer
    than 3 neighbours."""
    rng = np.random.Generator(np.random.PCG64(5))
    v = rng.standard_normal((40_000, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    P = (0.5 * v + 0.0005 * rng.standard_normal((40_000, 3))).astype(np.float32)
    S = oracle_mod.OracleSurface(P)
    n = oracle_mod.lbvh_knn_normals(S, 20, flip=(0.0, 0.0, 0.0))
    idx, _, _ = S.knn(P, 20)
    Q = P.astype(np.float64)[idx[:, 1:].astype(np.int64)]
    C = Q - Q.mean(1, keepdims=True)
    _, vec = np.linalg.eigh(np.einsum("nki,nkj->nij", C, C))
    assert np.percentile(angle_deg(vec[:, :, 0], n, unsigned=True), 99) < 2.0
    assert np.all((n * P).sum(1) < 0)  # toward the centre
    line = np.c_[np.linspace(0, 1, 50), np.zeros(50), np.zeros(50)].astype(np.float32)
    assert not oracle_mod.lbvh_knn_normals(oracle_mod.OracleSurface(line), 10).any()
    two = np.array([[0, 0, 0], [1, 0, 0]], np.float32)
    assert not oracle_mod.lbvh_knn_normals(oracle_mod.OracleSurface(two), 10).any()


def _cells_and_tsdf(r):
    """Valid cells of an oracle reconstruction as stored chunk cells:
    centres (index + 0.5) * vs and the 8 corner distances."""
    vs = np.float32(r["voxelsize"])
    corners = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]])
    key = {tuple(v): i for i, v in enumerate(r["qp_lattice"].tolist())}
    cells = r["cells_valid"].astype(np.int64)
    ids = np.array([[key[tuple(c)] for c in (v + corners).tolist()] for v in cells])
    return (cells.astype(np.float32) + np.float32(0.5)) * vs, r["qp_dist"][ids]


def test_merged_grid_reproduces_the_chunk_mesh(oracle_mod):
    """HashGrid(chunks, innerBoxes, ...) restated: the stored cells of one
    reconstruction, merged back (as one chunk, and as two overlapping chunks
    cut by inner boxes), give the same marching-cubes mesh."""
    from lvr2_gb300 import synthetic
    P = synthetic.spheres_tori(20_000, seed=6)
    o = oracle_mod.OracleSurface(P)
    normals = o.normals(10, nem=3)
    r = o.reconstruct(normals, voxelsize=0.03, kd=10, decomposition="MC")
    centers, tsdf = _cells_and_tsdf(r)
    ref = canonical_mesh(r["vkeys"], r["vpos"], r["faces"])
    m = oracle_mod.reconstruct_cells(centers, tsdf, r["voxelsize"])
    got = canonical_mesh(m["vkeys"], m["vpos"], m["faces"])
    assert all(np.array_equal(a, b) for a, b in zip(ref, got))
    cut = np.float32(0.5)
    a = centers[:, 0] <= cut + 0.1
    b = centers[:, 0] >= cut - 0.1  # overlapping chunks; the inner boxes split them at `cut`
    C = np.concatenate([centers[a], centers[b]])
    T = np.concatenate([tsdf[a], tsdf[b]])
    off = np.array([0, a.sum(), a.sum() + b.sum()], np.int64)
    big = 1e9
    boxes = np.array([[-big, -big, -big, cut, big, big], [cut, -big, -big, big, big, big]], np.float32)
    m2 = oracle_mod.reconstruct_cells(C, T, r["voxelsize"], chunk_offsets=off, inner_boxes=boxes)
    got2 = canonical_mesh(m2["vkeys"], m2["vpos"], m2["faces"])
    assert len(m2["cells_all"]) == len(centers)
    assert all(np.array_equal(x, y) for x, y in zip(ref, got2))


def test_halfedge_restatement_is_a_valid_pmp_connectivity(oracle_mod):
    """The canonical half-edge arrays of an open marching-cubes mesh: next and
    prev are inverse, every face is one 3-cycle in corner order, boundary
    halfedges form closed loops, halfedge h leaves the vertex h ^ 1 points
    to, a boundary vertex's halfedge is a boundary one, and edges are numbered
    by first appearance (pmp's add_face over faces 0..F-1)."""
    from lvr2_gb300 import synthetic
    P = synthetic.spheres_tori(20_000, seed=6)
    P = P[P[:, 0] < 0.5]
    o = oracle_mod.OracleSurface(P)
    r = o.reconstruct(o.normals(10, nem=3), voxelsize=0.03, kd=10, decomposition="PMC")
    F = r["faces"].astype(np.int64)
    nv = len(r["vpos"])
    H = oracle_mod.halfedges(F, nv)
    assert H["complex_edges"] == 0 and H["boundary_halfedges"] > 0
    nxt, prv, hv, hf = (H[k].astype(np.int64) for k in ("he_next", "he_prev", "he_vertex", "he_face"))
    nh = 2 * H["edges"]
    assert np.array_equal(prv[nxt], np.arange(nh)) and np.array_equal(nxt[prv], np.arange(nh))
    fh = H["face_he"].astype(np.int64)
    assert np.array_equal(nxt[nxt[nxt[fh]]], fh)
    assert np.array_equal(hv[fh], F[:, 0]) and np.array_equal(hv[nxt[fh]], F[:, 1])
    assert np.array_equal(hv[nxt[nxt[fh]]], F[:, 2])
    assert np.array_equal(hf[fh], np.arange(len(F)))
    bnd = np.flatnonzero(hf == 0xFFFFFFFF)
    assert np.all(hf[nxt[bnd]] == 0xFFFFFFFF)  # boundary loops stay on the boundary
    assert np.array_equal(hv[bnd ^ 1], hv[prv[bnd]])  # consecutive boundary halfedges share a vertex
    vh = H["vertex_he"].astype(np.int64)
    used = vh != 0xFFFFFFFF
    assert np.array_equal(hv[vh[used] ^ 1], np.flatnonzero(used))
    on_b = np.zeros(nv, bool)
    on_b[hv[bnd ^ 1]] = True
    assert np.all(hf[vh[on_b]] == 0xFFFFFFFF)
    # first-appearance edge numbering
    seen, order = {}, []
    for f in F:
        for c in range(3):
            k = (min(f[c], f[(c + 1) % 3]), max(f[c], f[(c + 1) % 3]))
            if k not in seen:
                seen[k] = len(seen)
                order.append((f[c], f[(c + 1) % 3]))
    first = np.array(order)
    assert np.array_equal(hv[0::2], first[:, 1]) and np.array_equal(hv[1::2], first[:, 0])


def test_halfedge_restatement_topology_cases(oracle_mod):
    """Complex edges (three faces on an edge, two faces of one orientation)
    are reported; a bow-tie vertex (two boundary gaps) is counted and its
    boundary halfedges still form closed loops."""
    three = np.array([[0, 1, 2], [1, 0, 3], [0, 1, 4]])
    assert oracle_mod.halfedges(three, 5)["complex_edges"] == 1
    same = np.array([[0, 1, 2], [0, 1, 3]])
    assert oracle_mod.halfedges(same, 4)["complex_edges"] == 1
    bowtie = np.array([[0, 1, 2], [0, 3, 4]])  # two triangles sharing vertex 0 only
    H = oracle_mod.halfedges(bowtie, 5)
    assert H["complex_edges"] == 0 and H["complex_vertices"] == 1 and H["boundary_halfedges"] == 6
    nxt = H["he_next"].astype(np.int64)
    hf = H["he_face"]
    bnd = np.flatnonzero(hf == 0xFFFFFFFF)
    seen = set()
    for b in bnd:  # every boundary loop closes within the boundary halfedges
        h, steps = b, 0
        while True:
            seen.add(h)
            h = nxt[h]
            steps += 1
            assert hf[h] == 0xFFFFFFFF and steps <= len(bnd)
            if h == b:
                break
    assert seen == set(bnd.tolist())


def test_ransac_restatement_properties(oracle_mod):
    """nem 1 (calcPlaneRANSAC): on a plane every candidate plane is the plane
    itself, so the normals are exactly (0, 0, +-1), oriented to the flip
    point; the three plane points are the cloud's points at the drawn ranks
    (lvr2 indexes m_points with them), so with the cloud's first four points
    on a line and k = 4 every candidate is degenerate: the null normal scores
    0 and wins everywhere; fewer than three neighbours: no plane (NaN)."""
    rng = np.random.Generator(np.random.PCG64(11))
    P = np.zeros((3000, 3), np.float32)
    P[:, :2] = rng.uniform(-1, 1, (3000, 2))
    o = oracle_mod.OracleSurface(P)
    for kn, adaptive in ((10, False), (4, True)):
        n = o.normals(kn, nem=1, adaptive=adaptive, flip=np.array([0, 0, 5], np.float32))
        assert np.array_equal(n, np.tile(np.float32([0, 0, 1]), (len(P), 1)))
    n = o.normals(10, nem=1, adaptive=False, flip=np.array([0, 0, -5], np.float32))
    assert np.array_equal(n, np.tile(np.float32([0, 0, -1]), (len(P), 1)))

    Q = rng.uniform(-1, 1, (2000, 3)).astype(np.float32)
    Q[:4] = np.float32([[0, 0, 0], [0.5, 0, 0], [-0.25, 0, 0], [0.75, 0, 0]])
    n = oracle_mod.OracleSurface(Q).normals(2, nem=1, adaptive=False)
    assert np.array_equal(n, np.zeros_like(n))
    # the same cloud with the line moved away from the front: real planes
    n = oracle_mod.OracleSurface(np.roll(Q, 7, axis=0)).normals(2, nem=1, adaptive=False)
    assert np.isfinite(n).all() and (np.abs(np.linalg.norm(n, axis=1) - 1) < 1e-6).mean() > 0.9

    n = oracle_mod.OracleSurface(Q).normals(1, nem=1, adaptive=False)  # k = 2 neighbours
    assert np.isnan(n).all()


def _ransac_numpy(P, rows, draws, q, flip):
    """calcPlaneRANSAC (AdaptiveKSearchSurface.tcc:689-781) in float32 scalar
    numpy arithmetic, one rounding per operation in the reference's order,
    over a neighbour row (ascending (d2, index)) and the draw sequence."""
    f = np.float32
    m = len(rows)
    ns = min(50, m)
    best = (f(0), f(0), f(1))
    bestdist = f(np.finfo(np.float32).max)
    nonimproving = 0
    for t in range(10):
        if nonimproving >= 5:
            break
        a, b, c = (P[int(i)] for i in draws[t, :3])
        u = (a[0] - b[0], a[1] - b[1], a[2] - b[2])
        v = (a[0] - c[0], a[1] - c[1], a[2] - c[2])
        n = [u[1] * v[2] - u[2] * v[1], u[2] * v[0] - u[0] * v[2], u[0] * v[1] - u[1] * v[0]]
        if not (n[0] == 0 and n[1] == 0 and n[2] == 0):
            ln = np.sqrt((n[0] * n[0] + n[1] * n[1]) + n[2] * n[2])
            n = [n[0] / ln, n[1] / ln, n[2] / ln]
        d1 = (a[0] * n[0] + a[1] * n[1]) + a[2] * n[2]
        dist = f(0)
        for j in draws[t, 3:3 + ns]:
            p = P[int(rows[int(j)])]
            dist = dist + abs(((p[0] * n[0] + p[1] * n[1]) + p[2] * n[2]) - d1)
        dist = dist / f(ns)
        if dist < bestdist:
            bestdist, best, nonimproving = dist, tuple(n), 0
        else:
            nonimproving += 1
    n = list(best)
    t = (flip[0] - q[0], flip[1] - q[1], flip[2] - q[2])
    if (n[0] * t[0] + n[1] * t[1]) + n[2] * t[2] < 0:
        n = [-n[0], -n[1], -n[2]]
        if not (n[0] == 0 and n[1] == 0 and n[2] == 0):
            ln = np.sqrt((n[0] * n[0] + n[1] * n[1]) + n[2] * n[2])
            n = [n[0] / ln, n[1] / ln, n[2] / ln]
    return np.array(n, np.float32)


@pytest.mark.parametrize("name", ["sphere", "lattice"])
def test_ransac_oracle_against_numpy_restatement(oracle_mod, name):
    """The oracle's nem 1 equals a second, numpy restatement bit for bit,
    given the same neighbour rows, adaptive k and draw sequence."""
    P = GOLD[name + "/points"]
    flip = np.float32([0.5, 0.5, 0.5]) if name == "sphere" else np.zeros(3, np.float32)
    s = oracle_mod.OracleSurface(P, threads=1)
    ref, k = s.normals(5, nem=1, adaptive=True, flip=flip, with_k=True)
    sample = np.arange(0, len(P), max(1, len(P) // 150))
    draws = {}
    for i in sample:
        K = int(k[i])
        m = min(K, len(P))
        if m not in draws:
            draws[m] = oracle_mod.ransac_draws(m)
        rows, _, cnt = s.knn(P[i:i + 1], K)
        got = _ransac_numpy(P, rows[0, :int(cnt[0])], draws[m], P[i], flip)
        assert np.array_equal(got.view(np.uint32), ref[i].view(np.uint32)), (i, got, ref[i])


def _pmp_add_faces(faces):
    """pmp SurfaceMesh::add_face over faces 0..F-1
    (src/liblvr2/geometry/pmp/SurfaceMesh.cpp:283-460), sequentially, for the
    parts that do not depend on boundary relinking: an edge is created when a
    face first meets it, corners in order (new_edge(v_i, v_i+1): halfedge 2e
    points to v_i+1), the face's halfedges link in a cycle, and the face keeps
    the halfedge from its last corner to its first."""
    NONE = 0xFFFFFFFF
    he_of, he_vertex, he_face, he_next, face_he = {}, [], [], [], []
    for f, tri in enumerate(faces):
        vs = [int(v) for v in tri]
        hs = []
        for i in range(3):
            a, b = vs[i], vs[(i + 1) % 3]
            h = he_of.get((a, b))
            if h is None:
                h = len(he_vertex)
                he_of[(a, b)], he_of[(b, a)] = h, h + 1
                he_vertex += [b, a]
                he_face += [NONE, NONE]
                he_next += [NONE, NONE]
            hs.append(h)
        for i, h in enumerate(hs):
            he_face[h] = f
            he_next[h] = hs[(i + 1) % 3]
        face_he.append(hs[2])
    return (np.array(he_vertex, np.int64), np.array(he_face, np.int64), np.array(he_next, np.int64),
            np.array(face_he, np.int64))


@pytest.mark.parametrize("n,holes,seed", [(2, 0.0, 0), (9, 0.3, 1), (40, 0.1, 2)])
def test_halfedge_restatement_matches_sequential_add_face(oracle_mod, n, holes, seed):
    rng = np.random.default_rng(seed)
    ij = np.arange(n * n).reshape(n, n)
    a, b, c, d = ij[:-1, :-1].ravel(), ij[:-1, 1:].ravel(), ij[1:, :-1].ravel(), ij[1:, 1:].ravel()
    F = np.concatenate([np.stack([a, b, d], 1), np.stack([a, d, c], 1)])
    F = F[rng.random(len(F)) >= holes]
    F = F[rng.permutation(len(F))]
    r = rng.integers(0, 3, len(F))
    F = np.stack([F[np.arange(len(F)), (r + j) % 3] for j in range(3)], 1)
    H = oracle_mod.halfedges(F, n * n)
    hv, hf, hn, fh = _pmp_add_faces(F)
    assert H["complex_edges"] == 0 and H["edges"] * 2 == len(hv)
    assert np.array_equal(H["he_vertex"], hv) and np.array_equal(H["he_face"], hf)
    assert np.array_equal(H["face_he"], fh)
    inner = hf != 0xFFFFFFFF
    assert np.array_equal(H["he_next"][inner], hn[inner])
    # where a vertex has a single boundary gap, pmp's choices are forced: the
    # boundary halfedge into it continues with the one leaving it, and the
    # vertex keeps that outgoing boundary halfedge (adjust_outgoing_halfedge)
    bnd = np.flatnonzero(~inner)
    src = hv[bnd ^ 1]
    starts, counts = np.unique(src, return_counts=True)
    single = set(starts[counts == 1].tolist())
    out_of = {int(v): int(h) for v, h in zip(src, bnd) if int(v) in single}
    for h in bnd:
        v = int(hv[h])
        if v in single:
            assert H["he_next"][h] == out_of[v]
    for v, h in out_of.items():
        assert H["vertex_he"][v] == h


def test_ransac_independent_of_tie_order(oracle_mod):
    """RANSAC draws neighbours by rank, so it depends on the neighbour order;
    with the reference kd-tree's own order (double d2, ties in traversal
    order) in place of (float d2, index) its normals stay bit-identical on
    the golden clouds, the lattice's many exact ties included."""
    for name in ("sphere", "scan", "lattice"):
        P = GOLD[name + "/points"]
        s = oracle_mod.OracleSurface(P)
        flip = ((P.min(0) + P.max(0)) / 2).astype(np.float32)
        a = s.normals(10, nem=1, adaptive=True, flip=flip, canonical=True)
        b = s.normals(10, nem=1, adaptive=True, flip=flip, canonical=False)
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), name


def _iterative_numpy(P, rows, q, flip):
    """calcPlaneIterative, nem 2 (AdaptiveKSearchSurface.tcc:522-607), in
    float32 scalar numpy arithmetic in the reference's order."""
    f = np.float32
    xx = xy = xz = yy = yz = zz = f(0)
    for j in rows:
        r = P[int(j)] - q
        xx = xx + r[0] * r[0]
        xy = xy + r[0] * r[1]
        xz = xz + r[0] * r[2]
        yy = yy + r[1] * r[1]
        yz = yz + r[1] * r[2]
        zz = zz + r[2] * r[2]
    det_x, det_y, det_z = yy * zz - yz * yz, xx * zz - xz * xz, xx * yy - xy * xy
    if det_x >= det_y and det_x >= det_z:
        d = (f(1), (xz * yz - xy * zz) / det_x, (xy * yz - xz * yy) / det_x)
    elif det_y >= det_x and det_y >= det_z:
        d = ((yz * xz - xy * zz) / det_y, f(1), (xy * xz - yz * xx) / det_y)
    else:
        d = ((yz * xy - xz * yy) / det_z, (xz * xy - yz * xx) / det_z, f(1))
    inv = f(1) / np.sqrt((d[0] * d[0] + d[1] * d[1]) + d[2] * d[2])
    n = [d[0] * inv, d[1] * inv, d[2] * inv]
    t = (flip[0] - q[0], flip[1] - q[1], flip[2] - q[2])
    if (n[0] * t[0] + n[1] * t[1]) + n[2] * t[2] < 0:
        n = [-n[0], -n[1], -n[2]]
        if not (n[0] == 0 and n[1] == 0 and n[2] == 0):
            ln = np.sqrt((n[0] * n[0] + n[1] * n[1]) + n[2] * n[2])
            n = [n[0] / ln, n[1] / ln, n[2] / ln]
    return np.array(n, np.float32)


@pytest.mark.parametrize("name", ["sphere", "scan"])
def test_iterative_oracle_against_numpy_restatement(oracle_mod, name):
    """The oracle's nem 2 equals a second, numpy restatement bit for bit,
    given the same neighbour rows and adaptive k."""
    P = GOLD[name + "/points"]
    flip = np.float32([0.5, 0.5, 0.5]) if name == "sphere" else np.zeros(3, np.float32)
    s = oracle_mod.OracleSurface(P, threads=1)
    ref, k = s.normals(5, nem=2, adaptive=True, flip=flip, with_k=True)
    with np.errstate(divide="ignore", invalid="ignore"):
        for i in np.arange(0, len(P), max(1, len(P) // 200)):
            rows, _, cnt = s.knn(P[i:i + 1], int(k[i]))
            got = _iterative_numpy(P, rows[0, :int(cnt[0])], P[i], flip)
            assert np.array_equal(got.view(np.uint32), ref[i].view(np.uint32)), (i, got, ref[i])


@pytest.mark.parametrize("name", ["sphere", "scan", "lattice"])
def test_distance_oracle_against_numpy_restatement(oracle_mod, name):
    """AdaptiveKSearchSurface::distance (AdaptiveKSearchSurface.tcc:414-457)
    restated a second time in float32 numpy scalar arithmetic: running sums
    of the kd nearest points and normals, both divided by kd, the mean normal
    normalised (a null mean stays null), then the projected and Euclidean
    distances.  Equals the oracle bit for bit."""
    P = GOLD[name + "/points"]
    N = GOLD[name + "/interp"]
    Q = GOLD[name + "/dist_q"]
    s = oracle_mod.OracleSurface(P, threads=1)
    proj, eucl = s.distance(N, 4, Q)
    assert np.array_equal(proj, GOLD[name + "/dist_proj"], equal_nan=True)
    f = np.float32
    rows, _, cnt = s.knn(Q, 4)
    for i in range(0, len(Q), max(1, len(Q) // 200)):
        c = [f(0), f(0), f(0)]
        m = [f(0), f(0), f(0)]
        for j in rows[i, :int(cnt[i])]:
            for a in range(3):
                c[a] = c[a] + P[int(j), a]
                m[a] = m[a] + N[int(j), a]
        kf = f(int(cnt[i]))
        c = [x / kf for x in c]
        m = [x / kf for x in m]
        if not (m[0] == 0 and m[1] == 0 and m[2] == 0):
            ln = np.sqrt((m[0] * m[0] + m[1] * m[1]) + m[2] * m[2])
            m = [x / ln for x in m]
        d = [Q[i, a] - c[a] for a in range(3)]
        p_ = (d[0] * m[0] + d[1] * m[1]) + d[2] * m[2]
        e_ = np.sqrt((d[0] * d[0] + d[1] * d[1]) + d[2] * d[2])
        assert np.float32(p_).view(np.uint32) == proj[i].view(np.uint32), i
        assert np.float32(e_).view(np.uint32) == eucl[i].view(np.uint32), i


@pytest.mark.parametrize("name", ["sphere", "scan", "lattice"])
def test_interpolation_oracle_against_numpy_restatement(oracle_mod, name):
    """interpolateSurfaceNormals (AdaptiveKSearchSurface.tcc:293-335) restated
    a second time in float32 numpy scalar arithmetic: the point's own normal
    plus the normals of its ki nearest (itself among them), normalised (a
    null sum stays null).  Equals the oracle bit for bit."""
    P = GOLD[name + "/points"]
    N = GOLD[name + "/normals_nem3"]
    s = oracle_mod.OracleSurface(P, threads=1)
    out = s.interpolate(N, 6)
    assert np.array_equal(out, GOLD[name + "/interp"], equal_nan=True)
    rows, _, cnt = s.knn(P, 6)
    for i in range(0, len(P), max(1, len(P) // 300)):
        m = [N[i, 0], N[i, 1], N[i, 2]]
        for j in rows[i, :int(cnt[i])]:
            m = [m[a] + N[int(j), a] for a in range(3)]
        if not (m[0] == 0 and m[1] == 0 and m[2] == 0):
            ln = np.sqrt((m[0] * m[0] + m[1] * m[1]) + m[2] * m[2])
            m = [x / ln for x in m]
        assert np.array_equal(np.float32(m).view(np.uint32), out[i].view(np.uint32)), i


@pytest.mark.parametrize("name", ["sphere", "scan", "lattice"])
def test_mc_vertices_against_numpy_restatement(oracle_mod, name):
    """FastBox::calcIntersection (FastBox.tcc:133-158) restated a second time:
    every MC vertex lies on the lattice edge its key names, between the grid
    vertices at lattice l and l + e_axis, at x2 - d2 (x1 - x2) / (d1 - d2)
    in float32 (low corner first; an exact zero returns that corner).  Equals
    the oracle's vertex positions bit for bit."""
    P = GOLD[name + "/points"]
    s = oracle_mod.OracleSurface(P, threads=1)
    vs = float(GOLD[name + "/voxelsize"])
    r = s.reconstruct(GOLD[name + "/interp"], voxelsize=vs, kd=4, decomposition="MC")
    at = {tuple(l): i for i, l in enumerate(r["qp_lattice"].tolist())}
    pos, dist = r["qp_pos"], r["qp_dist"]
    assert len(r["vkeys"]) > 50
    for key, vp in zip(r["vkeys"], r["vpos"]):
        l, axis = tuple(int(x) for x in key[:3]), int(key[3])
        h = list(l)
        h[axis] += 1
        a, b = at[l], at[tuple(h)]
        x1, x2, d1, d2 = pos[a, axis], pos[b, axis], dist[a], dist[b]
        assert (d1 < 0 < d2) or (d2 < 0 < d1) or d1 == 0 or d2 == 0
        x = x1 if d1 == 0 else x2 if d2 == 0 else x2 - d2 * (x1 - x2) / (d1 - d2)
        want = pos[a].copy()
        want[axis] = x
        assert np.array_equal(want.view(np.uint32), vp.view(np.uint32)), (key, want, vp)


@pytest.mark.parametrize("name", ["sphere", "scan", "lattice"])
def test_grid_vertex_positions_against_numpy_restatement(oracle_mod, name):
    """HashGrid::indexToCenter and addBox (HashGrid.hpp:276-281,
    HashGrid.tcc:246-249) restated: the grid vertex at lattice L is corner 0
    (offset (-1, -1, -1)) of cell L, at (L + 0.5f) * vs + (-1) * (vs / 2.0f)
    in float32 per coordinate.  Equals the oracle's positions bit for bit."""
    P = GOLD[name + "/points"]
    s = oracle_mod.OracleSurface(P, threads=1)
    r = s.reconstruct(GOLD[name + "/interp"], voxelsize=float(GOLD[name + "/voxelsize"]), kd=4, decomposition="MC")
    vs = np.float32(r["voxelsize"])
    L = r["qp_lattice"]
    centre = (L.astype(np.float32) + np.float32(0.5)) * vs
    want = centre + np.float32(-1.0) * (vs / np.float32(2.0))
    assert want.dtype == np.float32 and len(want) > 100
    assert np.array_equal(want.view(np.uint32), r["qp_pos"].view(np.uint32))


@pytest.mark.parametrize("name", ["sphere", "scan", "lattice"])
def test_culling_against_numpy_restatement(oracle_mod, name):
    """PointsetGrid::calcDistanceValues (PointsetGrid.tcc:111-185) restated:
    a grid vertex is invalid when its Euclidean distance exceeds
    1.75 * voxelsize, compared in double (1.75 is a double literal); its
    distance is the projected one; a cell with an invalid corner is erased."""
    P = GOLD[name + "/points"]
    N = GOLD[name + "/interp"]
    s = oracle_mod.OracleSurface(P, threads=1)
    r = s.reconstruct(N, voxelsize=float(GOLD[name + "/voxelsize"]), kd=4, decomposition="MC")
    proj, eucl = s.distance(N, 4, r["qp_pos"])
    assert np.array_equal(proj.view(np.uint32), r["qp_dist"].view(np.uint32))
    invalid = eucl.astype(np.float64) > 1.75 * np.float64(np.float32(r["voxelsize"]))
    assert np.array_equal(invalid, r["qp_invalid"].astype(bool))
    bad = {tuple(l) for l, x in zip(r["qp_lattice"].tolist(), invalid) if x}
    offs = [(i, j, k) for i in (0, 1) for j in (0, 1) for k in (0, 1)]
    keep = {tuple(c) for c in r["cells_all"].tolist()
            if not any((c[0] + o[0], c[1] + o[1], c[2] + o[2]) in bad for o in offs)}
    assert keep == {tuple(c) for c in r["cells_valid"].tolist()}
    assert 0 < len(keep) < len(r["cells_all"]) or name == "lattice"


@pytest.mark.parametrize("name", ["sphere", "scan", "lattice"])
@pytest.mark.parametrize("extrude", [True, False])
def test_grid_cells_against_numpy_restatement(oracle_mod, name, extrude):
    """PointsetGrid's cells (PointsetGrid.tcc:41-109) restated: the cell of a
    point is floor(p / vs) in float32 (HashGrid::calcIndex), kept when its
    centre (index + 0.5f) * vs lies in the surface's bounding box (min <= c
    <= max, BoundingBox::contains; the box given to the constructor, not
    the grown grid box); extrusion adds the 26 neighbours whose centres lie
    in that box."""
    P = GOLD[name + "/points"]
    s = oracle_mod.OracleSurface(P, threads=1)
    r = s.reconstruct(GOLD[name + "/interp"], voxelsize=float(GOLD[name + "/voxelsize"]), kd=4,
                      decomposition="MC", extrude=extrude)
    vs = np.float32(r["voxelsize"])
    lo, hi, _ = s.bbox()

    def inside(idx):
        c = (idx.astype(np.float32) + np.float32(0.5)) * vs
        return np.all((lo <= c) & (c <= hi), axis=1)

    idx = np.floor(P / vs).astype(np.int64)
    cells = np.unique(idx[inside(idx)], axis=0)
    if extrude:
        offs = np.array([(i, j, k) for i in (-1, 0, 1) for j in (-1, 0, 1) for k in (-1, 0, 1)], np.int64)
        cand = np.unique((cells[:, None, :] + offs[None]).reshape(-1, 3), axis=0)
        cells = cand[inside(cand)]
    assert {tuple(c) for c in cells.tolist()} == {tuple(c) for c in r["cells_all"].tolist()}


@pytest.mark.parametrize("name", ["sphere", "scan", "lattice"])
def test_adaptive_k_against_numpy_restatement(oracle_mod, name):
    """The adaptive k of calculateSurfaceNormals (AdaptiveKSearchSurface.tcc:
    187-216, boundingBoxOK :337-350) restated: k doubles before each of at
    most 5 searches; the search stops once every side of the neighbourhood's
    box (max - min, float32) is >= 0.05f times each other side."""
    P = GOLD[name + "/points"]
    s = oracle_mod.OracleSurface(P, threads=1)
    kn = 5
    _, kused = s.normals(kn, nem=3, adaptive=True, flip=np.zeros(3, np.float32), with_k=True)
    assert (kused == GOLD[name + "/kused_nem3"]).all()
    e = np.float32(0.05)
    sample = np.arange(0, len(P), max(1, len(P) // 200))
    want = np.zeros(len(sample), np.int64)
    todo = np.ones(len(sample), bool)
    k = kn
    for rnd in range(5):
        k *= 2
        rows, _, cnt = s.knn(P[sample], k)
        for t in np.flatnonzero(todo):
            nb = P[rows[t, :int(cnt[t])].astype(np.int64)]
            d = nb.max(0) - nb.min(0)
            ok = all(d[a] >= e * d[b] for a in range(3) for b in range(3) if a != b)
            if ok or rnd == 4:
                want[t] = k
                todo[t] = False
    assert np.array_equal(want, kused[sample])
    if name != "lattice":
        assert (want > 2 * kn).any() or name == "sphere"


def test_interpolated_normal_against_numpy_restatement(oracle_mod):
    """PointsetSurface::getInterpolatedNormal (PointsetSurface.tcc:61-74)
    restated: the default Normal (0, 1, 0) plus the ki nearest points'
    normals, each normalised as it is read, divided by ki; the result is
    returned through the Normal copy constructor, so it is not normalised."""
    P = GOLD["scan/points"]
    N = GOLD["scan/interp"]
    Q = GOLD["scan/dist_q"]
    s = oracle_mod.OracleSurface(P, threads=1)
    out = s.interpolated_normal(N, 6, Q)
    rows, _, cnt = s.knn(Q, 6)
    f = np.float32
    for i in range(0, len(Q), max(1, len(Q) // 300)):
        r = [f(0), f(1), f(0)]
        for j in rows[i, :int(cnt[i])]:
            n = [N[int(j), a] for a in range(3)]
            if not (n[0] == 0 and n[1] == 0 and n[2] == 0):
                ln = np.sqrt((n[0] * n[0] + n[1] * n[1]) + n[2] * n[2])
                n = [x / ln for x in n]
            r = [r[a] + n[a] for a in range(3)]
        r = [x / f(6) for x in r]
        assert np.array_equal(np.float32(r).view(np.uint32), out[i].view(np.uint32)), i
    assert (np.abs(np.linalg.norm(out, axis=1) - 1) > 1e-3).mean() > 0.5  # means, not unit vectors
