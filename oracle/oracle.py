"""ctypes wrapper of the CPU oracle (oracle/lvr_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() to
check its result, and by bench.py for the CPU baseline / reference arm.  The
product path (lvr2_gb300) never imports this module.
"""
import ctypes
import os
import subprocess
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "liblvroracle.so"

_f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
_u32p = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_i64p = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")
_u8p = np.ctypeslib.ndpointer(dtype=np.uint8, flags="C_CONTIGUOUS")
_vp = ctypes.c_void_p
_i64 = ctypes.c_int64
_int = ctypes.c_int

_lib = None


def build(quiet=True):
    """Compile the oracle with its Makefile (g++, OpenMP)."""
    out = subprocess.run(["make", "-C", str(HERE)], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    if not quiet:
        print(out.stdout)


def lib():
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        build()
    L = ctypes.CDLL(str(LIB_PATH))
    L.orc_create.restype = _vp
    L.orc_create.argtypes = [_f32p, _i64, _int, _int]
    L.orc_destroy.argtypes = [_vp]
    L.orc_bbox.argtypes = [_vp, _f32p]
    L.orc_knn.argtypes = [_vp, _f32p, _i64, _int, _int, _u32p, _f32p, _i32p, _int]
    L.orc_normals.argtypes = [_vp, _int, _int, _int, ctypes.c_void_p, _int, _f32p, ctypes.c_void_p, _int,
                              ctypes.c_void_p]
    L.orc_interpolate.argtypes = [_vp, _int, _f32p, _f32p, _int, _int]
    L.orc_ransac_draws.argtypes = [_i64, _u32p]
    L.orc_distance.argtypes = [_vp, _f32p, _int, _f32p, _i64, _int, _f32p, _f32p, _int]
    L.orc_interpolated_normal.argtypes = [_vp, _f32p, _int, _f32p, _i64, _int, _f32p, _int]
    L.orc_reconstruct.restype = _vp
    L.orc_reconstruct.argtypes = [_vp, _f32p, ctypes.c_float, _int, _int, _int, _int, _int,
                                  ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, _i64, _int]
    L.orc_recon_destroy.argtypes = [_vp]
    L.orc_recon_counts.argtypes = [_vp, _i64p, _f32p]
    L.orc_recon_grid.argtypes = [_vp, _i32p, _f32p, _f32p, _u8p]
    L.orc_recon_cells.argtypes = [_vp, _i32p, _i32p]
    L.orc_recon_mesh.argtypes = [_vp, _i32p, _f32p, _i32p]
    L.orc_recon_optimize_planar.restype = _i64
    L.orc_recon_optimize_planar.argtypes = [_vp, _vp, _int, _int, _int]
    L.orc_mc_table.argtypes = [_i32p]
    L.orc_reconstruct_cells.restype = _vp
    L.orc_reconstruct_cells.argtypes = [_f32p, _f32p, _i64, _i64p, _int, ctypes.c_void_p, ctypes.c_float, _int]
    _lib = L
    return L


def _pts(a):
    return np.ascontiguousarray(a, dtype=np.float32).reshape(-1, 3)


class OracleSurface:
    """The reference CPU surface: SearchKDTree + AdaptiveKSearchSurface."""

    def __init__(self, points, leaf_size=20, threads=0):
        self.points = _pts(points)
        self.threads = threads
        self._h = lib().orc_create(self.points.reshape(-1), len(self.points), leaf_size, threads)

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_destroy(self._h)
            self._h = None

    @property
    def n(self):
        return len(self.points)

    def bbox(self):
        out = np.zeros(9, np.float32)
        lib().orc_bbox(self._h, out)
        return out[0:3], out[3:6], out[6:9]

    def knn(self, queries, k, canonical=True):
        q = _pts(queries)
        idx = np.empty((len(q), k), np.uint32)
        dist = np.empty((len(q), k), np.float32)
        cnt = np.empty(len(q), np.int32)
        lib().orc_knn(self._h, q.reshape(-1), len(q), k, int(canonical), idx, dist, cnt, self.threads)
        return idx, dist, cnt

    def normals(self, kn, nem=3, adaptive=True, flip=None, canonical=True, with_k=False, flip_targets=None):
        """flip_targets: optional (n, 3) per-point flip points (NaN row: use
        flip), as the scan-pose flip gives them."""
        out = np.empty((self.n, 3), np.float32)
        kused = np.empty(self.n, np.int32) if with_k else None
        fl = None
        if flip is not None:
            fl_arr = np.ascontiguousarray(flip, np.float32)
            fl = fl_arr.ctypes.data_as(ctypes.c_void_p)
        ft = None
        if flip_targets is not None:
            ft_arr = np.ascontiguousarray(flip_targets, np.float32).reshape(self.n, 3)
            ft = ft_arr.ctypes.data_as(ctypes.c_void_p)
        rc = lib().orc_normals(self._h, kn, nem, int(adaptive), fl, int(canonical), out,
                               kused.ctypes.data_as(ctypes.c_void_p) if with_k else None, self.threads, ft)
        if rc != 0:
            raise ValueError("oracle normals: unsupported nem %d" % nem)
        return (out, kused) if with_k else out

    def interpolate(self, normals, ki, canonical=True):
        nin = _pts(normals)
        out = np.empty_like(nin)
        lib().orc_interpolate(self._h, ki, nin.reshape(-1), out, int(canonical), self.threads)
        return out

    def distance(self, normals, kd, queries, canonical=True):
        nrm = _pts(normals)
        q = _pts(queries)
        proj = np.empty(len(q), np.float32)
        eucl = np.empty(len(q), np.float32)
        lib().orc_distance(self._h, nrm.reshape(-1), kd, q.reshape(-1), len(q), int(canonical),
                           proj, eucl, self.threads)
        return proj, eucl

    def interpolated_normal(self, normals, ki, queries, canonical=True):
        nrm = _pts(normals)
        q = _pts(queries)
        out = np.empty((len(q), 3), np.float32)
        lib().orc_interpolated_normal(self._h, nrm.reshape(-1), ki, q.reshape(-1), len(q),
                                      int(canonical), out, self.threads)
        return out

    def reconstruct(self, normals, voxelsize=None, intersections=None, extrude=True, kd=5,
                    decomposition="PMC", canonical=True, grid_override=None, planar_kc=0):
        """PointsetGrid + calcDistanceValues + marching cubes (+ the PMC
        optimizePlanarFaces post-pass with planar_kc nearest points when
        planar_kc > 0).  Returns a dict."""
        nrm = _pts(normals)
        if intersections is not None and intersections > 0:
            res, isvs = float(intersections), 0
        else:
            res, isvs = float(voxelsize), 1
        dec = {"MC": 0, "PMC": 1}[decomposition]
        args = [None, None, None, 0]
        keep = None
        if grid_override is not None:
            lat, dist, inv = grid_override
            keep = (np.ascontiguousarray(lat, np.int32), np.ascontiguousarray(dist, np.float32),
                    np.ascontiguousarray(inv, np.uint8))
            args = [keep[0].ctypes.data_as(ctypes.c_void_p), keep[1].ctypes.data_as(ctypes.c_void_p),
                    keep[2].ctypes.data_as(ctypes.c_void_p), len(keep[1])]
        L = lib()
        t0 = time.perf_counter()
        h = L.orc_reconstruct(self._h, nrm.reshape(-1), res, isvs, int(extrude), kd, dec,
                              int(canonical), *args, self.threads)
        t1 = time.perf_counter()
        try:
            moved = 0
            if planar_kc > 0:
                moved = int(L.orc_recon_optimize_planar(h, self._h, int(planar_kc), int(canonical), self.threads))
        except BaseException:
            L.orc_recon_destroy(h)
            raise
        t2 = time.perf_counter()
        out = _recon_result(h)
        out["planar_moved"] = moved
        # wall-clock of the two library calls (grid + distances + culling +
        # marching cubes; the planar pass), for the CPU baseline's stages
        out["seconds_reconstruct"] = t1 - t0
        out["seconds_planar"] = t2 - t1
        return out


def _recon_result(h):
    """Arrays of an orc_recon handle (destroyed here)."""
    L = lib()
    try:
        c = np.zeros(8, np.int64)
        f = np.zeros(4, np.float32)
        L.orc_recon_counts(h, c, f)
        ncell, nqp, nvalid, nv, nf = (int(x) for x in c[:5])
        lat = np.empty((nqp, 3), np.int32)
        pos = np.empty((nqp, 3), np.float32)
        dist = np.empty(nqp, np.float32)
        inv = np.empty(nqp, np.uint8)
        L.orc_recon_grid(h, lat, pos, dist, inv)
        cells_all = np.empty((ncell, 3), np.int32)
        cells_valid = np.empty((nvalid, 3), np.int32)
        L.orc_recon_cells(h, cells_all, cells_valid)
        vkeys = np.empty((nv, 4), np.int32)
        vpos = np.empty((nv, 3), np.float32)
        faces = np.empty((nf, 3), np.int32)
        L.orc_recon_mesh(h, vkeys, vpos, faces)
    finally:
        L.orc_recon_destroy(h)
    return dict(voxelsize=float(f[0]), cells_all=cells_all, cells_valid=cells_valid,
                qp_lattice=lat, qp_pos=pos, qp_dist=dist, qp_invalid=inv,
                vkeys=vkeys, vpos=vpos, faces=faces, planar_moved=0)


def lbvh_knn_normals(surface, kn, flip=(1e6, 1e6, 1e6)):
    """The plane fit of lvr2's LBVH comparator, LBVHIndex::knn_normals
    (src/liblvr2/reconstruction/cuda/lbvh/knn_normals_kernel.cu:54-206), over
    the canonical kNN(kn) of every point (ascending (d2, index))."""
    idx, _, cnt = surface.knn(surface.points, kn)
    return lbvh_fit_lists(surface.points, surface.points, idx, cnt, flip)


def lbvh_fit_lists(points, queries, idx, cnt, flip=(1e6, 1e6, 1e6)):
    """LBVHIndex::calculate_normals (lbvh/normals_kernel.cu:11-180) and the
    fit of knn_normals: for each query, neighbours idx[i, 1:cnt[i]] (slot 0,
    the query itself, is left out); FP64 centroid and covariance with each
    term divided by n - 1 before it is added, the det^2-weighted, sign-aligned
    sum of the three cofactor axes, normalised, flipped toward `flip`; fewer
    than 3 neighbours or a NaN / infinite flip product give the zero normal.
    numpy float64 rounds every operation on its own, in the kernel's order."""
    P = np.asarray(points, np.float32).astype(np.float64)
    Qp = np.asarray(queries, np.float32).astype(np.float64).reshape(-1, 3)
    idx = np.asarray(idx).astype(np.int64).reshape(len(Qp), -1)
    kn = idx.shape[1]
    m = len(Qp)
    n = np.asarray(cnt).astype(np.int64).reshape(m)
    nf = n.astype(np.float64) - 1.0
    ok = n >= 3
    sx = np.zeros(m); sy = np.zeros(m); sz = np.zeros(m)
    with np.errstate(divide="ignore", invalid="ignore"):
        for j in range(1, kn):
            r = ok & (j < n)
            p = P[idx[r, j]]
            sx[r] = sx[r] + p[:, 0] / nf[r]
            sy[r] = sy[r] + p[:, 1] / nf[r]
            sz[r] = sz[r] + p[:, 2] / nf[r]
        xx = np.zeros(m); xy = np.zeros(m); xz = np.zeros(m); yy = np.zeros(m); yz = np.zeros(m); zz = np.zeros(m)
        for j in range(1, kn):
            r = ok & (j < n)
            p = P[idx[r, j]]
            rx, ry, rz = p[:, 0] - sx[r], p[:, 1] - sy[r], p[:, 2] - sz[r]
            f = nf[r]
            xx[r] = xx[r] + rx * rx / f
            xy[r] = xy[r] + rx * ry / f
            xz[r] = xz[r] + rx * rz / f
            yy[r] = yy[r] + ry * ry / f
            yz[r] = yz[r] + ry * rz / f
            zz[r] = zz[r] + rz * rz / f
        w = np.zeros((m, 3))

        def add_axis(ax, ay, az, det):
            wt = det * det
            dot = (w[:, 0] * ax + w[:, 1] * ay) + w[:, 2] * az
            wt = np.where(dot < 0.0, -wt, wt)
            w[:, 0] = w[:, 0] + ax * wt
            w[:, 1] = w[:, 1] + ay * wt
            w[:, 2] = w[:, 2] + az * wt

        det_x = yy * zz - yz * yz
        add_axis(det_x, xz * yz - xy * zz, xy * yz - xz * yy, det_x)
        det_y = xx * zz - xz * xz
        add_axis(xz * yz - xy * zz, det_y, xy * xz - yz * xx, det_y)
        det_z = xx * yy - xy * xy
        add_axis(xy * yz - xz * yy, xy * xz - yz * xx, det_z, det_z)
        mag = np.sqrt((w[:, 0] * w[:, 0] + w[:, 1] * w[:, 1]) + w[:, 2] * w[:, 2])
        w = w / mag[:, None]
        fl = np.asarray(flip, np.float32).astype(np.float64)
        d = fl[None, :] - Qp
        scalar = (d[:, 0] * w[:, 0] + d[:, 1] * w[:, 1]) + d[:, 2] * w[:, 2]
    bad = ~np.isfinite(scalar)
    w[bad] = 0.0
    w[scalar < 0] = -w[scalar < 0]
    w[~ok] = 0.0
    return w.astype(np.float32)


def _normalize(v):
    """BaseVector::normalize (include/lvr2/geometry/BaseVector.hpp:130-143):
    divide by sqrt(x*x + y*y + z*z) unless the vector is zero; float32."""
    v = np.array(v, np.float32, copy=True)
    x, y, z = v[:, 0], v[:, 1], v[:, 2]
    nz = ~((x == 0) & (y == 0) & (z == 0))
    ln = np.sqrt((x * x + y * y) + z * z)
    v[nz] = v[nz] / ln[nz, None]
    return v


def face_normals(vpos, faces):
    """calcFaceNormals / getFaceNormal (include/lvr2/algorithm/NormalAlgorithms.tcc:45-72):
    normalize((v1 - v2) x (v1 - v3)), (0, 0, 1) when its length2 is zero."""
    V = np.asarray(vpos, np.float32)
    F = np.asarray(faces, np.int64)
    if len(F) == 0:
        return np.zeros((0, 3), np.float32)
    v1, v2, v3 = V[F[:, 0]], V[F[:, 1]], V[F[:, 2]]
    a, b = v1 - v2, v1 - v3
    c = np.stack([a[:, 1] * b[:, 2] - a[:, 2] * b[:, 1],
                  a[:, 2] * b[:, 0] - a[:, 0] * b[:, 2],
                  a[:, 0] * b[:, 1] - a[:, 1] * b[:, 0]], 1).astype(np.float32)
    l2 = (c[:, 0] * c[:, 0] + c[:, 1] * c[:, 1]) + c[:, 2] * c[:, 2]
    c[l2 == 0] = np.array([0, 0, 1], np.float32)
    return _normalize(c)


def vertex_normals(vpos, faces, point_normals, surface):
    """calcVertexNormals(mesh, faceNormals, surface)
    (include/lvr2/algorithm/NormalAlgorithms.tcc:74-152): the normalised sum of
    each vertex's face normals, summed in ascending face order; the nearest
    point's normal (kSearch k = 1, canonical (d2, index) ties) where there
    are no faces or the sum is zero.  surface: an OracleSurface of the points
    whose normals are point_normals.  Returns (normals, fallback count)."""
    V = np.asarray(vpos, np.float32)
    F = np.asarray(faces, np.int64).reshape(-1, 3)
    fn = face_normals(V, F)
    acc = np.zeros((len(V), 3), np.float32)
    ref = F.reshape(-1)
    order = np.argsort(ref, kind="stable")  # each vertex's references, ascending face
    vk = ref[order]
    start = np.ones(len(vk), bool)
    start[1:] = vk[1:] != vk[:-1]
    run = np.cumsum(start) - 1
    first = np.flatnonzero(start)
    rank = np.arange(len(vk)) - first[run]
    for t in range(int(rank.max()) + 1 if len(rank) else 0):
        m = rank == t  # one addition per vertex per pass, in face order
        acc[vk[m]] = acc[vk[m]] + fn[order[m] // 3]
    l2 = (acc[:, 0] * acc[:, 0] + acc[:, 1] * acc[:, 1]) + acc[:, 2] * acc[:, 2]
    out = _normalize(acc)
    fb = np.flatnonzero(l2 == 0)
    if len(fb):
        idx, _, cnt = surface.knn(V[fb], 1)
        ok = cnt > 0
        out[fb[ok]] = _normalize(np.asarray(point_normals, np.float32)[idx[ok, 0].astype(np.int64)])
    return out, len(fb)


def vertex_colors(vpos, point_colors, surface):
    """calcColorFromPointCloud (include/lvr2/algorithm/ColorAlgorithms.tcc:43-92):
    the colour of each vertex's nearest point (k = 1; r / 1 casts back to the
    same byte)."""
    V = np.asarray(vpos, np.float32)
    c = np.asarray(point_colors, np.uint8)
    c = c.reshape(len(c), -1)
    idx, _, cnt = surface.knn(V, 1)
    out = c[idx[:, 0].astype(np.int64)].copy()
    out[cnt <= 0] = 0
    return out


def ransac_draws(m):
    """calcPlaneRANSAC's draw sequence for m neighbours
    (AdaptiveKSearchSurface.tcc:715-753), replayed with libstdc++: (10, 53)
    uint32, per iteration 3 plane ranks in set order, then min(50, m)
    scoring ranks."""
    out = np.zeros((10, 53), np.uint32)
    if lib().orc_ransac_draws(int(m), out) != 0:
        raise ValueError("no three distinct plane draws for m = %d" % m)
    return out


def pose_flip_targets(points, poses):
    """Per-point flip points of the scan-pose flip
    (include/lvr2/reconstruction/AdaptiveKSearchSurface.tcc:252-265): the cloud
    point whose input index is the nearest pose's index (lvr2 indexes m_points
    with the pose index); nearest = smallest (float d2, pose index); NaN rows
    where that index is not a point."""
    P = np.asarray(points, np.float32)
    Q = np.asarray(poses, np.float32).reshape(-1, 3)
    best = np.full(len(P), np.inf, np.float32)
    arg = np.zeros(len(P), np.int64)
    for j, p in enumerate(Q):
        d = P - p
        d2 = (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]
        better = d2 < best
        best[better] = d2[better]
        arg[better] = j
    out = np.full((len(P), 3), np.nan, np.float32)
    ok = arg < len(P)
    out[ok] = P[arg[ok]]
    return out


def halfedges(faces, nv):
    """Half-edge connectivity in pmp::SurfaceMesh's layout with the canonical
    choices of the GPU builder (lvr2_gb300/csrc/meshops.cu): edges in the order
    pmp's add_face (src/liblvr2/geometry/pmp/SurfaceMesh.cpp:283-460) creates
    them over faces 0..F-1, halfedge 2e along the first appearance, face
    halfedge = corner 2 -> corner 0, boundary halfedges linked to the boundary
    halfedge leaving their end vertex (paired in ascending order at vertices
    with several gaps), vertex halfedge = smallest outgoing boundary halfedge,
    else smallest outgoing halfedge.  Returns a dict (complex_edges > 0: no
    arrays)."""
    NONE = np.uint32(0xFFFFFFFF)
    F = np.asarray(faces, np.int64).reshape(-1, 3)
    nf = len(F)
    m = 3 * nf
    a = F.reshape(-1)
    b = F[:, [1, 2, 0]].reshape(-1)
    key = (np.minimum(a, b) << 32) | np.maximum(a, b)
    order = np.argsort(key, kind="stable")
    ks = key[order]
    head = np.ones(m, bool)
    head[1:] = ks[1:] != ks[:-1]
    run = np.cumsum(head) - 1
    starts = np.flatnonzero(head)
    ne = len(starts)
    counts = np.diff(np.r_[starts, m])
    first = order[starts]
    edge_of_run = np.empty(ne, np.int64)
    edge_of_run[np.argsort(first, kind="stable")] = np.arange(ne)
    second = order[np.minimum(starts + 1, m - 1)]
    complex_ = (counts > 2) | (a[first] == b[first]) | ((counts == 2) & (a[second] == a[first]))
    out = dict(vertices=int(nv), faces=nf, edges=ne, complex_edges=int(complex_.sum()))
    if out["complex_edges"]:
        return out
    r = order
    rr = run
    e = edge_of_run[rr]
    he_of_ref = np.empty(m, np.int64)
    he_of_ref[r] = 2 * e + (a[r] != a[first[rr]])
    he_vertex = np.empty(2 * ne, np.int64)
    e_of_first = edge_of_run
    he_vertex[2 * e_of_first] = b[first]
    he_vertex[2 * e_of_first + 1] = a[first]
    he_face = np.full(2 * ne, 0xFFFFFFFF, np.int64)
    he_face[he_of_ref] = np.arange(m) // 3
    he_next = np.full(2 * ne, 0xFFFFFFFF, np.int64)
    hr = he_of_ref.reshape(-1, 3)
    he_next[hr[:, 0]] = hr[:, 1]
    he_next[hr[:, 1]] = hr[:, 2]
    he_next[hr[:, 2]] = hr[:, 0]
    face_he = hr[:, 2].copy()
    bnd = np.sort(2 * edge_of_run[counts == 1] + 1)
    frm = he_vertex[bnd ^ 1]
    to = he_vertex[bnd]
    out_sorted = bnd[np.argsort(frm, kind="stable")]
    in_sorted = bnd[np.argsort(to, kind="stable")]
    fs, ts = frm[np.argsort(frm, kind="stable")], to[np.argsort(to, kind="stable")]
    out_count = np.bincount(frm, minlength=nv)
    out_start = np.searchsorted(fs, np.arange(nv))
    in_start = np.searchsorted(ts, np.arange(nv))
    rank = np.arange(len(in_sorted)) - in_start[ts]
    he_next[in_sorted] = out_sorted[out_start[ts] + rank]
    he_prev = np.full(2 * ne, 0xFFFFFFFF, np.int64)
    he_prev[he_next] = np.arange(2 * ne)
    vmin_all = np.full(nv, 0xFFFFFFFF, np.int64)
    np.minimum.at(vmin_all, he_vertex[np.arange(2 * ne) ^ 1], np.arange(2 * ne))
    vmin_b = np.full(nv, 0xFFFFFFFF, np.int64)
    isb = he_face == 0xFFFFFFFF
    np.minimum.at(vmin_b, he_vertex[np.flatnonzero(isb) ^ 1], np.flatnonzero(isb))
    vertex_he = np.where(vmin_b != 0xFFFFFFFF, vmin_b, vmin_all)
    out.update(he_vertex=he_vertex.astype(np.uint32), he_next=he_next.astype(np.uint32),
               he_prev=he_prev.astype(np.uint32), he_face=he_face.astype(np.uint32),
               vertex_he=vertex_he.astype(np.uint32), face_he=face_he.astype(np.uint32),
               boundary_halfedges=len(bnd), complex_vertices=int((out_count > 1).sum()))
    return out


def reconstruct_cells(centers, tsdf, voxelsize, chunk_offsets=None, inner_boxes=None, decomposition="MC"):
    """HashGrid(chunks, innerBoxes, bb, voxelsize) over stored chunk cells,
    then marching cubes (oracle/lvr_oracle.cpp orc_reconstruct_cells).
    Returns a dict like OracleSurface.reconstruct."""
    c = np.ascontiguousarray(centers, np.float32).reshape(-1, 3)
    t = np.ascontiguousarray(tsdf, np.float32).reshape(-1, 8)
    off = np.array([0, len(c)], np.int64) if chunk_offsets is None else np.ascontiguousarray(chunk_offsets, np.int64)
    box = None if inner_boxes is None else np.ascontiguousarray(inner_boxes, np.float32).reshape(-1, 6)
    L = lib()
    h = L.orc_reconstruct_cells(c.reshape(-1), t.reshape(-1), len(c), off, len(off) - 1,
                                None if box is None else box.ctypes.data_as(ctypes.c_void_p), float(voxelsize),
                                {"MC": 0, "PMC": 1}[decomposition])
    return _recon_result(h)


def mc_table():
    out = np.empty((256, 13), np.int32)
    lib().orc_mc_table(out)
    return out


def reference_tables():
    """Tables printed by oracle/_ref/ref_tables (compiled from the lvr2 headers),
    or None when that binary has not been built (no lvr2 tree present)."""
    import json
    exe = HERE / "_ref" / "ref_tables"
    if not exe.exists():
        return None
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True)
    return json.loads(out.stdout)
