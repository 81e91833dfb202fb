"""Python mirror of the lvr2 surface interface over liblvrgb.so.

`Surface` follows AdaptiveKSearchSurface / PointsetSurface
(include/lvr2/reconstruction/AdaptiveKSearchSurface.hpp:99-107,
PointsetSurface.hpp:61-166) and CudaSurface
(include/lvr2/reconstruction/cuda/CudaSurface.hpp:70-158): same parameter
names and defaults, same call order (construct, setKn/Ki/Kd, setFlipPoint,
calculateSurfaceNormals, distance, reconstruction).  Arrays are numpy
float32 (N, 3) on the host, or torch CUDA tensors (device path, pointers are
passed straight to the library).
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import GridConfig, HalfedgeInfo, LvrgbError, MeshInfo, SurfaceConfig, check


def _is_torch_cuda(a):
    return type(a).__module__.startswith("torch") and getattr(a, "is_cuda", False)


def _ptr(a):
    if a is None:
        return None
    if _is_torch_cuda(a):
        return ctypes.c_void_p(a.data_ptr())
    return a.ctypes.data_as(ctypes.c_void_p)


def _f32x3(a):
    if _is_torch_cuda(a):
        if a.dtype != __import__("torch").float32 or not a.is_contiguous() or a.dim() != 2 or a.shape[1] != 3:
            raise ValueError("device points must be a contiguous float32 (N, 3) CUDA tensor")
        return a, 1
    arr = np.ascontiguousarray(a, dtype=np.float32)
    if arr.ndim != 2 or arr.shape[1] != 3:
        arr = arr.reshape(-1, 3)
    return arr, 0


def _host_out(buf, shape, dtype):
    """A host array of `shape`: the leading rows of `buf` when given (it must
    be C-contiguous with enough rows), else a new array."""
    if buf is None:
        return np.empty(shape, dtype)
    a = np.asarray(buf)
    if a.dtype != dtype or not a.flags["C_CONTIGUOUS"] or a.shape[1:] != tuple(shape[1:]) or a.shape[0] < shape[0]:
        raise ValueError("output buffer must be a C-contiguous %s array with at least %s rows" % (dtype, shape[0]))
    return a[:shape[0]]


def _stream_ptr(stream):
    if stream is None:
        return None
    if hasattr(stream, "cuda_stream"):
        return ctypes.c_void_p(stream.cuda_stream)
    return ctypes.c_void_p(int(stream))


class Surface:
    """A point cloud on the GPU with its LBVH, normals and signed distance.

    Surface(points, kn=10, ki=10, kd=5, nem=0, flip_point=(0,0,0)) matches the
    way lvr2_reconstruct sets up AdaptiveKSearchSurface (Main.cpp:283-349);
    flip_point=None keeps AdaptiveKSearchSurface's own default, the bounding
    box centroid.
    """

    def __init__(self, points, kn=10, ki=10, kd=5, nem=0, adaptive=True, flip_point=(0.0, 0.0, 0.0),
                 bucket=32, gap_threshold=1e-3, device=0, stream=None, seed_radius=1):
        L = _lib.load()
        cfg = SurfaceConfig()
        L.lvrgb_surface_config_default(ctypes.byref(cfg))
        cfg.kn, cfg.ki, cfg.kd, cfg.nem = int(kn), int(ki), int(kd), int(nem)
        cfg.adaptive = int(bool(adaptive))
        if flip_point is None:
            cfg.flip_set = 0
        else:
            cfg.flip_set = 1
            cfg.flip[0], cfg.flip[1], cfg.flip[2] = (float(v) for v in flip_point)
        cfg.bucket = int(bucket)
        cfg.gap_threshold = float(gap_threshold)
        cfg.device = int(device)
        cfg.seed_radius = int(seed_radius)
        pts, on_dev = _f32x3(points)
        self._h = ctypes.c_void_p()
        self._stream = _stream_ptr(stream)
        check(L.lvrgb_surface_create(ctypes.byref(cfg), _ptr(pts), len(pts), on_dev, self._stream,
                                     ctypes.byref(self._h)))
        self.n = int(len(pts))
        self.kn, self.ki, self.kd = int(kn), int(ki), int(kd)

    def close(self):
        if getattr(self, "_h", None):
            _lib.load().lvrgb_surface_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_points(self, points):
        """Replaces the points (rebuilds the LBVH in the handle's memory)."""
        pts, on_dev = _f32x3(points)
        check(_lib.load().lvrgb_surface_set_points(self._h, _ptr(pts), len(pts), on_dev, self._stream))
        self.n = int(len(pts))

    def timings(self):
        """Device ms of the last calls: build, normals, interpolation, grid,
        signed distance, culling, marching cubes, PMC planar post-pass."""
        out = np.zeros(8, np.float32)
        check(_lib.load().lvrgb_surface_timings(self._h, _ptr(out)))
        return out

    # ---- parameters (PointsetSurface::setKn/setKi/setKd/setFlipPoint) ------
    def set_k(self, kn=-1, ki=-1, kd=-1):
        check(_lib.load().lvrgb_surface_set_k(self._h, kn, ki, kd))
        if kn > 0:
            self.kn = kn
        if ki >= 0:
            self.ki = ki
        if kd > 0:
            self.kd = kd

    def set_flip_point(self, x, y, z):
        check(_lib.load().lvrgb_surface_set_flip_point(self._h, x, y, z))

    def set_scan_poses(self, poses):
        """AdaptiveKSearchSurface's scan poses: (np, 3), or None to remove."""
        p = np.zeros((0, 3), np.float32) if poses is None else np.ascontiguousarray(poses, np.float32).reshape(-1, 3)
        check(_lib.load().lvrgb_surface_set_scan_poses(self._h, _ptr(p), len(p)))

    def set_method(self, nem):
        check(_lib.load().lvrgb_surface_set_method(self._h, nem))

    def bounding_box(self):
        out = np.zeros(9, np.float32)
        check(_lib.load().lvrgb_surface_bounding_box(self._h, _ptr(out)))
        return out[:3], out[3:6], out[6:]

    # ---- normals -------------------------------------------------------------
    def calculate_normals(self):
        check(_lib.load().lvrgb_calculate_normals(self._h, self._stream))

    def interpolate_normals(self):
        check(_lib.load().lvrgb_interpolate_normals(self._h, self._stream))

    def normals(self, out=None):
        """Final normals (n, 3) in input order.  out: a CUDA tensor, or a
        C-contiguous float32 host array (e.g. over pinned memory) to fill."""
        if out is not None and _is_torch_cuda(out):
            check(_lib.load().lvrgb_get_normals(self._h, _ptr(out), 1, self._stream))
            return out
        res = _host_out(out, (self.n, 3), np.float32)
        check(_lib.load().lvrgb_get_normals(self._h, _ptr(res), 0, self._stream))
        return res

    def normals_async(self, out, copy_stream):
        """Starts the copy of the final normals into `out` (a C-contiguous
        float32 (n, 3) host array, best over pinned memory) on copy_stream (a
        torch.cuda.Stream or a raw stream handle), ordered after the work
        issued so far and overlapping what comes next.  Synchronize
        copy_stream before reading `out`; do not change the points or normals
        until then."""
        arr = np.asarray(out)
        if arr.dtype != np.float32 or arr.shape != (self.n, 3) or not arr.flags["C_CONTIGUOUS"]:
            raise ValueError("out must be a C-contiguous float32 (%d, 3) array" % self.n)
        cs = getattr(copy_stream, "cuda_stream", copy_stream)
        check(_lib.load().lvrgb_get_normals_async(self._h, _ptr(arr), self._stream, ctypes.c_void_p(cs)))
        return arr

    def distance_stats(self):
        """Counters of the last reconstruct's signed-distance searches:
        buckets scanned, nodes expanded, heap insertions, candidate chunks,
        warp insertion rounds (sums; 8 entries)."""
        out = np.zeros(8, np.uint64)
        check(_lib.load().lvrgb_distance_stats(self._h, _ptr(out)))
        return out

    def raw_normals(self):
        res = np.empty((self.n, 3), np.float32)
        k = np.empty(self.n, np.int32)
        check(_lib.load().lvrgb_get_raw_normals(self._h, _ptr(res), _ptr(k), 0, self._stream))
        return res, k

    def set_normals(self, normals):
        arr, on_dev = _f32x3(normals)
        check(_lib.load().lvrgb_set_normals(self._h, _ptr(arr), on_dev, self._stream))

    def normal_stats(self):
        out = np.zeros(16, np.uint32)
        check(_lib.load().lvrgb_normal_stats(self._h, _ptr(out)))
        return out

    # ---- queries -------------------------------------------------------------
    def knn(self, queries, k):
        q, on_dev = _f32x3(queries)
        if on_dev:
            import torch
            idx = torch.empty((len(q), k), dtype=torch.int32, device=q.device)
            dist = torch.empty((len(q), k), dtype=torch.float32, device=q.device)
            cnt = torch.empty(len(q), dtype=torch.int32, device=q.device)
        else:
            idx = np.empty((len(q), k), np.uint32)
            dist = np.empty((len(q), k), np.float32)
            cnt = np.empty(len(q), np.int32)
        check(_lib.load().lvrgb_knn(self._h, _ptr(q), len(q), int(k), _ptr(idx), _ptr(dist), _ptr(cnt), on_dev,
                                    self._stream))
        return idx, dist, cnt

    def normals_from_neighbors(self, queries, n_neighbors, indices):
        """LBVHIndex::calculate_normals: the nem 4 fit of given neighbour lists
        (indices (nq, k) of this surface's points, n_neighbors (nq,))."""
        q = np.ascontiguousarray(queries, np.float32).reshape(-1, 3)
        idx = np.ascontiguousarray(indices, np.uint32).reshape(len(q), -1)
        cnt = np.ascontiguousarray(n_neighbors, np.uint32).reshape(len(q))
        out = np.empty((len(q), 3), np.float32)
        check(_lib.load().lvrgb_normals_from_neighbors(self._h, _ptr(q), len(q), idx.shape[1], _ptr(cnt), _ptr(idx),
                                                       _ptr(out), 0, self._stream))
        return out

    def radius_search(self, queries, k, radius):
        """SearchTree::radiusSearch: up to k nearest points with distance
        below radius (host arrays): idx, dist (padded), count."""
        q, on_dev = _f32x3(queries)
        if on_dev:
            raise ValueError("use host arrays with radius_search()")
        idx = np.empty((len(q), k), np.uint32)
        dist = np.empty((len(q), k), np.float32)
        cnt = np.empty(len(q), np.int32)
        check(_lib.load().lvrgb_radius_search(self._h, _ptr(q), len(q), int(k), float(radius), _ptr(idx), _ptr(dist),
                                              _ptr(cnt), 0, self._stream))
        return idx, dist, cnt

    def distance(self, queries):
        q, on_dev = _f32x3(queries)
        proj = np.empty(len(q), np.float32)
        eucl = np.empty(len(q), np.float32)
        if on_dev:
            raise ValueError("use host arrays with distance()")
        check(_lib.load().lvrgb_distance(self._h, _ptr(q), len(q), _ptr(proj), _ptr(eucl), 0, self._stream))
        return proj, eucl

    def distance_adjoint(self, queries, grad_projected=None, grad_euclidean=None, want_points=True,
                         want_normals=True):
        """Reverse mode of distance(): returns (projected, euclidean, grad_q,
        grad_points, grad_normals) for upstream gradients of the projected
        and Euclidean distances (None = 0).  Host numpy arrays or CUDA
        tensors (all outputs then on the device)."""
        q, on_dev = _f32x3(queries)
        nq = len(q)
        n = self.n
        if on_dev:
            import torch
            dev = q.device

            def empty(*shape):
                return torch.empty(shape, dtype=torch.float32, device=dev)

            def vec(a):
                return None if a is None else a.to(device=dev, dtype=torch.float32).contiguous()
        else:
            def empty(*shape):
                return np.empty(shape, np.float32)

            def vec(a):
                return None if a is None else np.ascontiguousarray(a, dtype=np.float32)
        gd, ge = vec(grad_projected), vec(grad_euclidean)
        proj, eucl, gq = empty(nq), empty(nq), empty(nq, 3)
        gp = empty(n, 3) if want_points else None
        gn = empty(n, 3) if want_normals else None
        check(_lib.load().lvrgb_distance_adjoint(self._h, _ptr(q), nq, _ptr(gd), _ptr(ge), _ptr(proj), _ptr(eucl),
                                                 _ptr(gq), _ptr(gp), _ptr(gn), on_dev, self._stream))
        return proj, eucl, gq, gp, gn

    def project_to_surface(self, positions, steps=3):
        """Newton steps x <- x - d(x) n(x) onto the zero level; returns
        (positions, unit normals)."""
        v, on_dev = _f32x3(positions)
        if on_dev:
            import torch
            pos = torch.empty_like(v)
            nrm = torch.empty_like(v)
        else:
            pos = np.empty_like(v)
            nrm = np.empty_like(v)
        check(_lib.load().lvrgb_project_to_surface(self._h, _ptr(v), len(v), int(steps), _ptr(pos), _ptr(nrm), on_dev,
                                                   self._stream))
        return pos, nrm

    def grid_distances(self, queries, voxel_size):
        q, on_dev = _f32x3(queries)
        if on_dev:
            raise ValueError("use host arrays with grid_distances()")
        dist = np.empty(len(q), np.float32)
        inv = np.empty(len(q), np.uint8)
        check(_lib.load().lvrgb_grid_distances(self._h, _ptr(q), len(q), float(voxel_size), _ptr(dist), _ptr(inv),
                                               0, self._stream))
        return dist, inv

    def interpolated_normal(self, queries):
        """PointsetSurface::getInterpolatedNormal at each query: ((0, 1, 0) +
        the ki nearest normals, each normalised) / ki, not normalised (as
        lvr2 returns it)."""
        q, on_dev = _f32x3(queries)
        if on_dev:
            raise ValueError("use host arrays with interpolated_normal()")
        out = np.empty((len(q), 3), np.float32)
        check(_lib.load().lvrgb_interpolated_normal(self._h, _ptr(q), len(q), _ptr(out), 0, self._stream))
        return out

    # ---- grid + marching cubes ---------------------------------------------------
    def reconstruct(self, voxelsize=10.0, intersections=-1, extrude=True, decomposition="PMC"):
        g = GridConfig()
        if intersections is not None and intersections > 0:
            g.resolution, g.is_voxelsize = float(intersections), 0
        else:
            g.resolution, g.is_voxelsize = float(voxelsize), 1
        g.extrude = int(bool(extrude))
        g.decomposition = {"MC": 0, "PMC": 1}[decomposition]
        info = MeshInfo()
        check(_lib.load().lvrgb_reconstruct(self._h, ctypes.byref(g), ctypes.byref(info), self._stream))
        self.info = info
        return info

    def optimize_planar_faces(self, kc=5):
        """BilinearFastBox::optimizePlanarFaces on the last mesh (in place);
        returns the number of moved vertices."""
        moved = ctypes.c_int64(0)
        check(_lib.load().lvrgb_optimize_planar_faces(self._h, int(kc), ctypes.byref(moved), self._stream))
        return int(moved.value)

    def _mesh_info(self):
        """Counts of the last reconstruction (zeros before the first: the
        library then reports the missing mesh)."""
        return getattr(self, "info", None) or MeshInfo()

    def vertex_normals(self, vertices=None, faces=None):
        """calcVertexNormals: per-vertex normals (V, 3) of the last mesh, or of
        the mesh given as vertices (V, 3) and faces (F, 3) against this
        surface's points and normals.  For a given mesh also returns the number
        of vertices that took their nearest point's normal."""
        L = _lib.load()
        if vertices is None:
            out = np.empty((self._mesh_info().vertices, 3), np.float32)
            check(L.lvrgb_mesh_vertex_normals(self._h, _ptr(out), 0, self._stream))
            return out
        v = np.ascontiguousarray(vertices, np.float32).reshape(-1, 3)
        f = np.ascontiguousarray(faces, np.uint32).reshape(-1, 3)
        out = np.empty((len(v), 3), np.float32)
        cnt = ctypes.c_int64(0)
        check(L.lvrgb_vertex_normals(self._h, _ptr(v), len(v), _ptr(f), len(f), _ptr(out), ctypes.byref(cnt), 0,
                                     self._stream))
        return out, int(cnt.value)

    def reconstruct_cells(self, centers, tsdf, voxelsize, chunk_offsets=None, inner_boxes=None, decomposition="MC"):
        """HashGrid(chunks, innerBoxes, bb, voxelsize) + marching cubes over
        stored chunk cells (centres (n, 3), corner distances (n, 8));
        chunk_offsets (nchunks + 1) and inner_boxes (nchunks, 6) optional.
        The mesh replaces this surface's last mesh."""
        c = np.ascontiguousarray(centers, np.float32).reshape(-1, 3)
        t = np.ascontiguousarray(tsdf, np.float32).reshape(-1, 8)
        if len(c) != len(t):
            raise ValueError("centers and tsdf differ in length")
        off = None if chunk_offsets is None else np.ascontiguousarray(chunk_offsets, np.int64)
        box = None if inner_boxes is None else np.ascontiguousarray(inner_boxes, np.float32).reshape(-1, 6)
        nch = 0 if off is None else len(off) - 1
        info = MeshInfo()
        dec = {"MC": 0, "PMC": 1}[decomposition]
        check(_lib.load().lvrgb_reconstruct_cells(self._h, float(voxelsize), dec, _ptr(c), _ptr(t), len(c), _ptr(off),
                                                  nch, _ptr(box), ctypes.byref(info), 0, self._stream))
        self.info = info
        return info

    def halfedges(self, faces=None, nverts=None):
        """Half-edge connectivity (pmp::SurfaceMesh layout) of the last mesh,
        or of the triangles faces (F, 3) over nverts vertices: dict of
        he_vertex, he_next, he_prev, he_face (2E), vertex_he (V), face_he (F)
        and the counts."""
        L = _lib.load()
        if faces is None:
            def call(info, *arrs):
                return L.lvrgb_mesh_halfedges(self._h, ctypes.byref(info), *arrs, 0, self._stream)
        else:
            f = np.ascontiguousarray(faces, np.uint32).reshape(-1, 3)
            if nverts is None:
                nverts = int(f.max()) + 1 if len(f) else 0

            def call(info, *arrs):
                return L.lvrgb_halfedges(self._h, _ptr(f), len(f), int(nverts), ctypes.byref(info), *arrs, 0,
                                         self._stream)
        info = HalfedgeInfo()
        check(call(info, None, None, None, None, None, None))
        nh = 2 * info.edges
        arrs = {k: np.empty(n, np.uint32) for k, n in (("he_vertex", nh), ("he_next", nh), ("he_prev", nh),
                                                       ("he_face", nh), ("vertex_he", info.vertices),
                                                       ("face_he", info.faces))}
        check(call(info, *(_ptr(arrs[k]) for k in ("he_vertex", "he_next", "he_prev", "he_face", "vertex_he",
                                                    "face_he"))))
        arrs.update(edges=info.edges, boundary_halfedges=info.boundary_halfedges,
                    complex_edges=info.complex_edges, complex_vertices=info.complex_vertices)
        return arrs

    def cell_tsdf(self):
        """HashGrid::toPointBuffer of the culled grid: cell centres (C, 3) and
        the distances at their 8 corners (C, 8), cells in lattice-key order."""
        n = self._mesh_info().cells_valid
        c = np.empty((n, 3), np.float32)
        t = np.empty((n, 8), np.float32)
        check(_lib.load().lvrgb_get_cell_tsdf(self._h, _ptr(c), _ptr(t), 0, self._stream))
        return c, t

    def vertex_colors(self, point_colors):
        """calcColorFromPointCloud: each vertex of the last mesh takes the
        colour of its nearest point.  point_colors: (n, width) uint8 in input
        order; returns (V, width) uint8."""
        c = np.ascontiguousarray(point_colors, np.uint8)
        c = c.reshape(len(c), -1)
        if len(c) != self.n:
            raise ValueError("point_colors has %d rows, the surface %d points" % (len(c), self.n))
        out = np.empty((self._mesh_info().vertices, c.shape[1]), np.uint8)
        check(_lib.load().lvrgb_mesh_vertex_colors(self._h, _ptr(c), c.shape[1], _ptr(out), 0, self._stream))
        return out

    def mesh(self, with_edges=True, out_vertices=None, out_faces=None):
        """The last mesh: vertices (V, 3), faces (F, 3) and, optionally, edge
        keys (V, 4).  out_vertices / out_faces: host arrays (e.g. over pinned
        memory) with at least V / F rows; their leading rows are filled and
        returned."""
        info = self._mesh_info()
        v = _host_out(out_vertices, (info.vertices, 3), np.float32)
        f = _host_out(out_faces, (info.faces, 3), np.uint32)
        e = np.empty((info.vertices, 4), np.int32) if with_edges else None
        check(_lib.load().lvrgb_get_mesh(self._h, _ptr(v), _ptr(f), _ptr(e), 0, self._stream))
        return v, f, e

    def grid(self):
        nq = self.info.grid_vertices
        lat = np.empty((nq, 3), np.int32)
        pos = np.empty((nq, 3), np.float32)
        dist = np.empty(nq, np.float32)
        inv = np.empty(nq, np.uint8)
        check(_lib.load().lvrgb_get_grid(self._h, _ptr(lat), _ptr(pos), _ptr(dist), _ptr(inv), 0, self._stream))
        return lat, pos, dist, inv

    def cells(self):
        a = np.empty((self.info.cells_all, 3), np.int32)
        v = np.empty((self.info.cells_valid, 3), np.int32)
        check(_lib.load().lvrgb_get_cells(self._h, _ptr(a), _ptr(v), 0, self._stream))
        return a, v


class Batch:
    """Normals for every scan of a scan project in one pass (lvrgb_batch_*):
    the per-scan CudaSurface runs of lvr2_cuda_normals' directory mode, with
    kNN restricted to each scan and each scan flipped toward its own point."""

    def __init__(self, scans, flip_points, kn=10, ki=10, nem=3, adaptive=True, bucket=32, seed_radius=1,
                 gap_threshold=1e-3, device=0, stream=None, kd=5):
        L = _lib.load()
        cfg = SurfaceConfig()
        L.lvrgb_surface_config_default(ctypes.byref(cfg))
        cfg.kn, cfg.ki, cfg.kd, cfg.nem = int(kn), int(ki), int(kd), int(nem)
        cfg.adaptive = int(bool(adaptive))
        cfg.bucket, cfg.seed_radius = int(bucket), int(seed_radius)
        cfg.gap_threshold = float(gap_threshold)
        cfg.device = int(device)
        if not isinstance(scans, (list, tuple)):
            raise ValueError("scans must be a list of (n_i, 3) arrays")
        sizes = [len(s) for s in scans]
        if scans and _is_torch_cuda(scans[0]):
            import torch
            pts = torch.cat([s.reshape(-1, 3).float() for s in scans]).contiguous()
            on_dev = 1
        else:
            pts = np.ascontiguousarray(np.concatenate([np.asarray(s, np.float32).reshape(-1, 3) for s in scans]))
            on_dev = 0
        self.offsets = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
        self.flips = np.ascontiguousarray(flip_points, np.float32).reshape(-1, 3)
        self.n = int(self.offsets[-1])
        self._stream = _stream_ptr(stream)
        self._h = ctypes.c_void_p()
        check(L.lvrgb_batch_create(ctypes.byref(cfg), _ptr(pts), _ptr(self.offsets), len(sizes), _ptr(self.flips),
                                   on_dev, self._stream, ctypes.byref(self._h)))

    def close(self):
        if getattr(self, "_h", None):
            _lib.load().lvrgb_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def calculate_normals(self, use_graph=False):
        check(_lib.load().lvrgb_batch_calculate_normals(self._h, int(bool(use_graph)), self._stream))

    def normals(self):
        out = np.empty((self.n, 3), np.float32)
        check(_lib.load().lvrgb_batch_get_normals(self._h, _ptr(out), 0, self._stream))
        return out

    def grid_distances(self, queries, voxel_size):
        """Signed distance and invalid flag of every scan's (chunk's) grid
        vertices against that scan: `queries` is a list of (m_i, 3) arrays,
        one per scan.  Returns (distance, invalid) concatenated."""
        sizes = [len(q) for q in queries]
        q = np.ascontiguousarray(np.concatenate([np.asarray(x, np.float32).reshape(-1, 3) for x in queries]))
        off = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
        dist = np.empty(len(q), np.float32)
        inv = np.empty(len(q), np.uint8)
        check(_lib.load().lvrgb_batch_grid_distances(self._h, _ptr(q), _ptr(off), float(voxel_size), _ptr(dist),
                                                     _ptr(inv), 0, self._stream))
        return dist, inv

    def autotune(self):
        b = np.zeros(1, np.int32)
        r = np.zeros(1, np.int32)
        check(_lib.load().lvrgb_batch_autotune(self._h, _ptr(b), _ptr(r), self._stream))
        return int(b[0]), int(r[0])

    def stats(self):
        c = np.zeros(16, np.uint32)
        ms = np.zeros(4, np.float32)
        check(_lib.load().lvrgb_batch_stats(self._h, _ptr(c), _ptr(ms)))
        return c, ms

    def tuning(self):
        """(bucket, seed radius, wide tile, wide buffer slack) in use."""
        out = np.zeros(4, np.int32)
        check(_lib.load().lvrgb_batch_tuning(self._h, _ptr(out)))
        return tuple(int(x) for x in out)

    def round_times(self):
        """Device ms of each search round of the last eager run."""
        ms = np.zeros(5, np.float32)
        check(_lib.load().lvrgb_batch_round_times(self._h, _ptr(ms)))
        return ms


def kernel_launches():
    """Kernels launched by liblvrgb.so in this process."""
    out = np.zeros(1, np.uint64)
    check(_lib.load().lvrgb_kernel_launches(_ptr(out)))
    return int(out[0])


__all__ = ["Surface", "Batch", "LvrgbError", "kernel_launches"]
