"""ctypes binding of liblvrgb.so (include/lvrgb.h).

The library is the only compute path: if it is missing or cannot be loaded
every call raises; there is no CPU fallback.
"""
import ctypes
from pathlib import Path

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "liblvrgb.so"

STATUS = {
    0: "LVRGB_OK",
    1: "LVRGB_ERR_INVALID_ARGUMENT",
    2: "LVRGB_ERR_CUDA",
    3: "LVRGB_ERR_OUT_OF_MEMORY",
    4: "LVRGB_ERR_UNSUPPORTED",
    5: "LVRGB_ERR_STATE",
    6: "LVRGB_ERR_KERNEL",
    7: "LVRGB_ERR_TOPOLOGY",
}

# Every function declared in include/lvrgb.h.
EXPORTS = [
    "lvrgb_surface_config_default", "lvrgb_surface_create", "lvrgb_surface_destroy", "lvrgb_surface_set_k",
    "lvrgb_surface_set_flip_point", "lvrgb_surface_set_method", "lvrgb_surface_bounding_box",
    "lvrgb_surface_num_points", "lvrgb_calculate_normals", "lvrgb_get_normals", "lvrgb_get_normals_async", "lvrgb_get_raw_normals", "lvrgb_distance_stats",
    "lvrgb_set_normals", "lvrgb_interpolate_normals", "lvrgb_normal_stats", "lvrgb_knn", "lvrgb_distance",
    "lvrgb_distance_adjoint", "lvrgb_project_to_surface", "lvrgb_grid_distances",
    "lvrgb_interpolated_normal", "lvrgb_reconstruct", "lvrgb_optimize_planar_faces", "lvrgb_mesh_vertex_normals", "lvrgb_vertex_normals", "lvrgb_mesh_vertex_colors", "lvrgb_get_cell_tsdf", "lvrgb_reconstruct_cells", "lvrgb_radius_search", "lvrgb_normals_from_neighbors", "lvrgb_debug_fail_allocation", "lvrgb_debug_round_collapse", "lvrgb_mesh_halfedges", "lvrgb_halfedges", "lvrgb_surface_set_scan_poses", "lvrgb_get_mesh", "lvrgb_get_grid", "lvrgb_get_cells",
    "lvrgb_surface_set_points", "lvrgb_surface_timings", "lvrgb_kernel_launches", "lvrgb_knn_small_noalloc",
    "lvrgb_batch_create", "lvrgb_batch_destroy", "lvrgb_batch_calculate_normals", "lvrgb_batch_get_normals",
    "lvrgb_batch_grid_distances", "lvrgb_batch_autotune", "lvrgb_batch_stats", "lvrgb_batch_round_times", "lvrgb_batch_tuning",
    "lvrgb_last_error", "lvrgb_version",
]


class LvrgbError(RuntimeError):
    def __init__(self, status, message):
        super().__init__("%s: %s" % (STATUS.get(status, str(status)), message))
        self.status = status


class HalfedgeInfo(ctypes.Structure):
    _fields_ = [("vertices", ctypes.c_int64), ("faces", ctypes.c_int64), ("edges", ctypes.c_int64),
                ("boundary_halfedges", ctypes.c_int64), ("complex_edges", ctypes.c_int64),
                ("complex_vertices", ctypes.c_int64)]


class SurfaceConfig(ctypes.Structure):
    _fields_ = [
        ("kn", ctypes.c_int32), ("ki", ctypes.c_int32), ("kd", ctypes.c_int32), ("nem", ctypes.c_int32),
        ("adaptive", ctypes.c_int32), ("flip_set", ctypes.c_int32), ("flip", ctypes.c_float * 3),
        ("bucket", ctypes.c_int32), ("gap_threshold", ctypes.c_float), ("device", ctypes.c_int32),
        ("seed_radius", ctypes.c_int32),
    ]


class GridConfig(ctypes.Structure):
    _fields_ = [("resolution", ctypes.c_float), ("is_voxelsize", ctypes.c_int32), ("extrude", ctypes.c_int32),
                ("decomposition", ctypes.c_int32)]


class MeshInfo(ctypes.Structure):
    _fields_ = [("cells_all", ctypes.c_int64), ("grid_vertices", ctypes.c_int64), ("cells_valid", ctypes.c_int64),
                ("vertices", ctypes.c_int64), ("faces", ctypes.c_int64), ("voxelsize", ctypes.c_float),
                ("stage_ms", ctypes.c_float * 4)]


_lib = None


def load(path=None):
    """Loads liblvrgb.so (raises when it is missing: the GPU path is the product)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError("liblvrgb.so not built: run `python -m lvr2_gb300.build` (%s missing)" % p)
    L = ctypes.CDLL(str(p))
    vp, i32, i64, f32 = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, ctypes.c_float
    S = ctypes.c_int
    L.lvrgb_surface_config_default.argtypes = [ctypes.POINTER(SurfaceConfig)]
    L.lvrgb_surface_config_default.restype = None
    L.lvrgb_surface_create.argtypes = [ctypes.POINTER(SurfaceConfig), vp, i64, i32, vp, ctypes.POINTER(vp)]
    L.lvrgb_surface_destroy.argtypes = [vp]
    L.lvrgb_surface_set_k.argtypes = [vp, i32, i32, i32]
    L.lvrgb_surface_set_flip_point.argtypes = [vp, f32, f32, f32]
    L.lvrgb_surface_set_method.argtypes = [vp, i32]
    L.lvrgb_surface_bounding_box.argtypes = [vp, vp]
    L.lvrgb_surface_num_points.argtypes = [vp, ctypes.POINTER(i64)]
    L.lvrgb_calculate_normals.argtypes = [vp, vp]
    L.lvrgb_get_normals.argtypes = [vp, vp, i32, vp]
    L.lvrgb_get_normals_async.argtypes = [vp, vp, vp, vp]
    L.lvrgb_distance_stats.argtypes = [vp, vp]
    L.lvrgb_get_raw_normals.argtypes = [vp, vp, vp, i32, vp]
    L.lvrgb_set_normals.argtypes = [vp, vp, i32, vp]
    L.lvrgb_interpolate_normals.argtypes = [vp, vp]
    L.lvrgb_normal_stats.argtypes = [vp, vp]
    L.lvrgb_knn.argtypes = [vp, vp, i64, i32, vp, vp, vp, i32, vp]
    L.lvrgb_distance.argtypes = [vp, vp, i64, vp, vp, i32, vp]
    L.lvrgb_distance_adjoint.argtypes = [vp, vp, i64, vp, vp, vp, vp, vp, vp, vp, i32, vp]
    L.lvrgb_project_to_surface.argtypes = [vp, vp, i64, i32, vp, vp, i32, vp]
    L.lvrgb_grid_distances.argtypes = [vp, vp, i64, f32, vp, vp, i32, vp]
    L.lvrgb_interpolated_normal.argtypes = [vp, vp, i64, vp, i32, vp]
    L.lvrgb_reconstruct.argtypes = [vp, ctypes.POINTER(GridConfig), ctypes.POINTER(MeshInfo), vp]
    L.lvrgb_optimize_planar_faces.argtypes = [vp, i32, ctypes.POINTER(i64), vp]
    L.lvrgb_mesh_vertex_normals.argtypes = [vp, vp, i32, vp]
    L.lvrgb_debug_fail_allocation.argtypes = [i64]
    L.lvrgb_debug_round_collapse.argtypes = [i32]
    L.lvrgb_surface_set_scan_poses.argtypes = [vp, vp, i64]
    L.lvrgb_mesh_halfedges.argtypes = [vp, ctypes.POINTER(HalfedgeInfo), vp, vp, vp, vp, vp, vp, i32, vp]
    L.lvrgb_halfedges.argtypes = [vp, vp, i64, i64, ctypes.POINTER(HalfedgeInfo), vp, vp, vp, vp, vp, vp, i32, vp]
    L.lvrgb_normals_from_neighbors.argtypes = [vp, vp, i64, i32, vp, vp, vp, i32, vp]
    L.lvrgb_radius_search.argtypes = [vp, vp, i64, i32, f32, vp, vp, vp, i32, vp]
    L.lvrgb_reconstruct_cells.argtypes = [vp, f32, i32, vp, vp, i64, vp, i32, vp, ctypes.POINTER(MeshInfo), i32,
                                          vp]
    L.lvrgb_get_cell_tsdf.argtypes = [vp, vp, vp, i32, vp]
    L.lvrgb_mesh_vertex_colors.argtypes = [vp, vp, i32, vp, i32, vp]
    L.lvrgb_vertex_normals.argtypes = [vp, vp, i64, vp, i64, vp, vp, i32, vp]
    L.lvrgb_get_mesh.argtypes = [vp, vp, vp, vp, i32, vp]
    L.lvrgb_get_grid.argtypes = [vp, vp, vp, vp, vp, i32, vp]
    L.lvrgb_get_cells.argtypes = [vp, vp, vp, i32, vp]
    L.lvrgb_surface_set_points.argtypes = [vp, vp, i64, i32, vp]
    L.lvrgb_surface_timings.argtypes = [vp, vp]
    L.lvrgb_kernel_launches.argtypes = [vp]
    L.lvrgb_knn_small_noalloc.argtypes = [vp, i64, vp, i64, i32, vp, vp, vp]
    L.lvrgb_batch_create.argtypes = [ctypes.POINTER(SurfaceConfig), vp, vp, i32, vp, i32, vp, ctypes.POINTER(vp)]
    L.lvrgb_batch_destroy.argtypes = [vp]
    L.lvrgb_batch_calculate_normals.argtypes = [vp, i32, vp]
    L.lvrgb_batch_get_normals.argtypes = [vp, vp, i32, vp]
    L.lvrgb_batch_grid_distances.argtypes = [vp, vp, vp, f32, vp, vp, i32, vp]
    L.lvrgb_batch_autotune.argtypes = [vp, vp, vp, vp]
    L.lvrgb_batch_stats.argtypes = [vp, vp, vp]
    L.lvrgb_batch_round_times.argtypes = [vp, vp]
    L.lvrgb_batch_tuning.argtypes = [vp, vp]
    L.lvrgb_last_error.restype = ctypes.c_char_p
    L.lvrgb_version.restype = ctypes.c_char_p
    for name in EXPORTS:
        if name not in ("lvrgb_surface_config_default", "lvrgb_last_error", "lvrgb_version"):
            getattr(L, name).restype = S
    if path is None:
        _lib = L
    return L


def check(status):
    if status != 0:
        raise LvrgbError(status, load().lvrgb_last_error().decode())
