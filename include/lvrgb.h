/*
 * lvrgb.h -- C ABI of liblvrgb.so, the GB300 (sm_103a) implementation of the
 * lvr2 surface-reconstruction hot path: LBVH kNN, point normals, normal
 * interpolation, signed distance at grid vertices and marching cubes.
 *
 * Each entry point replaces one piece of the lvr2 interface; the citation in
 * its comment names the lvr2 declaration (path inside the lvr2 source tree).
 *
 * Conventions
 *  - Point, normal and query arrays are float32 x,y,z triples (AoS), in the
 *    caller's order, like PointBuffer's "points" / "normals" channels.
 *  - on_device = 0: pointers are host memory; the call copies through pinned
 *    staging and returns when the result is in host memory.
 *    on_device = 1: pointers are device memory of the handle's GPU; the call
 *    is asynchronous on `stream` unless stated otherwise.
 *  - stream: a cudaStream_t passed as void* (NULL = legacy default stream).
 *  - No exception crosses the ABI.  Every call returns an lvrgb_status; the
 *    message of the last failure on the calling thread is lvrgb_last_error().
 *  - A handle is not thread-safe: use one handle per host thread (lvr2 calls
 *    PointsetSurface::distance from OpenMP threads; route those through
 *    lvrgb_distance in one batched call instead).
 *  - Neighbour order: k nearest = the k smallest keys (d2, index), where
 *    d2 = fl(fl(fl(dx*dx) + fl(dy*dy)) + fl(dz*dz)), dx = fl(qx - px) in
 *    float32 without fused multiply-add, and index is the point's position in
 *    the input array.  lvr2's kd-tree ranks by double-precision d2 with
 *    traversal-order tie handling; both agree except on float32 near-ties.
 */
#ifndef LVRGB_H
#define LVRGB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum lvrgb_status {
    LVRGB_OK = 0,
    LVRGB_ERR_INVALID_ARGUMENT = 1, /* bad size, pointer, k, voxel size or method */
    LVRGB_ERR_CUDA = 2,             /* a CUDA runtime call failed */
    LVRGB_ERR_OUT_OF_MEMORY = 3,    /* device allocation failed (lvr2 retries smaller chunks) */
    LVRGB_ERR_UNSUPPORTED = 4,      /* e.g. nem 1 (RANSAC) on a scan project */
    LVRGB_ERR_STATE = 5,            /* call order: no normals yet, no mesh yet */
    LVRGB_ERR_KERNEL = 6,           /* a kernel reported an internal limit (traversal depth) */
    LVRGB_ERR_TOPOLOGY = 7          /* complex edges: pmp's add_face would throw TopologyException */
} lvrgb_status;

typedef struct lvrgb_surface_s* lvrgb_surface;

/* Construction parameters of a surface.
 * Replaces AdaptiveKSearchSurface(PointBufferPtr, string searchTreeName,
 * int kn, int ki, int kd, int calcMethod, string posefile)
 * (include/lvr2/reconstruction/AdaptiveKSearchSurface.hpp:99-107) and
 * CudaSurface(floatArr& points, size_t num_points, int device)
 * (include/lvr2/reconstruction/cuda/CudaSurface.hpp:80). */
typedef struct lvrgb_surface_config {
    int32_t kn;            /* normal estimation neighbourhood (first search uses 2*kn) */
    int32_t ki;            /* interpolation neighbourhood, 0 = no interpolation */
    int32_t kd;            /* signed-distance neighbourhood */
    int32_t nem;           /* plane fit: 0 least squares (lvr2 default), 1 RANSAC, 2 iterative, 3 PCA,
                              4 the LBVH comparator's FP64 fit (LBVHIndex::knn_normals,
                              src/liblvr2/reconstruction/cuda/lbvh/knn_normals_kernel.cu:54-206;
                              CudaKSearchSurface, --pcm LBVH_CUDA): one search with k = kn <= 96,
                              no adaptive rounds, slot 0 (the query) left out.
                              1: calcPlaneRANSAC (AdaptiveKSearchSurface.tcc:689-781) with
                              lvr2's draws (a default-seeded std::default_random_engine per
                              call, libstdc++) and indexing (plane points = the cloud's
                              points at the drawn neighbour ranks); needs min(2kn, n) >= 3.
                              lvr2 reads the fit's `ok` flag uninitialised (:223-231): the
                              RANSAC plane is kept here; the fallback reading is nem 0 */
    int32_t adaptive;      /* 1: k = 2kn, 4kn, ... 32kn until the neighbourhood box is well formed */
    int32_t flip_set;      /* 0: flip point = bounding-box centroid (AdaptiveKSearchSurface::init) */
    float flip[3];         /* flip point when flip_set != 0 */
    int32_t bucket;        /* LBVH bucket size 1..32 (0 = 32) */
    float gap_threshold;   /* relative eigengap below which PCA solves in FP64 (0 = 1e-3) */
    int32_t device;        /* CUDA device ordinal */
    int32_t seed_radius;   /* Morton-neighbour buckets scanned on each side of a search's start (0 = 1) */
} lvrgb_surface_config;

/* Fills the lvr2_reconstruct defaults: kn 10, ki 10, kd 5, nem 0, adaptive,
 * flip point (0,0,0) (src/tools/lvr2_reconstruct/Options.cpp:69-118,
 * Main.cpp:335-349). */
void lvrgb_surface_config_default(lvrgb_surface_config* cfg);

/* Builds the search structure over n points.  Replaces the search-tree
 * construction of AdaptiveKSearchSurface (getSearchTree,
 * include/lvr2/util/Factories.tcc:44-83; SearchKDTree ctor,
 * include/lvr2/algorithm/KDTree.tcc:317-329), PointsetSurface's bounding box
 * (include/lvr2/reconstruction/PointsetSurface.tcc:39-58) and
 * LBVHIndex::build (include/lvr2/reconstruction/cuda/LBVHIndex.hpp:114).
 * A point with a NaN or infinite coordinate is LVRGB_ERR_INVALID_ARGUMENT (the
 * same holds for lvrgb_surface_set_points and lvrgb_batch_create); a query
 * with one has no neighbours. */
lvrgb_status lvrgb_surface_create(const lvrgb_surface_config* cfg, const float* xyz, int64_t n,
                                  int32_t on_device, void* stream, lvrgb_surface* out);

/* Frees the handle and its device memory (CudaSurface::freeGPU,
 * include/lvr2/reconstruction/cuda/CudaSurface.hpp:158). */
lvrgb_status lvrgb_surface_destroy(lvrgb_surface s);

/* PointsetSurface::setKn/setKi/setKd (PointsetSurface.hpp:112-126),
 * CudaSurface::setKn/setKi/setKd (CudaSurface.hpp:108-126).  A value < 0
 * leaves that parameter unchanged. */
lvrgb_status lvrgb_surface_set_k(lvrgb_surface s, int32_t kn, int32_t ki, int32_t kd);

/* PointsetSurface::setFlipPoint (PointsetSurface.hpp:128-131),
 * CudaSurface::setFlippoint (CudaSurface.hpp:136). */
lvrgb_status lvrgb_surface_set_flip_point(lvrgb_surface s, float x, float y, float z);

/* Scan poses (AdaptiveKSearchSurface's posefile argument,
 * AdaptiveKSearchSurface.tcc:94-139): with poses, each normal is flipped
 * toward the cloud point whose input index is its nearest pose's index
 * (m_points[nearestPoseIds[0]], :252-265; lvr2 indexes the cloud with the pose
 * index), or toward the flip point when that index is not a point.  Nearest =
 * smallest (float d2, pose index).  poses: np x 3 (host), np <= 8192; np = 0
 * removes them. */
lvrgb_status lvrgb_surface_set_scan_poses(lvrgb_surface s, const float* poses, int64_t np);

/* Plane-fit method: AdaptiveKSearchSurface calcMethod / CudaSurface::setMethod
 * (CudaSurface.hpp:144), 0..4 as in lvrgb_surface_config; nem 4 is the fit of
 * CudaKSearchSurface. */
lvrgb_status lvrgb_surface_set_method(lvrgb_surface s, int32_t nem);

/* PointsetSurface::getBoundingBox (PointsetSurface.hpp:106): out9 = min xyz,
 * max xyz, centroid xyz (BoundingBox.tcc:198-215 arithmetic). */
lvrgb_status lvrgb_surface_bounding_box(lvrgb_surface s, float out9[9]);
lvrgb_status lvrgb_surface_num_points(lvrgb_surface s, int64_t* n);

/* AdaptiveKSearchSurface::calculateSurfaceNormals
 * (include/lvr2/reconstruction/AdaptiveKSearchSurface.tcc:158-290) followed,
 * when ki > 0, by interpolateSurfaceNormals (:293-335).  Replaces
 * CudaSurface::calculateNormals (CudaSurface.hpp:88) and
 * LBVHIndex::knn_normals (LBVHIndex.hpp:301).  Synchronous. */
lvrgb_status lvrgb_calculate_normals(lvrgb_surface s, void* stream);

/* AdaptiveKSearchSurface::interpolateSurfaceNormals
 * (include/lvr2/reconstruction/AdaptiveKSearchSurface.hpp:188, .tcc:293-335),
 * CudaSurface::interpolateNormals (CudaSurface.hpp:93): replaces the current
 * normals (estimated or set) by their ki-neighbourhood interpolation.
 * Synchronous. */
lvrgb_status lvrgb_interpolate_normals(lvrgb_surface s, void* stream);

/* Normals in input order (n x 3).  CudaSurface::getNormals(floatArr)
 * (CudaSurface.hpp:99); PointBuffer "normals" channel. */
lvrgb_status lvrgb_get_normals(lvrgb_surface s, float* normals, int32_t on_device, void* stream);

/* lvrgb_get_normals into host memory without waiting: the copy is ordered
 * after the work issued so far on `stream` and runs on `copy_stream`, so it
 * overlaps whatever the caller issues next on `stream` (lvrgb_reconstruct,
 * lvrgb_optimize_planar_faces).  `normals` should be pinned host memory.  The
 * caller synchronizes copy_stream before reading `normals`, and does not call
 * lvrgb_surface_set_points, lvrgb_calculate_normals, lvrgb_set_normals,
 * lvrgb_interpolate_normals or this function on the same surface until then.
 * No lvr2 counterpart (lvr2 copies normals synchronously). */
lvrgb_status lvrgb_get_normals_async(lvrgb_surface s, float* normals, void* stream, void* copy_stream);

/* Normals before interpolation (n x 3), and the k of the search whose
 * neighbourhood fitted each plane (may be NULL). */
lvrgb_status lvrgb_get_raw_normals(lvrgb_surface s, float* normals, int32_t* k_used, int32_t on_device,
                                   void* stream);

/* Use given normals instead of estimating them (lvr2_reconstruct without
 * --recalcNormals on a cloud with normals, Main.cpp:380-383). */
lvrgb_status lvrgb_set_normals(lvrgb_surface s, const float* normals, int32_t on_device, void* stream);

/* Counters of the last lvrgb_calculate_normals: out[0..4] planes fitted in
 * search round 1..5, out[5] PCA eigensolves done in FP64, out[8] LBVH
 * buckets scanned (per 32-query warp), out[9] tree nodes expanded (per warp),
 * out[10] heap insertions (per query), out[11] 32-candidate chunks scanned
 * (per warp); other entries 0. */
lvrgb_status lvrgb_normal_stats(lvrgb_surface s, uint32_t out[16]);

/* Counters of the signed-distance searches of the last lvrgb_reconstruct
 * (sums over its grid vertices): out[0] LBVH buckets scanned, out[1] tree
 * nodes expanded (both per 32-query warp tile), out[2] heap insertions,
 * out[3] 32-candidate chunks scanned, out[4] warp insertion rounds; other
 * entries 0.  Diagnostics; no lvr2 counterpart. */
lvrgb_status lvrgb_distance_stats(lvrgb_surface s, uint64_t out[8]);

/* Batched k-nearest-neighbour search: SearchTree::kSearch / kSearchParallel
 * (include/lvr2/reconstruction/SearchTree.hpp:71, 101-125),
 * LBVHIndex::kSearch (LBVHIndex.hpp:135).  Rows of k, ascending; idx =
 * input indices (0xffffffff padding), dist = Euclidean distance (+inf
 * padding), count (may be NULL) = neighbours found.  Synchronous for host
 * pointers. */
lvrgb_status lvrgb_knn(lvrgb_surface s, const float* q, int64_t nq, int32_t k, uint32_t* idx, float* dist,
                       int32_t* count, int32_t on_device, void* stream);

/* LBVHIndex::calculate_normals (src/liblvr2/reconstruction/cuda/LBVHIndex.cu:586-642,
 * lbvh/normals_kernel.cu:11-180): the nem 4 plane fit from given neighbour
 * lists.  queries: nq x 3; n_neighbors[nq] (<= k); indices: nq x k input
 * indices of this surface's points, the first n_neighbors of each row used,
 * slot 0 taken as the query itself and left out.  Flipped toward the
 * surface's flip point (the comparator's default is (1e6, 1e6, 1e6)).  A count
 * above k or a used index >= n is LVRGB_ERR_INVALID_ARGUMENT. */
lvrgb_status lvrgb_normals_from_neighbors(lvrgb_surface s, const float* queries, int64_t nq, int32_t k,
                                          const uint32_t* n_neighbors, const uint32_t* indices, float* normals,
                                          int32_t on_device, void* stream);

/* SearchTree::radiusSearch (include/lvr2/reconstruction/SearchTree.hpp:86,
 * SearchKDTree::radiusSearch in include/lvr2/algorithm/KDTree.tcc:368-380): up
 * to k nearest points with distance below radius, for nq queries; rows as in
 * lvrgb_knn (ascending (d2, index), idx 0xffffffff and dist +inf padding;
 * count = points found).  Canonical test: float d2 < radius * radius (the
 * reference compares double d2 with a double radius^2). */
lvrgb_status lvrgb_radius_search(lvrgb_surface s, const float* q, int64_t nq, int32_t k, float radius,
                                 uint32_t* idx, float* dist, int32_t* count, int32_t on_device, void* stream);

/* AdaptiveKSearchSurface::distance for nq positions
 * (AdaptiveKSearchSurface.tcc:414-457, PointsetSurface.hpp:74-75): projected
 * and Euclidean distance to the mean of the kd nearest points along their
 * normalised mean normal. */
lvrgb_status lvrgb_distance(lvrgb_surface s, const float* q, int64_t nq, float* projected, float* euclidean,
                            int32_t on_device, void* stream);

/* CudaSurface::distances(std::vector<QueryPoint<Vec>>&, float voxel_size)
 * (CudaSurface.hpp:156): projected distance and the invalid flag of
 * PointsetGrid::calcDistanceValues (euclidean > 1.75 * voxel_size,
 * PointsetGrid.tcc:133-140). */
lvrgb_status lvrgb_grid_distances(lvrgb_surface s, const float* q, int64_t nq, float voxel_size, float* distance,
                                  uint8_t* invalid, int32_t on_device, void* stream);

/* PointsetSurface::getInterpolatedNormal (PointsetSurface.tcc:61-74) for nq
 * positions (n x 3 out): ((0, 1, 0) + the sum of the ki nearest points'
 * normals, each normalised) / ki.  Like lvr2 (whose final
 * Normal<float>(result) is a copy, :72-73) the mean is not normalised. */
lvrgb_status lvrgb_interpolated_normal(lvrgb_surface s, const float* q, int64_t nq, float* out,
                                       int32_t on_device, void* stream);

/* Reverse mode of lvrgb_distance (AdaptiveKSearchSurface::distance,
 * AdaptiveKSearchSurface.tcc:414-457).  No lvr2 counterpart: lvr2 has no
 * gradients; this is the adjoint form of its signed distance for
 * optimisation and learning pipelines.  Each position's kd nearest points are
 * held fixed (the distance is piecewise smooth in q).  With c = mean point,
 * m = mean normal, nh = m/|m|, r = q - c, d = r.nh, e = |r| and upstream
 * gradients gd = grad_projected[i], ge = grad_euclidean[i] (either array may
 * be NULL = 0):
 *   grad_q[i]          = gd nh + ge r/e
 *   grad_points[j]    += -grad_q[i] / kd       for each neighbour j of q_i
 *   grad_normals[j]   += gd (r - d nh) / (kd |m|)
 * grad_points / grad_normals (n x 3, input point order) are written (sums
 * over all queries; float atomics, so their last bits depend on summation
 * order).  projected / euclidean (may be NULL) equal lvrgb_distance's bit for
 * bit.  Any output may be NULL. */
lvrgb_status lvrgb_distance_adjoint(lvrgb_surface s, const float* q, int64_t nq, const float* grad_projected,
                                    const float* grad_euclidean, float* projected, float* euclidean, float* grad_q,
                                    float* grad_points, float* grad_normals, int32_t on_device, void* stream);

/* Newton projection of nv positions onto the zero level of the signed
 * distance: `steps` (1..64) updates x <- x - d(x) nh(x), each with the kd
 * nearest points of the current x; out_normals = nh of the last step (the
 * analytic gradient of d, a vertex normal for mesh vertices).  No lvr2
 * counterpart (lvr2 places marching-cubes vertices by linear interpolation
 * only); used to refine lvrgb_get_mesh vertices.  out_positions or
 * out_normals may be NULL. */
lvrgb_status lvrgb_project_to_surface(lvrgb_surface s, const float* v, int64_t nv, int32_t steps,
                                      float* out_positions, float* out_normals, int32_t on_device, void* stream);

/* Grid and marching-cubes parameters: the lvr2_reconstruct flags --voxelsize,
 * --intersections, --noExtrusion, --decomposition (Options.cpp:69-74). */
typedef struct lvrgb_grid_config {
    float resolution;       /* voxel size, or intersections when is_voxelsize == 0 */
    int32_t is_voxelsize;
    int32_t extrude;        /* 0 = --noExtrusion */
    int32_t decomposition;  /* 0 = MC (FastBox), 1 = PMC (BilinearFastBox, lvr2 default) */
} lvrgb_grid_config;

typedef struct lvrgb_mesh_info {
    int64_t cells_all;      /* grid cells before culling */
    int64_t grid_vertices;  /* query points */
    int64_t cells_valid;    /* cells after culling ("Grid Cells" log line) */
    int64_t vertices;       /* mesh vertices */
    int64_t faces;          /* mesh faces */
    float voxelsize;
    float stage_ms[4];      /* device time: grid build, signed distance, culling, marching cubes */
} lvrgb_mesh_info;

/* PointsetGrid construction (include/lvr2/reconstruction/PointsetGrid.tcc:41-109),
 * calcDistanceValues (:111-185) and FastReconstruction::getMesh
 * (include/lvr2/reconstruction/FastReconstruction.tcc:47-66) with FastBox /
 * BilinearFastBox::getSurface (FastBox.tcc:205-269, BilinearFastBox.tcc:55-138),
 * as called by createGridAndReconstruction (src/tools/lvr2_reconstruct/Main.cpp:404-453).
 * Needs normals (lvrgb_calculate_normals or lvrgb_set_normals).  The mesh
 * stays on the handle until the next call.  Synchronous. */
lvrgb_status lvrgb_reconstruct(lvrgb_surface s, const lvrgb_grid_config* g, lvrgb_mesh_info* info, void* stream);

/* The last mesh: vertices (V x 3), faces (F x 3 vertex indices, MC-table
 * orientation) and, optionally, each vertex's grid edge (V x 4: lattice x, y,
 * z of the edge's lower corner and the edge axis 0/1/2).  Replaces the
 * BaseMesh::addVertex / addFace calls of FastBox::getSurface
 * (include/lvr2/geometry/BaseMesh.hpp:115, 131). */
lvrgb_status lvrgb_get_mesh(lvrgb_surface s, float* vertices, uint32_t* faces, int32_t* vertex_edges,
                            int32_t on_device, void* stream);

/* BilinearFastBox::optimizePlanarFaces (BilinearFastBox.tcc:140-212), the
 * post-pass that FastReconstruction::getMesh runs for PMC with kc = 5
 * (FastReconstruction.tcc:158-168), on the last mesh in place: in every cell
 * whose faces have one or two border edges, both end vertices of each such
 * edge move to the centroid of their kc (1..96) nearest points.  lvr2 moves
 * vertices in place in hash-map order, so a vertex on several such edges can
 * move twice; here each moves once, from its marching-cubes position.
 * moved (may be NULL) receives the number of moved vertices.  Synchronous. */
lvrgb_status lvrgb_optimize_planar_faces(lvrgb_surface s, int32_t kc, int64_t* moved, void* stream);

/* calcVertexNormals(mesh, calcFaceNormals(mesh), surface)
 * (include/lvr2/algorithm/NormalAlgorithms.tcc:57-152), as lvr2_reconstruct
 * computes them for the finished mesh (src/tools/lvr2_reconstruct/Main.cpp:855-871):
 * each vertex normal is the normalised sum of the normals of its faces
 * (summed in ascending face order), or the normal of its nearest point when
 * that sum is zero.  Applies to the last mesh (after lvrgb_optimize_planar_faces
 * if that ran).  vertex_normals: V x 3. */
lvrgb_status lvrgb_mesh_vertex_normals(lvrgb_surface s, float* vertex_normals, int32_t on_device, void* stream);

/* calcColorFromPointCloud (include/lvr2/algorithm/ColorAlgorithms.tcc:43-92):
 * each vertex of the last mesh takes the colour of its nearest point
 * (kSearch with k = 1; ties to the lower point index).  point_colors: n x width
 * bytes in input order (width 3 for RGB8, 4 for RGBA8; 1..16); vertex_colors:
 * V x width. */
lvrgb_status lvrgb_mesh_vertex_colors(lvrgb_surface s, const uint8_t* point_colors, int32_t width,
                                      uint8_t* vertex_colors, int32_t on_device, void* stream);

/* The same for any triangle mesh against this surface's points and normals
 * (the reference's calcVertexNormals takes any BaseMesh and PointsetSurface):
 * vertices V x 3, faces F x 3 with indices < V (checked; an index out of range
 * is LVRGB_ERR_INVALID_ARGUMENT).  nearest_count (optional) receives the number
 * of vertices that took their nearest point's normal (no faces, or a zero
 * face normal sum). */
lvrgb_status lvrgb_vertex_normals(lvrgb_surface s, const float* vertices, int64_t nv, const uint32_t* faces,
                                  int64_t nf, float* vertex_normals, int64_t* nearest_count, int32_t on_device,
                                  void* stream);

/* The last grid, sorted by lattice key: each grid vertex's lattice index
 * (Q x 3), position (Q x 3), projected distance and invalid flag; any
 * pointer may be NULL.  Same content as HashGrid::getQueryPoints
 * (include/lvr2/reconstruction/HashGrid.hpp:179). */
lvrgb_status lvrgb_get_grid(lvrgb_surface s, int32_t* lattice, float* position, float* distance,
                            uint8_t* invalid, int32_t on_device, void* stream);

/* The large-scale reconstruction's merge and mesh step
 * (LargeScaleReconstruction.tcc:433-449, 781-789): HashGrid(chunks, innerBoxes,
 * bb, voxelsize) (include/lvr2/reconstruction/HashGrid.tcc:136-193) built from
 * stored chunk grids, then FastReconstruction::getMesh.  The cells are the
 * concatenation of the chunks' lvrgb_get_cell_tsdf outputs: centers (n x 3)
 * and tsdf_values (n x 8), chunk c holding cells [chunk_offsets[c],
 * chunk_offsets[c + 1]) (host array of nchunks + 1, or NULL for one chunk).
 * inner_boxes (host, nchunks x 6: min xyz, max xyz, or NULL): a cell is kept
 * when its chunk's box contains its centre (BoundingBox::contains).  A cell
 * index (floor(centre / voxel_size)) already present keeps its first copy, and
 * a grid vertex takes the distance of the earliest cell holding it, as
 * HashGrid::addBox does.  decomposition 0 = FastBox (the large-scale default),
 * 1 = BilinearFastBox.  The result replaces the surface's last mesh (read it
 * with lvrgb_get_mesh); the surface's points are not used. */
lvrgb_status lvrgb_reconstruct_cells(lvrgb_surface s, float voxel_size, int32_t decomposition, const float* centers,
                                     const float* tsdf_values, int64_t ncells, const int64_t* chunk_offsets,
                                     int32_t nchunks, const float* inner_boxes, lvrgb_mesh_info* info,
                                     int32_t on_device, void* stream);

/* Half-edge connectivity of the last mesh in pmp::SurfaceMesh's layout
 * (include/lvr2/geometry/pmp/SurfaceMesh.h), for building the PMPMesh that
 * lvr2_reconstruct fills face by face (PMPMesh::addFace,
 * include/lvr2/geometry/PMPMesh.tcc; pmp SurfaceMesh::add_face,
 * src/liblvr2/geometry/pmp/SurfaceMesh.cpp:283-460) in one pass:
 *   edge e owns halfedges 2e and 2e + 1 (opposite = h ^ 1), numbered in the
 *   order in which add_face over faces 0..F-1 creates them, 2e pointing the
 *   way the edge first appeared; he_vertex[h] = the vertex h points to;
 *   he_face[h] = its face or 0xffffffff on the boundary; he_next, he_prev;
 *   vertex_he[v] = an outgoing halfedge, a boundary one on the boundary
 *   (0xffffffff for a vertex without faces); face_he[f] = the halfedge from
 *   its corner 2 to corner 0.
 * At a vertex with several boundary gaps (info->complex_vertices) the
 * boundary links pair incoming and outgoing boundary halfedges in ascending
 * order.  Complex edges (more than two faces, or two of one orientation)
 * return LVRGB_ERR_TOPOLOGY with info->complex_edges set.  Any array may be
 * NULL (info only); he_* arrays have 2 * info->edges entries. */
typedef struct lvrgb_halfedge_info {
    int64_t vertices, faces, edges;
    int64_t boundary_halfedges;
    int64_t complex_edges;
    int64_t complex_vertices;
} lvrgb_halfedge_info;
lvrgb_status lvrgb_mesh_halfedges(lvrgb_surface s, lvrgb_halfedge_info* info, uint32_t* he_vertex, uint32_t* he_next,
                                  uint32_t* he_prev, uint32_t* he_face, uint32_t* vertex_he, uint32_t* face_he,
                                  int32_t on_device, void* stream);
/* The same for a caller's triangle list faces (nf x 3 vertex indices < nv),
 * e.g. a mesh read from a file before PMPMesh construction or a merged
 * large-scale mesh; s supplies the device and workspace only.  A face that
 * repeats a vertex counts as a complex edge. */
lvrgb_status lvrgb_halfedges(lvrgb_surface s, const uint32_t* faces, int64_t nf, int64_t nv, lvrgb_halfedge_info* info,
                             uint32_t* he_vertex, uint32_t* he_next, uint32_t* he_prev, uint32_t* he_face,
                             uint32_t* vertex_he, uint32_t* face_he, int32_t on_device, void* stream);

/* HashGrid::toPointBuffer (include/lvr2/reconstruction/HashGrid.tcc:196-233),
 * the per-chunk grid the large-scale reconstruction stores and merges: for
 * each cell kept after culling (lattice-key order, in place of the hash map's
 * bucket order) its centre (centers, C x 3) and the projected distances at
 * its 8 corners in FastBox corner order (tsdf_values, C x 8, the
 * "tsdf_values" channel).  C = lvrgb_mesh_info.cells_valid.  Either array
 * may be NULL. */
lvrgb_status lvrgb_get_cell_tsdf(lvrgb_surface s, float* centers, float* tsdf_values, int32_t on_device,
                                 void* stream);

/* Cells of the last grid as lattice indices (x, y, z of the cell's lowest
 * corner): all cells before culling and the valid cells (either may be NULL).
 * HashGrid::getCells (HashGrid.hpp:182). */
lvrgb_status lvrgb_get_cells(lvrgb_surface s, int32_t* cells_all, int32_t* cells_valid, int32_t on_device,
                             void* stream);

/* Replaces the points of an existing handle and rebuilds its search
 * structure, reusing its device memory (LBVHIndex::build on an existing
 * index, include/lvr2/reconstruction/cuda/LBVHIndex.hpp:114).  Normals and
 * the mesh of the previous points are dropped. */
lvrgb_status lvrgb_surface_set_points(lvrgb_surface s, const float* xyz, int64_t n, int32_t on_device,
                                      void* stream);

/* Device time in ms of the handle's last calls: out[0] search-structure
 * build, [1] normal estimation, [2] interpolation, [3] grid build, [4]
 * signed distance, [5] culling, [6] marching cubes, [7] the PMC planar
 * post-pass (lvrgb_optimize_planar_faces on the last mesh; 0 if none).  These
 * are the stage boundaries of lvr2_reconstruct's log lines
 * (README.md:118-124).  No lvr2 counterpart beyond those log lines. */
lvrgb_status lvrgb_surface_timings(lvrgb_surface s, float out[8]);

/* Number of kernels this library has launched in the process (diagnostics;
 * no lvr2 counterpart). */
lvrgb_status lvrgb_kernel_launches(uint64_t* out);

/* Fault injection for tests of the out-of-memory path that lvr2's large-scale
 * tool handles (LargeScaleReconstruction.tcc:647-671): the n-th device
 * allocation from now on (through any handle's workspace) fails with
 * LVRGB_ERR_OUT_OF_MEMORY, on the host, without touching the GPU.  n <= 0
 * turns it off.  The handle stays usable after such a failure. */
lvrgb_status lvrgb_debug_fail_allocation(int64_t n);

/* Round collapsing of the adaptive normal search (on by default).  lvr2
 * searches k = 2kn, 4kn, ... 32kn until the neighbourhood box passes
 * (AdaptiveKSearchSurface.tcc:187-216); on scans, points on axis-aligned
 * walls fail every round.  When almost nothing fits in round 2 or 3, the
 * library searches once with the last round's k and tests the rounds in
 * between on the prefixes of that sorted kNN, since kNN(k) is the first k of
 * kNN(32 kn): the same normals and rounds with fewer searches.  enable = 0
 * runs every round on its own (for tests that compare the two).  No lvr2
 * counterpart. */
lvrgb_status lvrgb_debug_round_collapse(int32_t enable);

/* k nearest neighbours of nq queries among n points WITHOUT ANY DEVICE
 * ALLOCATION.  No counterpart in lvr2: it exists for callers that cannot
 * call cudaMalloc during a call (real-time loops or driver callbacks where an
 * allocation would synchronize the device, hosts that give a library a fixed
 * device-memory budget, plugins whose host owns every allocation).
 *  - points (n x 3), queries (nq x 3), idx and dist (nq x k) are DEVICE
 *    pointers on the current device; results as lvrgb_knn (ascending,
 *    0xffffffff / +inf padding when n < k).
 *  - Limits: 1 <= n <= 65536, 0 <= nq <= 65536, 1 <= k <= 96; larger inputs
 *    are rejected with LVRGB_ERR_INVALID_ARGUMENT.  Use lvrgb_surface_create
 *    and lvrgb_knn for anything bigger.
 *  - A point with a NaN or infinite coordinate is rejected with
 *    LVRGB_ERR_INVALID_ARGUMENT naming the first such point (as
 *    lvrgb_surface_create does); a query with one gets padding rows.
 *  - Scratch is one 8 MiB static device array that every GPU loading this
 *    library holds until the process exits.  The first call on a device looks
 *    up its address (cudaGetSymbolAddress).
 *  - All calls share the array: calls that overlap on the GPU (other streams,
 *    other host threads) race and must be serialized by the caller.
 *  - Every call synchronizes `stream` (small reads of the point bounding box,
 *    the non-finite marker and the error flag into host memory), so it must
 *    not be called while `stream` is being captured into a CUDA graph. */
lvrgb_status lvrgb_knn_small_noalloc(const float* points, int64_t n, const float* queries, int64_t nq, int32_t k,
                                     uint32_t* idx, float* dist, void* stream);

/* ---- scan projects ----------------------------------------------------
 * Normals of every scan of a scan project in one pass: the per-scan
 * CudaSurface runs of lvr2_cuda_normals' directory mode
 * (src/tools/lvr2_cuda_normals/Main.cpp:60-111, 166-190), with kNN restricted
 * to each scan and a per-scan flip point, over one segmented LBVH (one sort,
 * one tree, one normals launch per search round).  Results equal
 * lvrgb_calculate_normals run on each scan alone. */
typedef struct lvrgb_batch_s* lvrgb_batch;

/* xyz: all scans concatenated (n x 3); scan_offsets: nscans + 1 entries,
 * scan_offsets[0] = 0, strictly increasing; flip_points: nscans x 3 (the
 * scanner positions).  cfg: kn, ki (<= 2 kn), kd (lvrgb_batch_grid_distances),
 * nem (not 1), adaptive, bucket, seed_radius, device as for a surface (flip
 * fields ignored).  Host arrays
 * for offsets and flips; xyz on host or device (on_device). */
lvrgb_status lvrgb_batch_create(const lvrgb_surface_config* cfg, const float* xyz, const int64_t* scan_offsets,
                                int32_t nscans, const float* flip_points, int32_t on_device, void* stream,
                                lvrgb_batch* out);
lvrgb_status lvrgb_batch_destroy(lvrgb_batch b);

/* Builds the segmented LBVH and computes (and interpolates) all normals.
 * use_graph != 0: the first call runs once and captures the whole launch
 * sequence in a CUDA graph; later calls replay it.  Synchronous. */
lvrgb_status lvrgb_batch_calculate_normals(lvrgb_batch b, int32_t use_graph, void* stream);

/* Normals of all scans in input order (n x 3). */
lvrgb_status lvrgb_batch_get_normals(lvrgb_batch b, float* normals, int32_t on_device, void* stream);

/* Signed distance and invalid flag at the grid vertices of every scan
 * (chunk), each against its own scan's points and normals: the GPU block of
 * LargeScaleReconstruction::createChunk (LargeScaleReconstruction.tcc:636-688),
 * which builds one GpuSurface per chunk, computes its normals and then
 * GpuSurface::distances for the chunk grid's query points, for all chunks at
 * once.  q: every chunk's query positions concatenated (host or device);
 * q_offsets: nscans + 1 host entries, q_offsets[0] = 0, non-decreasing.
 * Semantics per query as lvrgb_grid_distances with the batch's kd.  Needs
 * lvrgb_batch_calculate_normals.  Synchronous for host pointers. */
lvrgb_status lvrgb_batch_grid_distances(lvrgb_batch b, const float* q, const int64_t* q_offsets, float voxel_size,
                                        float* distance, uint8_t* invalid, int32_t on_device, void* stream);

/* Times the pipeline on this project and keeps the fastest candidate, stage
 * by stage: LBVH bucket 16/32 with seed radius 1/2; then the queries per warp
 * tile of the one-warp-per-query searches (automatic, 4, 16, 32); then their
 * key buffer size (2, 3 or 4 times k).  Returns the bucket and seed radius;
 * lvrgb_batch_tuning reports all four. */
lvrgb_status lvrgb_batch_autotune(lvrgb_batch b, int32_t* bucket, int32_t* seed_radius, void* stream);

/* The launch shape the batch uses (what lvrgb_batch_autotune chose): out[0]
 * LBVH bucket size, [1] seed radius, [2] queries per warp tile of the
 * one-warp-per-query searches (k > 96; 0 = chosen from the query count),
 * [3] their key buffer size in units of k.  No lvr2 counterpart. */
lvrgb_status lvrgb_batch_tuning(lvrgb_batch b, int32_t out[4]);

/* Device time in ms of each of the five search rounds (k = 2kn ... 32kn;
 * 0 for rounds that did not run) of the last eager (non-graph) run, which
 * lvrgb_batch_calculate_normals(use_graph = 0) and lvrgb_batch_autotune make.
 * Diagnostics; no lvr2 counterpart. */
lvrgb_status lvrgb_batch_round_times(lvrgb_batch b, float ms[5]);

/* Counters of the last run (layout of lvrgb_normal_stats) and device ms:
 * ms[0] tree, ms[1] normals, ms[2] interpolation (eager runs), ms[3] total. */
lvrgb_status lvrgb_batch_stats(lvrgb_batch b, uint32_t counters[16], float ms[4]);

/* Message of the last failed call on this thread ("" if none). */
const char* lvrgb_last_error(void);

/* Library version string. */
const char* lvrgb_version(void);

#ifdef __cplusplus
}
#endif
#endif /* LVRGB_H */
