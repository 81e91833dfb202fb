/*
 * lvr_oracle.h -- C ABI of the CPU oracle for the lvr2 reconstruction hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  The oracle is a CPU restatement of the lvr2
 * reference algorithm (kd-tree kNN, AdaptiveKSearchSurface normals,
 * interpolation and distance, HashGrid/PointsetGrid, FastBox /
 * BilinearFastBox marching cubes).  It is used by the test-suite as the
 * checker and by bench.py as the timed CPU baseline.  The product
 * (lvr2_gb300, liblvrgb.so) never links or calls it.
 *
 * All point arrays are AoS float32 xyz in the caller's (original) order.
 * "canonical" selects the neighbour order used for parity with the GPU:
 *   canonical = 0 : reference-faithful kd-tree search (double squared
 *                   distances, std::priority_queue admission, strict '<'),
 *   canonical = 1 : exact k smallest of the key (d2_f32, index), where
 *                   d2_f32 = fl(fl(fl(dx*dx) + fl(dy*dy)) + fl(dz*dz)),
 *                   dx = fl(qx - px), no fused multiply-add.
 */
#ifndef LVR_ORACLE_H
#define LVR_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_surface orc_surface;
typedef struct orc_recon orc_recon;

/* SearchKDTree over the points (leaf size 20 in the reference) + bounding box. */
orc_surface* orc_create(const float* xyz, int64_t n, int leaf_size, int threads);
void orc_destroy(orc_surface* s);
/* out[0..2] = bb min, out[3..5] = bb max, out[6..8] = bb centroid. */
void orc_bbox(const orc_surface* s, float* out9);

/* k nearest neighbours of nq queries.  idx/dist are nq*k, rows padded with
 * 0xffffffff / +inf when fewer than k points exist; dist = sqrt(d2).
 * count[i] = number found. */
int orc_knn(const orc_surface* s, const float* q, int64_t nq, int k, int canonical,
            uint32_t* idx, float* dist, int32_t* count, int threads);

/* calculateSurfaceNormals without interpolation.  nem: 0 LSQ plane,
 * 2 iterative, 3 IPCA exact.  adaptive=1 reproduces the k = 2kn..32kn
 * doubling with the bounding-box test.  k_used (optional) receives the k of
 * the search whose neighbours fitted the plane. */
int orc_normals(const orc_surface* s, int kn, int nem, int adaptive, const float* flip3,
                int canonical, float* normals, int32_t* k_used, int threads,
                const float* flip_targets);

/* interpolateSurfaceNormals: out_i = normalize(in_i + sum_{j in kNN(ki)} in_j). */
/* The draw sequence of calcPlaneRANSAC for m neighbours (10 x 53 entries:
 * 3 plane ranks, then min(50, m) scoring ranks); -1 when it fails. */
int orc_ransac_draws(int64_t m, uint32_t* out);

int orc_interpolate(const orc_surface* s, int ki, const float* normals_in, float* normals_out,
                    int canonical, int threads);

/* AdaptiveKSearchSurface::distance for nq query positions. */
int orc_distance(const orc_surface* s, const float* normals, int kd, const float* q, int64_t nq,
                 int canonical, float* projected, float* euclidean, int threads);

/* PointsetSurface::getInterpolatedNormal for nq query positions. */
int orc_interpolated_normal(const orc_surface* s, const float* normals, int ki, const float* q,
                            int64_t nq, int canonical, float* out, int threads);

/* PointsetGrid construction + calcDistanceValues + FastReconstruction::getMesh.
 * decomposition: 0 = MC (FastBox), 1 = PMC (BilinearFastBox, no
 * optimizePlanarFaces).  If qp_lattice != NULL the distance values of the
 * grid vertices are taken from (qp_lattice, qp_dist, qp_invalid) instead of
 * being computed (used to test the marching cubes stage on identical input). */
orc_recon* orc_reconstruct(const orc_surface* s, const float* normals, float resolution,
                           int is_voxelsize, int extrude, int kd, int decomposition, int canonical,
                           const int32_t* qp_lattice, const float* qp_dist,
                           const uint8_t* qp_invalid, int64_t n_qp, int threads);
void orc_recon_destroy(orc_recon* r);
/* counts[0]=cells before culling, [1]=grid vertices, [2]=cells after culling,
 * [3]=mesh vertices, [4]=faces; fvals[0]=voxelsize. */
void orc_recon_counts(const orc_recon* r, int64_t* counts, float* fvals);
/* grid vertices sorted by lattice (x, y, z): lattice int32 x3, position
 * float x3, projected distance, invalid flag. */
void orc_recon_grid(const orc_recon* r, int32_t* lattice, float* pos, float* dist, uint8_t* invalid);
/* cells before culling (lattice x3, sorted) and cells after culling (sorted). */
void orc_recon_cells(const orc_recon* r, int32_t* cells_all, int32_t* cells_valid);
/* mesh: vertex keys (lattice of the edge's low corner x3, axis), positions,
 * faces as vertex indices (emission order within a cell follows the MC table). */
void orc_recon_mesh(const orc_recon* r, int32_t* vkeys, float* vpos, int32_t* faces);
/* BilinearFastBox::optimizePlanarFaces on the mesh of r, in canonical form
 * (each marked vertex moves once, from its marching-cubes position); returns
 * the number of moved vertices. */
int64_t orc_recon_optimize_planar(orc_recon* r, const orc_surface* s, int kc, int canonical, int threads);

/* Table dump (used to pin the tables against the reference headers). */
int orc_mc_table(int32_t* out256x13);

#ifdef __cplusplus
}
#endif
#endif
