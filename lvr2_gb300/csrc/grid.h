// grid.h -- sparse voxel grid, signed distance at grid vertices, invalid-cell
// culling and marching cubes (grid.cu).
#pragma once
#include "lbvh.cuh"
#include "workspace.h"

namespace lvrgb {

struct GridConfig {
    float resolution = 10.0f;  // voxel size, or number of intersections along the longest side
    int is_voxelsize = 1;
    int extrude = 1;
    int kd = 5;
    int decomposition = 1;  // 0 = MC (FastBox), 1 = PMC (BilinearFastBox)
    // optional device counters of the signed-distance searches (added to):
    // buckets scanned, nodes expanded, heap insertions, candidate chunks,
    // warp insertion rounds
    unsigned long long* sdf_stats = nullptr;
};

// Device results of grid_reconstruct; pointers live in the workspace.
struct GridResult {
    float vs = 0;
    int base[3] = {0, 0, 0};     // lattice coordinate = base + decoded key coordinate
    int nbits = 0;               // bits per axis used by lattice keys
    long long ncells_all = 0;    // cells before culling
    long long nqp = 0;           // grid vertices (query points)
    long long ncells_valid = 0;  // cells after culling
    long long nverts = 0;        // mesh vertices
    long long nfaces = 0;
    uint64_t* cell_keys = nullptr;   // [ncells_all] sorted lattice keys
    uint64_t* qp_keys = nullptr;     // [nqp] sorted lattice keys
    float4* qp_pos = nullptr;        // [nqp] position, w unused
    float* qp_dist = nullptr;        // [nqp] projected distance
    float* qp_eucl = nullptr;        // [nqp] euclidean distance
    uint8_t* qp_invalid = nullptr;   // [nqp]
    uint32_t* cell_corner = nullptr; // [ncells_all * 8] grid vertex of each cell corner
    uint32_t* valid_cells = nullptr; // [ncells_valid] indices into cell_keys
    uint64_t* vert_keys = nullptr;   // [nverts] (corner lattice key << 2) | axis
    float* verts = nullptr;          // [nverts * 3]
    uint32_t* faces = nullptr;       // [nfaces * 3]
    uint32_t* face_cell_off = nullptr;  // [ncells_valid + 1] faces of valid cell c: [off[c], off[c + 1])
};

// Per-stage device time (ms) of the last grid_reconstruct call when events
// are enabled: [0] grid build, [1] signed distance, [2] culling, [3] marching cubes.
struct GridTimings {
    float ms[4] = {0, 0, 0, 0};
};

// Builds the PointsetGrid of the surface, evaluates the signed distance at
// every grid vertex (or takes it from qp_override), culls cells with an
// invalid corner and extracts the marching-cubes mesh.  bb: surface bounding
// box (host, min xyz then max xyz).  normals: Morton order.
void grid_reconstruct(const Lbvh& T, const float4* normals, const float bb[6], const GridConfig& cfg,
                      Workspace& ws, GridResult& R, int* d_err, cudaStream_t s, GridTimings* timings = nullptr);

// HashGrid(chunks, innerBoxes, bb, voxelsize) (HashGrid.tcc:136-193) followed
// by marching cubes: n stored cells (centres n x 3, corner distances n x 8,
// device), chunk c holding cells [chunk_off[c], chunk_off[c + 1]) (device);
// boxes (device, nchunks x 6, or null): a cell is kept when its chunk's box
// contains its centre.  A cell already present keeps its first copy; a grid
// vertex takes the distance of the earliest cell holding it.
void grid_from_cells(const float* centers, const float* tsdf, int n, const int64_t* chunk_off, int nchunks,
                     const float* boxes, float vs, int decomposition, Workspace& ws, GridResult& R, int* d_err,
                     cudaStream_t s);

// HashGrid::toPointBuffer (HashGrid.tcc:196-233) of the culled grid: per valid
// cell (lattice-key order) its centre (centers, 3 floats) and the projected
// distances at its 8 corners in FastBox corner order (tsdf, 8 floats).
void cell_tsdf(const GridResult& R, float* centers, float* tsdf, cudaStream_t s);

// Batched AdaptiveKSearchSurface::distance at nq positions (float4 xyz, w =
// row index bits), rows written to dist/eucl; invalid (optional) uses the
// 1.75 * voxelsize rule of PointsetGrid::calcDistanceValues.
void signed_distance_rows(const Lbvh& T, const float4* normals, int kd, const float4* qs, int nq, float vs,
                          float* dist, float* eucl, uint8_t* invalid, Workspace& ws, int* d_err, cudaStream_t s,
                          unsigned long long* stats = nullptr);

}  // namespace lvrgb
