// meshops.h -- per-vertex normals of the reconstructed mesh (meshops.cu).
#pragma once
#include "grid.h"
#include "lbvh.cuh"
#include "workspace.h"

namespace lvrgb {

// calcVertexNormals(mesh, calcFaceNormals(mesh), surface)
// (NormalAlgorithms.tcc:57-152) on the mesh (verts V x 3, faces F x 3, all
// indices < V; device arrays): out (device, V x 3).  normals: the surface's
// point normals (Morton order); d_box: the tree's point bounding box.
// Returns the number of vertices that took the normal of their nearest point
// (no faces, or a zero face normal sum).
long long mesh_vertex_normals(const Lbvh& T, const float4* normals, const float* d_box, const float* verts,
                              int nv, const uint32_t* faces, int nf, float* out, Workspace& ws, int* d_err,
                              cudaStream_t s);

// calcColorFromPointCloud (ColorAlgorithms.tcc:43-92): each mesh vertex takes
// the colour (width bytes) of its nearest point (kSearch k = 1).  colors: n x
// width bytes in input order (device); out: V x width (device).
void mesh_vertex_colors(const Lbvh& T, const float* d_box, const float* verts, int nv, const uint8_t* colors,
                        int width, uint8_t* out, Workspace& ws, int* d_err, cudaStream_t s);

// Largest entry of a (device) index array, or 0 for an empty one.
uint32_t max_index(const uint32_t* a, size_t n, Workspace& ws, cudaStream_t s);

}  // namespace lvrgb

namespace lvrgb {

// Half-edge connectivity of a triangle mesh in pmp::SurfaceMesh's layout
// (include/lvr2/geometry/pmp/SurfaceMesh.h): edge e owns halfedges 2e and
// 2e + 1 (opposite = h ^ 1); he_vertex = the vertex a halfedge points to,
// he_face (0xffffffff on the boundary), he_next / he_prev, vertex_he (an
// outgoing halfedge, a boundary one on the boundary), face_he.  Device arrays
// in the workspace.
struct HalfedgeMesh {
    long long nverts = 0, nfaces = 0, nedges = 0;
    long long boundary = 0;          // boundary halfedges
    long long complex_edges = 0;     // edges of > 2 faces or of two faces of one orientation
    long long complex_vertices = 0;  // vertices with more than one boundary gap
    uint32_t* he_vertex = nullptr;
    uint32_t* he_next = nullptr;
    uint32_t* he_prev = nullptr;
    uint32_t* he_face = nullptr;
    uint32_t* vertex_he = nullptr;
    uint32_t* face_he = nullptr;
};

// Builds H for faces (device, nf x 3, indices < nv).  With complex edges the
// arrays are not built (H.complex_edges > 0).
void build_halfedges(const uint32_t* faces, int nf, int nv, Workspace& ws, HalfedgeMesh& H, cudaStream_t s);

}  // namespace lvrgb
