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
