// planar.h -- the PMC mesh post-pass BilinearFastBox::optimizePlanarFaces
// (planar.cu).
#pragma once
#include "grid.h"
#include "lbvh.cuh"
#include "workspace.h"

namespace lvrgb {

// In every valid cell whose faces have one or two border edges (edges of
// exactly one face of the mesh), both end vertices of each such edge move to
// the centroid of their kc nearest points (in place in R.verts).  Each marked
// vertex moves once, from its marching-cubes position.  d_box: the tree's
// point bounding box (device, 6 floats).  Returns the number of moved
// vertices.
long long optimize_planar_faces(const Lbvh& T, const float* d_box, GridResult& R, int kc, Workspace& ws,
                                int* d_err, cudaStream_t s);

}  // namespace lvrgb
