// chunks.h -- signed distance at each chunk's grid vertices against that
// chunk's points and normals, for all chunks of a batch (chunks.cu).
#pragma once
#include "lbvh_build.h"
#include "workspace.h"

namespace lvrgb {

// d_q: all chunks' query positions concatenated (AoS, device); d_qoff:
// tree.nscans + 1 offsets (device).  normals: the batch's final normals
// (padded Morton order).  dist / invalid: rows in query order (device).
void chunk_grid_distances(const SegTree& tree, const float4* normals, int kd, const float* d_q,
                          const int64_t* d_qoff, int nq, float vs, float* dist, uint8_t* invalid, Workspace& ws,
                          int* d_err, cudaStream_t s);

}  // namespace lvrgb
