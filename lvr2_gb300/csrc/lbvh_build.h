// lbvh_build.h -- host entry of the LBVH construction (lbvh.cu).
#pragma once
#include <string>

#include "lbvh.cuh"
#include "workspace.h"

namespace lvrgb {

// Builds the LBVH of n AoS float32 points held in device memory.  The sorted
// points, inverse permutation and nodes live in ws under the given tag;
// d_box (6 device floats) receives the point bounding box; d_err receives
// kErrWalk if the bottom-up pass meets a malformed parent chain.
void lbvh_build(const float* xyz, int n, int bucket, Workspace& ws, const std::string& tag, Lbvh& T,
                float* d_box, int* d_err, cudaStream_t s);

}  // namespace lvrgb
