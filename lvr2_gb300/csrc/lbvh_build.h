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

// Device buffers for lbvh_build_into, sized for n points (see
// lbvh_into_bytes); the caller owns them.
struct LbvhBuffers {
    float4* pts;
    uint32_t* inv;
    TreeNode* nodes;     // max(1, nb - 1)
    uint32_t* bkeys;     // nb
    int* bparent;        // nb
    int* counters;       // max(1, nb - 1), cleared by lbvh_build_into
    uint32_t* codes;
    uint32_t* codes2;
    uint32_t* idx;
    uint32_t* idx2;
    void* sort_tmp;      // radix_sort_temp_bytes<uint32_t>(n)
    void* box_tmp;       // bbox_temp_bytes(n)
    float* box;          // 6 floats
    int* err;
};

// Same construction as lbvh_build, into caller-provided buffers (no
// allocation).
void lbvh_build_into(const float* xyz, int n, int bucket, const LbvhBuffers& B, Lbvh& T, cudaStream_t s);

}  // namespace lvrgb
