// lbvh_build.h -- host entry of the LBVH construction (lbvh.cu).
#pragma once
#include <string>
#include <vector>

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
    uint64_t* bkeys;     // nb
    int* bparent;        // nb
    int* counters;       // max(1, nb - 1), cleared by lbvh_build_into
    uint64_t* codes;
    uint64_t* codes2;
    uint32_t* idx;
    uint32_t* idx2;
    void* sort_tmp;      // radix_sort_temp_bytes<uint64_t>(n)
    void* box_tmp;       // bbox_temp_bytes(n)
    float* box;          // 6 floats
    int* err;
};

// Same construction as lbvh_build, into caller-provided buffers (no
// allocation).
void lbvh_build_into(const float* xyz, int n, int bucket, const LbvhBuffers& B, Lbvh& T, cudaStream_t s);

// A segmented LBVH over the scans of a scan project: a radix sort of the
// points' Morton codes (each in its scan's frame) and a stable sort by scan
// id, each scan's points padded to whole buckets (padding:
// NaN coordinates, index 0xffffffff), one Karras tree whose per-scan subtrees
// are the scans' search roots.  T.n counts the padded positions.
struct SegTree {
    Lbvh T;
    int nscans = 0, npoints = 0, npadded = 0, nbuckets = 0, bucket = 32, sbits = 0;
    SegInfo* segs = nullptr;           // device, per scan
    uint16_t* bucket_scan = nullptr;   // device, per bucket
    int* d_off = nullptr;              // device scan offsets
    int* d_pad = nullptr;              // device padded offsets
    float* box = nullptr;
    uint64_t *keys = nullptr, *keys2 = nullptr, *pkeys = nullptr, *bkeys = nullptr;
    uint32_t *idx = nullptr, *idx2 = nullptr;
    uint32_t *sid = nullptr, *sid2 = nullptr, *perm = nullptr, *perm2 = nullptr;
    void* sort_tmp = nullptr;
    int *bparent = nullptr, *counters = nullptr;
};

// Uploads the scan layout (offsets, padding, per-scan info and flip points)
// and sizes every buffer; synchronises the stream.  Run when the layout or the
// bucket size changes.
void lbvh_segmented_prepare(const std::vector<int64_t>& offsets, const std::vector<float>& flips, int bucket,
                            Workspace& ws, const std::string& tag, SegTree& out, cudaStream_t s);
// Builds the tree from device points: kernels and device-side copies only (no
// allocation, no host transfer), so it can be captured in a CUDA graph.
void lbvh_segmented_build(const float* xyz, SegTree& out, int* d_err, cudaStream_t s);

}  // namespace lvrgb
