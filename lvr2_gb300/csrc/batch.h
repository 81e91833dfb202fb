// batch.h -- normals for every scan of a scan project in one pass over a
// segmented LBVH (batch.cu).
#pragma once
#include <vector>

#include "lbvh_build.h"
#include "surface.h"

namespace lvrgb {

struct BatchRun {
    SegTree tree;
    int prepared_bucket = 0;    // bucket size the tree buffers were prepared for
    float4* raw = nullptr;      // normals before interpolation, padded Morton order
    float4* normals = nullptr;  // final normals, padded Morton order
    int32_t* kused = nullptr;
    uint32_t* nbr = nullptr;    // interpolation lists (ki x padded n)
};

// Uploads the scan layout and sizes all buffers (outside any graph capture).
void batch_prepare(const std::vector<int64_t>& offsets, const std::vector<float>& flips, const NormalsConfig& cfg,
                   int ki, int bucket, Workspace& ws, BatchRun& R, cudaStream_t s);

// Per-stage device events recorded by batch_pipeline when ev != nullptr:
// ev[0] start, ev[1] after the tree, ev[2] after the normals, ev[3] end.
// Tree, normals and interpolation for a prepared batch.
// round_ev (6 events, optional) and collapse_after: see
// compute_normals_segmented.
void batch_pipeline(const float* d_xyz, const NormalsConfig& cfg, int ki, int seed_radius, Workspace& ws,
                    BatchRun& R, int* d_err, uint32_t* d_stats, cudaStream_t s, cudaEvent_t* ev = nullptr,
                    cudaEvent_t* round_ev = nullptr, int collapse_after = 0);

// Final normals in input order (AoS, npoints x 3).
void batch_scatter_normals(const BatchRun& R, float* out, cudaStream_t s);

}  // namespace lvrgb
