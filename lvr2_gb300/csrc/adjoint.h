// adjoint.h -- gradients of the signed distance of AdaptiveKSearchSurface and
// Newton projection onto its zero level (adjoint.cu).
#pragma once
#include "lbvh.cuh"
#include "workspace.h"

namespace lvrgb {

// Outputs of distance_adjoint; any pointer may be null.  Row arrays are in
// the callers' query order (row = qs[i].w); gp / gn are accumulated in Morton
// order (float4, w unused) and must be zeroed by the caller.
struct AdjointOut {
    const float* gdist = nullptr;  // upstream gradient of the projected distance, per row
    const float* geucl = nullptr;  // upstream gradient of the Euclidean distance, per row
    float* dist = nullptr;         // projected distance, per row
    float* eucl = nullptr;         // Euclidean distance, per row
    float* gq = nullptr;           // d/dq, rows x 3
    float4* gp = nullptr;          // d/d point, Morton order
    float4* gn = nullptr;          // d/d normal, Morton order
};

// Forward distance (bit-identical to signed_distance_rows) and reverse-mode
// gradients for nq sorted queries (float4 xyz, w = row index bits) with the
// kd nearest points as a fixed neighbourhood.
void distance_adjoint(const Lbvh& T, const float4* normals, int kd, const float4* qs, int nq, const AdjointOut& out,
                      Workspace& ws, int* d_err, cudaStream_t s);

// `steps` Newton steps x <- x - d(x) n(x) from nq positions (float4 xyz,
// w = row index bits, any order); writes the final positions and the unit
// normal n(x) of the last step's neighbourhood, rows x 3 each (either may be
// null).
void project_to_surface(const Lbvh& T, const float4* normals, int kd, const float4* qs, int nq, int steps,
                        float* out_pos, float* out_normal, Workspace& ws, int* d_err, cudaStream_t s);

}  // namespace lvrgb
