// batch.cu -- the scan-project form of the normal estimation: all scans of a
// project (the per-scan CudaSurface runs of lvr2_cuda_normals' directory mode,
// src/tools/lvr2_cuda_normals/Main.cpp:166-190) go through one segmented LBVH
// build and one normals launch per search round, with per-scan flip points and
// kNN restricted to each scan.  No step reads data back to the host, so the
// whole pipeline can be captured in a CUDA graph.
#include "batch.h"

namespace lvrgb {

namespace {

__global__ void scatter_real_kernel(const float4* __restrict__ v, const float4* __restrict__ pts, int np,
                                    float* __restrict__ out) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= np) return;
    const uint32_t o = __float_as_uint(pts[j].w);
    if (o == 0xffffffffu) return;  // padding
    const float4 a = v[j];
    out[3 * size_t(o)] = a.x;
    out[3 * size_t(o) + 1] = a.y;
    out[3 * size_t(o) + 2] = a.z;
}

}  // namespace

void batch_prepare(const std::vector<int64_t>& offsets, const std::vector<float>& flips, const NormalsConfig& cfg,
                   int ki, int bucket, Workspace& ws, BatchRun& R, cudaStream_t s) {
    lbvh_segmented_prepare(offsets, flips, bucket, ws, "batch", R.tree, s);
    const size_t np = size_t(R.tree.T.n);
    R.raw = ws.get<float4>("batch.raw", np);
    R.normals = ws.get<float4>("batch.normals", np);
    R.kused = ws.get<int32_t>("batch.kused", np);
    R.nbr = ki > 0 ? ws.get<uint32_t>("batch.nbr", np * size_t(ki)) : nullptr;
    R.prepared_bucket = bucket;
    (void)cfg;
}

void batch_pipeline(const float* d_xyz, const NormalsConfig& cfg, int ki, int seed_radius, Workspace& ws,
                    BatchRun& R, int* d_err, uint32_t* d_stats, cudaStream_t s, cudaEvent_t* ev,
                    cudaEvent_t* round_ev, int collapse_after) {
    if (ev) LVRGB_CUDA(cudaEventRecord(ev[0], s));
    LVRGB_CUDA(cudaMemsetAsync(d_stats, 0, kNormalStats * sizeof(uint32_t), s));
    lbvh_segmented_build(d_xyz, R.tree, d_err, s);
    R.tree.T.seed_radius = seed_radius;
    if (ev) LVRGB_CUDA(cudaEventRecord(ev[1], s));
    const size_t np = size_t(R.tree.T.n);
    compute_normals_segmented(R.tree.T, R.tree.segs, R.tree.bucket_scan, cfg, R.raw, R.kused, ws, d_err, d_stats, s,
                              R.nbr, ki, round_ev, collapse_after);
    if (ev) LVRGB_CUDA(cudaEventRecord(ev[2], s));
    if (ki > 0)
        interpolate_from_lists(int(np), ki, R.nbr, R.raw, R.normals, s, R.tree.T.pts);
    else
        LVRGB_CUDA(cudaMemcpyAsync(R.normals, R.raw, sizeof(float4) * np, cudaMemcpyDeviceToDevice, s));
    if (ev) LVRGB_CUDA(cudaEventRecord(ev[3], s));
}

void batch_scatter_normals(const BatchRun& R, float* out, cudaStream_t s) {
    const int np = R.tree.T.n;
    if (np == 0) return;
    scatter_real_kernel<<<ceil_div(np, 256), 256, 0, s>>>(R.normals, R.tree.T.pts, np, out);
    LVRGB_LAUNCH_CHECK();
}

}  // namespace lvrgb
