// surface.h -- host launchers of the point-surface kernels (surface.cu).
#pragma once
#include <algorithm>
#include <atomic>
#include "lbvh.cuh"
#include "workspace.h"

namespace lvrgb {

struct NormalsConfig {
    int kn = 10;          // AdaptiveKSearchSurface kn
    int nem = 0;          // 0 LSQ plane, 2 iterative, 3 PCA (IPCA exact), 4 LBVH comparator (FP64, k = kn)
    int adaptive = 1;     // k = 2kn, 4kn, ... 32kn until the neighbourhood box is well formed
    float flip[3] = {0, 0, 0};
    float gap_threshold = 1e-3f;  // relative eigengap below which the eigensolve runs in FP64
    // Optional per point (Morton position, device): its own flip point when w != 0.
    const float4* flip_target = nullptr;
    // Launch shape of the one-warp-per-query kernel (k > kSmemHeapMax):
    // queries per warp tile (0: chosen from the query count) and the key
    // buffer's size in units of k (wide_capacity).  Tuning knobs only.
    int wide_tile = 0;
    int wide_slack = 2;
};

// Device counters written by compute_normals (uint32[16]):
//   [0..4] number of points whose plane was fitted in search round 1..5,
//   [5]    number of PCA eigensolves that fell back to FP64,
//   [6]    bounded large-k searches that found fewer than k points and ran again,
//   [8]    buckets scanned (per warp), [9] tree nodes expanded (per warp),
//   [10]   heap insertions (per query), [11] 32-candidate chunks scanned (per warp),
//   [12]   warp insertion rounds,
//   [13..15] searches with k > kSmemHeapMax (one warp per query): candidates
//          buffered, buffer compactions, queries.
constexpr int kNormalStats = 16;

// Normals in Morton order (float4, w = 0).  kused (optional, Morton order)
// receives the k of the search whose neighbourhood was used.  When nbr is
// given and ki <= 2 * kn, every point's ki nearest neighbours (Morton
// positions, ascending (d2, index)) are written column-wise to nbr[s * n + pos]
// for interpolate_from_lists.
void compute_normals(const Lbvh& T, const NormalsConfig& cfg, float4* normals, int32_t* kused, Workspace& ws,
                     int* d_err, uint32_t* d_stats, cudaStream_t s, uint32_t* nbr = nullptr, int ki = 0);

// Interpolation from the neighbour lists written by compute_normals.
// pad_pts (optional): the tree's points, whose padding positions get a zero
// normal.
void interpolate_from_lists(int n, int ki, const uint32_t* nbr, const float4* in, float4* out, cudaStream_t s,
                            const float4* pad_pts = nullptr);

// compute_normals over a segmented tree (one search tree per scan, per-scan
// flip points).  All rounds are launched without host synchronisation: each
// later round reads the previous round's retry count on the device, so the
// sequence can be captured in a CUDA graph.
// round_ev (optional, 6 events): recorded before round 1 and after each round
// that runs (rounds that do not run get the previous round's event; a
// collapsed launch's time falls on its first round).
// collapse_after = r (2 or 3): one search with the last round's k stands in
// for rounds r + 1 .. 5, which are tested on its prefixes (same results);
// 0: round by round.  collapse_after_round picks r from a previous run's
// fitted-per-round counts.
void compute_normals_segmented(const Lbvh& T, const SegInfo* segs, const uint16_t* bucket_scan,
                               const NormalsConfig& cfg, float4* normals, int32_t* kused, Workspace& ws, int* d_err,
                               uint32_t* d_stats, cudaStream_t s, uint32_t* nbr, int ki,
                               cudaEvent_t* round_ev = nullptr, int collapse_after = 0);
int collapse_after_round(int kn, int nem, int adaptive, const uint32_t fitted[5], int64_t n);

// Whether compute_normals* may collapse rounds (lvrgb_debug_round_collapse).
extern std::atomic<int> g_round_collapse;

// out_i = normalize(in_i + sum_{j in kNN_ki(p_i)} in_j), Morton order.
void interpolate_normals(const Lbvh& T, int ki, const float4* in, float4* out, Workspace& ws, int* d_err,
                         cudaStream_t s);

// Sorts nq AoS query points into Morton order relative to the tree's box.
// qs[i] = (x, y, z, row index bits).  d_box: 6 floats (min, max).
void sort_queries(const float* q, int nq, const float* d_box, float4* qs, Workspace& ws, cudaStream_t s);

// k nearest neighbours for sorted queries; rows (by qs[i].w) of idx (original
// indices, 0xffffffff padding) and dist (sqrt of d2, +inf padding), ascending.
// radius2 (> 0): only points with d2 < radius2 (a radius search).
void knn_rows(const Lbvh& T, const float4* qs, int nq, int k, uint32_t* idx, float* dist, int32_t* count,
              Workspace& ws, int* d_err, cudaStream_t s, float radius2 = INFINITY);

// knn_rows with the heaps in shared memory only (k <= kSmemHeapMax) and no
// workspace: allocates nothing.
void knn_rows_smem(const Lbvh& T, const float4* qs, int nq, int k, uint32_t* idx, float* dist, int32_t* count,
                   int* d_err, cudaStream_t s);

// PointsetSurface::getInterpolatedNormal for sorted queries; out rows float3.
void interpolated_normal_rows(const Lbvh& T, const float4* normals, int ki, const float4* qs, int nq,
                              float* out, Workspace& ws, int* d_err, cudaStream_t s);

// Flip points from scan poses (AdaptiveKSearchSurface::parseScanPoses and the
// pose-tree flip, AdaptiveKSearchSurface.tcc:94-139, 252-265): per point
// (Morton position) the cloud point indexed by its nearest pose's index, w = 1,
// or w = 0 when that index is >= n.  d_poses: np x 3 (device).
void pose_flip_targets(const Lbvh& T, const float* d_poses, int np, float4* out, cudaStream_t s);

// LBVHIndex::calculate_normals: the nem 4 fit from given neighbour lists
// (device arrays: queries nq x 3, cnt[nq] <= k, idx nq x k input indices < T.n,
// slot 0 left out as the query itself), flipped toward flip; out nq x 3.
void normals_from_lists(const Lbvh& T, const float* queries, int nq, int k, const uint32_t* cnt, const uint32_t* idx,
                        const float flip[3], float* out, cudaStream_t s);
// out[0] = the largest count, out[1] = the largest index among the used
// entries (first min(cnt, k) of each row) of device neighbour lists.
void list_extent(const uint32_t* cnt, const uint32_t* idx, int nq, int k, Workspace& ws, uint32_t out[2],
                 cudaStream_t s);

// Common launch plan for the per-lane heaps: heaps of up to kSmemHeapMax
// entries live in shared memory, larger ones in a global scratch buffer.
constexpr int kWarpsPerBlock = 4;
constexpr int kSmemHeapMax = 96;
struct HeapPlan {
    int blocks = 0;
    size_t smem = 0;
    unsigned long long* gheap = nullptr;
};
HeapPlan plan_heap(int nq, int K, Workspace& ws);

// Persistent form of a per-lane kNN launch (kernels whose tile loop takes
// first_tile / next_tile): the grid is capped at the blocks that are resident
// at once, and warps take their tiles from the returned counter, zeroed here
// on the stream.  Lowers P.blocks in place.  The kernel's dynamic shared
// memory attribute must already be set.
template <typename Kernel>
int* persistent_tiles(Kernel k, int threads, size_t smem, int& blocks, Workspace& ws, cudaStream_t s) {
    int per_sm = 0, dev = 0, sms = 0;
    LVRGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, threads, smem));
    LVRGB_CUDA(cudaGetDevice(&dev));
    LVRGB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    if (per_sm > 0 && sms > 0) blocks = std::min(blocks, per_sm * sms);
    int* c = ws.get<int>("knn.tiles", 1);
    LVRGB_CUDA(cudaMemsetAsync(c, 0, sizeof(int), s));
    return c;
}
template <typename Kernel>
int* persistent_tiles(Kernel k, HeapPlan& P, Workspace& ws, cudaStream_t s) {
    return persistent_tiles(k, kWarpsPerBlock * 32, P.smem, P.blocks, ws, s);
}

}  // namespace lvrgb
