// chunks.cu -- signed distance at the grid vertices of every chunk (scan) of a
// batch against that chunk's own points and normals, in one pass: the GPU
// block of LargeScaleReconstruction::createChunk
// (LargeScaleReconstruction.tcc:636-688), which builds one GpuSurface per
// chunk, computes its normals and evaluates the chunk grid's query points,
// retrying smaller chunks when the GPU runs out of memory.  Here all chunks
// share the segmented LBVH of the batch:
//   1. queries get 63-bit Morton codes in their chunk's frame and are sorted
//      by code, then stably by chunk (each chunk contiguous, Morton ordered);
//   2. one warp serves 32 consecutive sorted queries; lanes of each chunk in
//      the warp search that chunk's subtree only, seeded at the chunk's bucket
//      whose key is nearest below the query group's code;
//   3. the kd nearest points and normals give AdaptiveKSearchSurface::distance
//      (AdaptiveKSearchSurface.tcc:414-457) and the invalid flag of
//      PointsetGrid::calcDistanceValues (PointsetGrid.tcc:133-140), with the
//      operations of sdf_kernel.
#include <algorithm>

#include "chunks.h"
#include "primitives.cuh"
#include "surface.h"

namespace lvrgb {

namespace {

__device__ __forceinline__ int chunk_of(const int64_t* __restrict__ off, int S, int64_t i) {
    int lo = 0, hi = S;  // off[lo] <= i < off[hi]
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(off + mid) <= i) lo = mid; else hi = mid;
    }
    return lo;
}

__global__ void query_codes_kernel(const float* __restrict__ q, int nq, const int64_t* __restrict__ qoff, int S,
                                   const float* __restrict__ box, uint64_t* __restrict__ codes,
                                   uint32_t* __restrict__ idx) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nq) return;
    const int c = chunk_of(qoff, S, i);
    const float* bx = box + 6 * c;
    const float ext = fmaxf(fmaxf(bx[3] - bx[0], bx[4] - bx[1]), bx[5] - bx[2]);
    codes[i] = morton63(q[3 * size_t(i)], q[3 * size_t(i) + 1], q[3 * size_t(i) + 2], bx[0], bx[1], bx[2],
                        morton_scale(ext));
    idx[i] = uint32_t(i);
}

__global__ void query_chunks_kernel(const uint32_t* __restrict__ sidx, int nq, const int64_t* __restrict__ qoff, int S,
                                    uint32_t* __restrict__ cid, uint32_t* __restrict__ pos) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nq) return;
    cid[j] = uint32_t(chunk_of(qoff, S, sidx[j]));
    pos[j] = uint32_t(j);
}

__global__ void query_pack_kernel(const float* __restrict__ q, const uint64_t* __restrict__ scodes,
                                  const uint32_t* __restrict__ sidx, const uint32_t* __restrict__ cid,
                                  const uint32_t* __restrict__ perm, int nq, float4* __restrict__ qs,
                                  uint32_t* __restrict__ qchunk, uint64_t* __restrict__ qcode) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nq) return;
    const uint32_t j = perm ? perm[t] : uint32_t(t);
    const uint32_t o = sidx[j];
    qs[t] = make_float4(q[3 * size_t(o)], q[3 * size_t(o) + 1], q[3 * size_t(o) + 2], __uint_as_float(o));
    qchunk[t] = cid[t];
    qcode[t] = scodes[j];
}

// Bucket of [blo, bhi] whose first code is the largest <= code (blo when
// none is): a warp 32-ary search (warp-uniform inputs and result).
__device__ __forceinline__ int seed_bucket_in(const uint64_t* __restrict__ bkeys, int blo, int bhi, uint64_t code) {
    const int lane = threadIdx.x & 31;
    int lo = blo, hi = bhi + 1;
    while (hi - lo > 1) {
        const int step = (hi - lo + 31) / 32;
        const int probe = lo + lane * step;
        const bool le = probe < hi && __ldg(bkeys + probe) <= code;
        const int c = __popc(__ballot_sync(kFull, le));
        if (c == 0) return lo;
        lo = lo + (c - 1) * step;
        hi = min(hi, lo + step);
    }
    return lo;
}

struct ChunkSdfArgs {
    Lbvh T;
    int K;
    const SegInfo* segs;
    const uint64_t* bkeys;
    const float4* normals;  // padded Morton order
    const float4* qs;
    const uint32_t* qchunk;
    const uint64_t* qcode;
    int nq;
    double limit;  // 1.75 * voxel size
    float* dist;
    uint8_t* invalid;
    unsigned long long* gheap;
    int* err;
    int* tiles = nullptr;  // tile counter of a persistent launch
};

__global__ void __launch_bounds__(kWarpsPerBlock * 32) chunk_sdf_kernel(ChunkSdfArgs A) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31;
    const WarpCtx ctx = warp_ctx<kWarpsPerBlock>(smem, A.gheap, A.K);
    for (int tile = first_tile<kWarpsPerBlock>(A.tiles); tile * 32 < A.nq;
         tile = next_tile<kWarpsPerBlock>(A.tiles, tile)) {
        const int qi = tile * 32 + lane;
        const bool active = qi < A.nq;
        const float4 q = active ? A.qs[qi] : make_float4(0, 0, 0, 0);
        const int sc = active ? int(A.qchunk[qi]) : -1;
        const uint64_t code = active ? A.qcode[qi] : 0ull;
        LaneHeap heap;
        heap.init(ctx.heap, A.K);
        unsigned remaining = __ballot_sync(kFull, active);
        while (remaining) {
            const int leader = __ffs(remaining) - 1;
            const int s = __shfl_sync(kFull, sc, leader);
            const unsigned grp = __ballot_sync(kFull, active && sc == s);
            remaining &= ~grp;
            const SegInfo g = A.segs[s];
            const uint64_t lcode = __shfl_sync(kFull, code, leader);
            const int seed = seed_bucket_in(A.bkeys, g.blo, g.bhi, lcode);
            TravStats st;
            knn_traverse(A.T, q.x, q.y, q.z, (grp >> lane) & 1u, heap, ctx.stage, A.err, st, seed, g.root, g.blo,
                         g.bhi);
        }
        if (!active) continue;
        heap.sort_ascending();
        float px = 0, py = 0, pz = 0, nx = 0, ny = 0, nz = 0;
        const int cnt = heap.real;
        for (int s = 0; s < cnt; s++) {
            const uint32_t j = __ldg(A.T.inv + key_idx(heap.at(s)));
            const float4 p = __ldg(A.T.pts + j);
            const float4 nn = __ldg(A.normals + j);
            px = __fadd_rn(px, p.x); py = __fadd_rn(py, p.y); pz = __fadd_rn(pz, p.z);
            nx = __fadd_rn(nx, nn.x); ny = __fadd_rn(ny, nn.y); nz = __fadd_rn(nz, nn.z);
        }
        float proj, eu;
        if (cnt == 0) {
            proj = eu = FLT_MAX;
        } else {
            const float c = float(cnt);
            nx = __fdiv_rn(nx, c); ny = __fdiv_rn(ny, c); nz = __fdiv_rn(nz, c);
            px = __fdiv_rn(px, c); py = __fdiv_rn(py, c); pz = __fdiv_rn(pz, c);
            if (!(nx == 0.0f && ny == 0.0f && nz == 0.0f)) {
                const float len = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(nx, nx), __fmul_rn(ny, ny)), __fmul_rn(nz, nz)));
                nx = __fdiv_rn(nx, len); ny = __fdiv_rn(ny, len); nz = __fdiv_rn(nz, len);
            }
            const float dx = __fsub_rn(q.x, px), dy = __fsub_rn(q.y, py), dz = __fsub_rn(q.z, pz);
            proj = __fadd_rn(__fadd_rn(__fmul_rn(dx, nx), __fmul_rn(dy, ny)), __fmul_rn(dz, nz));
            eu = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz)));
        }
        const uint32_t row = __float_as_uint(q.w);
        A.dist[row] = proj;
        A.invalid[row] = double(eu) > A.limit ? 1 : 0;
    }
}

template <typename Kernel>
void set_smem(Kernel k, size_t bytes) {
    if (bytes > 48 * 1024) LVRGB_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(bytes)));
}

}  // namespace

void chunk_grid_distances(const SegTree& tree, const float4* normals, int kd, const float* d_q,
                          const int64_t* d_qoff, int nq, float vs, float* dist, uint8_t* invalid, Workspace& ws,
                          int* d_err, cudaStream_t s) {
    if (nq == 0) return;
    const int S = tree.nscans;
    uint64_t* codes = ws.get<uint64_t>("chunk.codes", size_t(nq));
    uint64_t* codes2 = ws.get<uint64_t>("chunk.codes2", size_t(nq));
    uint32_t* idx = ws.get<uint32_t>("chunk.idx", size_t(nq));
    uint32_t* idx2 = ws.get<uint32_t>("chunk.idx2", size_t(nq));
    uint32_t* cid = ws.get<uint32_t>("chunk.cid", size_t(nq));
    uint32_t* cid2 = ws.get<uint32_t>("chunk.cid2", size_t(nq));
    uint32_t* perm = ws.get<uint32_t>("chunk.perm", size_t(nq));
    uint32_t* perm2 = ws.get<uint32_t>("chunk.perm2", size_t(nq));
    void* tmp = ws.get<unsigned char>("chunk.sorttmp", std::max(radix_sort_temp_bytes<uint64_t>(size_t(nq)),
                                                                radix_sort_temp_bytes<uint32_t>(size_t(nq))));
    query_codes_kernel<<<ceil_div(nq, 256), 256, 0, s>>>(d_q, nq, d_qoff, S, tree.box, codes, idx);
    LVRGB_LAUNCH_CHECK();
    const bool alt = radix_sort_pairs<uint64_t>(codes, idx, codes2, idx2, size_t(nq), 0, 63, tmp, s);
    const uint64_t* scodes = alt ? codes2 : codes;
    const uint32_t* sidx = alt ? idx2 : idx;
    query_chunks_kernel<<<ceil_div(nq, 256), 256, 0, s>>>(sidx, nq, d_qoff, S, cid, perm);
    LVRGB_LAUNCH_CHECK();
    const uint32_t* c_sorted = cid;
    const uint32_t* p_sorted = nullptr;
    if (tree.sbits > 0) {
        const bool alt2 = radix_sort_pairs<uint32_t>(cid, perm, cid2, perm2, size_t(nq), 0, tree.sbits, tmp, s);
        c_sorted = alt2 ? cid2 : cid;
        p_sorted = alt2 ? perm2 : perm;
    }
    float4* qs = ws.get<float4>("chunk.qs", size_t(nq));
    uint32_t* qchunk = ws.get<uint32_t>("chunk.qchunk", size_t(nq));
    uint64_t* qcode = ws.get<uint64_t>("chunk.qcode", size_t(nq));
    query_pack_kernel<<<ceil_div(nq, 256), 256, 0, s>>>(d_q, scodes, sidx, c_sorted, p_sorted, nq, qs, qchunk,
                                                       qcode);
    LVRGB_LAUNCH_CHECK();
    ChunkSdfArgs A;
    A.T = tree.T;
    A.K = kd > 0 ? kd : 1;
    A.segs = tree.segs;
    A.bkeys = tree.bkeys;
    A.normals = normals;
    A.qs = qs;
    A.qchunk = qchunk;
    A.qcode = qcode;
    A.nq = nq;
    A.limit = 1.75 * double(vs);
    A.dist = dist;
    A.invalid = invalid;
    A.err = d_err;
    HeapPlan P = plan_heap(nq, A.K, ws);
    A.gheap = P.gheap;
    set_smem(chunk_sdf_kernel, P.smem);
    A.tiles = persistent_tiles(chunk_sdf_kernel, P, ws, s);
    chunk_sdf_kernel<<<P.blocks, kWarpsPerBlock * 32, P.smem, s>>>(A);
    LVRGB_LAUNCH_CHECK();
}

}  // namespace lvrgb
