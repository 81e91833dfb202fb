// lbvh.cu -- LBVH construction: bounding box, 63-bit Morton codes, device
// radix sort, Karras radix tree over point buckets, bottom-up child boxes.
#include "lbvh_build.h"

#include <algorithm>
#include <stdexcept>
#include <vector>
#include "primitives.cuh"

namespace lvrgb {

namespace {

__global__ void morton_kernel(const float* __restrict__ xyz, int n, const float* __restrict__ box,
                              uint64_t* __restrict__ codes, uint32_t* __restrict__ idx) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float ext = fmaxf(fmaxf(box[3] - box[0], box[4] - box[1]), box[5] - box[2]);
    codes[i] = morton63(xyz[3 * size_t(i)], xyz[3 * size_t(i) + 1], xyz[3 * size_t(i) + 2], box[0], box[1], box[2],
                        morton_scale(ext));
    idx[i] = uint32_t(i);
}

__global__ void gather_sorted_kernel(const float* __restrict__ xyz, const uint32_t* __restrict__ order, int n,
                                     float4* __restrict__ pts, uint32_t* __restrict__ inv) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    uint32_t o = order[j];
    pts[j] = make_float4(xyz[3 * size_t(o)], xyz[3 * size_t(o) + 1], xyz[3 * size_t(o) + 2], __uint_as_float(o));
    inv[o] = uint32_t(j);
}

// Common-prefix length of buckets i and j in the key [scan id: sbits bits]
// [first point's 63-bit Morton code] [bucket index: 32 bits] -- the bucket
// index breaks ties between equal codes (Karras 2012).  Without per-bucket
// scan ids (bscan == nullptr) sbits is 0.
__device__ __forceinline__ int delta(const uint64_t* __restrict__ keys, const uint16_t* __restrict__ bscan, int sbits,
                                     int nb, int i, int j) {
    if (j < 0 || j >= nb) return -1;
    if (bscan) {
        const unsigned si = bscan[i], sj = bscan[j];
        if (si != sj) return __clz(int(si ^ sj)) - (32 - sbits);
    }
    const uint64_t ki = keys[i], kj = keys[j];
    if (ki != kj) return sbits + __clzll((long long)(ki ^ kj)) - 1;
    return sbits + 63 + __clz(int(uint32_t(i) ^ uint32_t(j)));
}

// Karras radix tree over the nb bucket keys.  With per-bucket scan ids, the
// node whose range is exactly one scan's buckets becomes that scan's root.
__global__ void karras_kernel(const uint64_t* __restrict__ keys, const uint16_t* __restrict__ bscan, int sbits, int nb,
                              TreeNode* __restrict__ nodes, int* __restrict__ bparent, SegInfo* __restrict__ segs) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nb - 1) return;
    const int dir = (delta(keys, bscan, sbits, nb, i, i + 1) - delta(keys, bscan, sbits, nb, i, i - 1)) >= 0 ? 1 : -1;
    const int dmin = delta(keys, bscan, sbits, nb, i, i - dir);
    int lmax = 2;
    while (delta(keys, bscan, sbits, nb, i, i + lmax * dir) > dmin) lmax <<= 1;
    int l = 0;
    for (int t = lmax >> 1; t >= 1; t >>= 1)
        if (delta(keys, bscan, sbits, nb, i, i + (l + t) * dir) > dmin) l += t;
    const int j = i + l * dir;
    const int dnode = delta(keys, bscan, sbits, nb, i, j);
    int s = 0;
    int div = 2;
    int t = (l + div - 1) / div;
    while (true) {
        if (delta(keys, bscan, sbits, nb, i, i + (s + t) * dir) > dnode) s += t;
        if (t == 1) break;
        div <<= 1;
        t = (l + div - 1) / div;
    }
    const int gamma = i + s * dir + (dir < 0 ? -1 : 0);
    const int lo = min(i, j), hi = max(i, j);
    int left, right;
    if (lo == gamma) {
        left = -1 - gamma;
        bparent[gamma] = (i << 1) | 0;
    } else {
        left = gamma;
        nodes[gamma].d.z = (i << 1) | 0;
    }
    if (hi == gamma + 1) {
        right = -1 - (gamma + 1);
        bparent[gamma + 1] = (i << 1) | 1;
    } else {
        right = gamma + 1;
        nodes[gamma + 1].d.z = (i << 1) | 1;
    }
    nodes[i].d.x = left;
    nodes[i].d.y = right;
    if (i == 0) nodes[0].d.z = -1;
    if (segs) {
        const int sc = bscan[lo];
        if (segs[sc].blo == lo && segs[sc].bhi == hi) segs[sc].root = i;
    }
}

__global__ void bucket_keys_kernel(const uint64_t* __restrict__ codes, int bucket, int nb, uint64_t* __restrict__ bkeys) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b < nb) bkeys[b] = codes[size_t(b) * bucket];
}

__device__ __forceinline__ void write_child_box(TreeNode* nd, int side, const float* lo, const float* hi) {
    float* f = reinterpret_cast<float*>(nd);
    const int o = side ? 6 : 0;
    f[o + 0] = lo[0]; f[o + 1] = lo[1]; f[o + 2] = lo[2];
    f[o + 3] = hi[0]; f[o + 4] = hi[1]; f[o + 5] = hi[2];
}

// One warp per bucket: reduce the bucket box, then lane 0 climbs the tree;
// the second child to arrive at a node merges both boxes and continues.
__global__ void bounds_kernel(const float4* __restrict__ pts, int n, int bucket, int nb, TreeNode* nodes,
                              const int* __restrict__ bparent, int* __restrict__ counters, int* __restrict__ err) {
    const int lane = threadIdx.x & 31;
    const int b = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (b >= nb) return;
    const int first = b * bucket;
    int cnt = min(bucket, n - first);
    float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    for (int j = lane; j < cnt; j += 32) {
        float4 p = pts[first + j];
        lo[0] = fminf(lo[0], p.x); lo[1] = fminf(lo[1], p.y); lo[2] = fminf(lo[2], p.z);
        hi[0] = fmaxf(hi[0], p.x); hi[1] = fmaxf(hi[1], p.y); hi[2] = fmaxf(hi[2], p.z);
    }
#pragma unroll
    for (int c = 0; c < 3; c++)
        for (int o = 16; o > 0; o >>= 1) {
            lo[c] = fminf(lo[c], __shfl_xor_sync(kFull, lo[c], o));
            hi[c] = fmaxf(hi[c], __shfl_xor_sync(kFull, hi[c], o));
        }
    if (lane != 0 || nb == 1) return;
    int pw = bparent[b];
    // The path to the root of a radix tree over (16-bit scan id, 63-bit code,
    // 32-bit index) keys has fewer than 16 + 63 + 32 links; the bound only
    // guards against a malformed parent chain.
    for (int hops = 0; pw >= 0; hops++) {
        if (hops > 128) {
            atomicOr(err, kErrWalk);
            return;
        }
        const int p = pw >> 1, side = pw & 1;
        TreeNode* nd = nodes + p;
        write_child_box(nd, side, lo, hi);
        __threadfence();
        if (atomicAdd(counters + p, 1) == 0) return;
        __threadfence();
        const float* f = reinterpret_cast<const float*>(nd);
        float o[12];
#pragma unroll
        for (int k = 0; k < 12; k++) o[k] = __ldcg(f + k);
        lo[0] = fminf(o[0], o[6]); lo[1] = fminf(o[1], o[7]); lo[2] = fminf(o[2], o[8]);
        hi[0] = fmaxf(o[3], o[9]); hi[1] = fmaxf(o[4], o[10]); hi[2] = fmaxf(o[5], o[11]);
        pw = __ldcg(&nd->d.z);
    }
}

// ---- segmented (multi-scan) construction --------------------------------

// Scan of position i from sorted offsets off[0..S] (binary search).
__device__ __forceinline__ int scan_of(const int* __restrict__ off, int S, int i) {
    int lo = 0, hi = S;  // off[lo] <= i < off[hi]
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(off + mid) <= i) lo = mid; else hi = mid;
    }
    return lo;
}

// One block per scan: the scan's bounding box.
__global__ void seg_bbox_kernel(const float* __restrict__ xyz, const int* __restrict__ off, float* __restrict__ box) {
    const int s = blockIdx.x;
    const int a = off[s], b = off[s + 1];
    float mn[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, mx[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    for (int i = a + threadIdx.x; i < b; i += blockDim.x)
        for (int c = 0; c < 3; c++) {
            const float v = xyz[3 * size_t(i) + c];
            mn[c] = fminf(mn[c], v);
            mx[c] = fmaxf(mx[c], v);
        }
    __shared__ float sh[32][6];
    for (int c = 0; c < 3; c++)
        for (int o = 16; o > 0; o >>= 1) {
            mn[c] = fminf(mn[c], __shfl_down_sync(kFull, mn[c], o));
            mx[c] = fmaxf(mx[c], __shfl_down_sync(kFull, mx[c], o));
        }
    if ((threadIdx.x & 31) == 0)
        for (int c = 0; c < 3; c++) { sh[threadIdx.x >> 5][c] = mn[c]; sh[threadIdx.x >> 5][3 + c] = mx[c]; }
    __syncthreads();
    if (threadIdx.x < 6) {
        float v = sh[0][threadIdx.x];
        for (int w = 1; w < int(blockDim.x >> 5); w++)
            v = threadIdx.x < 3 ? fminf(v, sh[w][threadIdx.x]) : fmaxf(v, sh[w][threadIdx.x]);
        box[6 * s + threadIdx.x] = v;
    }
}

// Morton code of every point in its own scan's frame (sorted first; the
// stable sort by scan id that follows groups the scans).
__global__ void seg_morton_kernel(const float* __restrict__ xyz, int n, const int* __restrict__ off, int S,
                                  const float* __restrict__ box, uint64_t* __restrict__ keys, uint32_t* __restrict__ idx) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int s = scan_of(off, S, i);
    const float* bx = box + 6 * s;
    const float ext = fmaxf(fmaxf(bx[3] - bx[0], bx[4] - bx[1]), bx[5] - bx[2]);
    keys[i] = morton63(xyz[3 * size_t(i)], xyz[3 * size_t(i) + 1], xyz[3 * size_t(i) + 2], bx[0], bx[1], bx[2],
                       morton_scale(ext));
    idx[i] = uint32_t(i);
}

// Scan id of every Morton-sorted point, and its position as the value.
__global__ void seg_scan_ids_kernel(const uint32_t* __restrict__ sidx, int n, const int* __restrict__ off, int S,
                                    uint32_t* __restrict__ sid, uint32_t* __restrict__ pos) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    sid[j] = uint32_t(scan_of(off, S, int(sidx[j])));
    pos[j] = uint32_t(j);
}

// Final position t (scan-grouped, Morton order within a scan) -> padded
// position pad_off[s] + (t - off[s]).  perm: Morton-sorted position of t
// (identity when null).
__global__ void seg_gather_kernel(const float* __restrict__ xyz, const uint64_t* __restrict__ scodes,
                                  const uint32_t* __restrict__ sidx, const uint32_t* __restrict__ sid,
                                  const uint32_t* __restrict__ perm, int n, const int* __restrict__ off,
                                  const int* __restrict__ pad_off, float4* __restrict__ pts, uint32_t* __restrict__ inv,
                                  uint64_t* __restrict__ pkeys) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const uint32_t j = perm ? perm[t] : uint32_t(t);
    const int s = int(sid[t]);
    const uint32_t o = sidx[j];
    const int pp = pad_off[s] + (t - off[s]);
    pts[pp] = make_float4(xyz[3 * size_t(o)], xyz[3 * size_t(o) + 1], xyz[3 * size_t(o) + 2], __uint_as_float(o));
    inv[o] = uint32_t(pp);
    pkeys[pp] = scodes[j];
}

// Padding after each scan's points: NaN coordinates (never within any bound)
// and index 0xffffffff.
__global__ void seg_pad_kernel(int np, const int* __restrict__ off, const int* __restrict__ pad_off, int S,
                               float4* __restrict__ pts) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= np) return;
    const int s = scan_of(pad_off, S, p);
    if (p - pad_off[s] >= off[s + 1] - off[s]) {
        const float nan = __int_as_float(0x7fffffff);
        pts[p] = make_float4(nan, nan, nan, __uint_as_float(0xffffffffu));
    }
}

__global__ void seg_bucket_keys_kernel(const uint64_t* __restrict__ pkeys, int bucket, int nb,
                                       const int* __restrict__ pad_off, int S, uint64_t* __restrict__ bkeys,
                                       uint16_t* __restrict__ bucket_scan) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    bkeys[b] = pkeys[size_t(b) * bucket];
    bucket_scan[b] = uint16_t(scan_of(pad_off, S, b * bucket));
}

}  // namespace

void lbvh_build(const float* xyz, int n, int bucket, Workspace& ws, const std::string& tag, Lbvh& T,
                float* d_box, int* d_err, cudaStream_t s) {
    if (bucket < 1 || bucket > 32) bucket = 32;
    T.n = n;
    T.bucket = bucket;
    T.nbuckets = n > 0 ? (n + bucket - 1) / bucket : 0;
    float4* pts = ws.get<float4>(tag + ".pts", size_t(n));
    uint32_t* inv = ws.get<uint32_t>(tag + ".inv", size_t(n));
    const int nb = T.nbuckets;
    TreeNode* nodes = ws.get<TreeNode>(tag + ".nodes", size_t(nb > 1 ? nb - 1 : 1));
    T.pts = pts;
    T.inv = inv;
    T.nodes = nodes;
    if (n == 0) return;

    void* btmp = ws.get<unsigned char>("lbvh.boxtmp", bbox_temp_bytes(size_t(n)));
    bbox_float3(xyz, size_t(n), 3, d_box, btmp, s);

    uint64_t* codes = ws.get<uint64_t>("lbvh.codes", size_t(n));
    uint64_t* codes2 = ws.get<uint64_t>("lbvh.codes2", size_t(n));
    uint32_t* idx = ws.get<uint32_t>("lbvh.idx", size_t(n));
    uint32_t* idx2 = ws.get<uint32_t>("lbvh.idx2", size_t(n));
    morton_kernel<<<ceil_div(n, 256), 256, 0, s>>>(xyz, n, d_box, codes, idx);
    LVRGB_LAUNCH_CHECK();
    void* stmp = ws.get<unsigned char>("lbvh.sorttmp", radix_sort_temp_bytes<uint64_t>(size_t(n)));
    bool alt = radix_sort_pairs<uint64_t>(codes, idx, codes2, idx2, size_t(n), 0, 63, stmp, s);
    const uint64_t* scodes = alt ? codes2 : codes;
    const uint32_t* sidx = alt ? idx2 : idx;
    gather_sorted_kernel<<<ceil_div(n, 256), 256, 0, s>>>(xyz, sidx, n, pts, inv);
    LVRGB_LAUNCH_CHECK();
    uint64_t* bkeys = ws.get<uint64_t>(tag + ".bkeys", size_t(nb));
    T.bkeys = bkeys;
    bucket_keys_kernel<<<ceil_div(nb, 256), 256, 0, s>>>(scodes, bucket, nb, bkeys);
    LVRGB_LAUNCH_CHECK();

    int* bparent = ws.get<int>("lbvh.bparent", size_t(nb));
    if (nb == 1) {
        LVRGB_CUDA(cudaMemsetAsync(bparent, 0xff, sizeof(int), s));
        return;
    }
    int* counters = ws.get<int>("lbvh.counters", size_t(nb - 1));
    LVRGB_CUDA(cudaMemsetAsync(counters, 0, sizeof(int) * size_t(nb - 1), s));
    karras_kernel<<<ceil_div(nb - 1, 256), 256, 0, s>>>(bkeys, nullptr, 0, nb, nodes, bparent, nullptr);
    LVRGB_LAUNCH_CHECK();
    bounds_kernel<<<ceil_div(size_t(nb) * 32, 256), 256, 0, s>>>(pts, n, bucket, nb, nodes, bparent, counters,
                                                                 d_err);
    LVRGB_LAUNCH_CHECK();
}

void lbvh_build_into(const float* xyz, int n, int bucket, const LbvhBuffers& B, Lbvh& T, cudaStream_t s) {
    if (bucket < 1 || bucket > 32) bucket = 32;
    T.n = n;
    T.bucket = bucket;
    T.nbuckets = n > 0 ? (n + bucket - 1) / bucket : 0;
    T.pts = B.pts;
    T.inv = B.inv;
    T.nodes = B.nodes;
    T.bkeys = B.bkeys;
    if (n == 0) return;
    const int nb = T.nbuckets;
    bbox_float3(xyz, size_t(n), 3, B.box, B.box_tmp, s);
    morton_kernel<<<ceil_div(n, 256), 256, 0, s>>>(xyz, n, B.box, B.codes, B.idx);
    LVRGB_LAUNCH_CHECK();
    bool alt = radix_sort_pairs<uint64_t>(B.codes, B.idx, B.codes2, B.idx2, size_t(n), 0, 63, B.sort_tmp, s);
    const uint64_t* scodes = alt ? B.codes2 : B.codes;
    const uint32_t* sidx = alt ? B.idx2 : B.idx;
    gather_sorted_kernel<<<ceil_div(n, 256), 256, 0, s>>>(xyz, sidx, n, B.pts, B.inv);
    LVRGB_LAUNCH_CHECK();
    bucket_keys_kernel<<<ceil_div(nb, 256), 256, 0, s>>>(scodes, bucket, nb, B.bkeys);
    LVRGB_LAUNCH_CHECK();
    if (nb == 1) {
        LVRGB_CUDA(cudaMemsetAsync(B.bparent, 0xff, sizeof(int), s));
        return;
    }
    LVRGB_CUDA(cudaMemsetAsync(B.counters, 0, sizeof(int) * size_t(nb - 1), s));
    karras_kernel<<<ceil_div(nb - 1, 256), 256, 0, s>>>(B.bkeys, nullptr, 0, nb, B.nodes, B.bparent, nullptr);
    LVRGB_LAUNCH_CHECK();
    bounds_kernel<<<ceil_div(size_t(nb) * 32, 256), 256, 0, s>>>(B.pts, n, bucket, nb, B.nodes, B.bparent, B.counters,
                                                                 B.err);
    LVRGB_LAUNCH_CHECK();
}

void lbvh_segmented_prepare(const std::vector<int64_t>& offsets, const std::vector<float>& flips, int bucket,
                            Workspace& ws, const std::string& tag, SegTree& out, cudaStream_t s) {
    if (bucket < 1 || bucket > 32) bucket = 32;
    const int S = int(offsets.size()) - 1;
    if (S < 1 || S > 65535) throw std::invalid_argument("scan count must be in 1..65535");
    const int n = int(offsets[size_t(S)]);
    std::vector<int> off(size_t(S) + 1), pad_off(size_t(S) + 1);
    std::vector<SegInfo> segs(static_cast<size_t>(S));
    int np = 0, nb = 0;
    for (int k = 0; k < S; k++) {
        const int64_t a = offsets[size_t(k)], b = offsets[size_t(k) + 1];
        if (b <= a) throw std::invalid_argument("scan offsets must be strictly increasing");
        off[size_t(k)] = int(a);
        pad_off[size_t(k)] = np;
        const int nbk = int((b - a + bucket - 1) / bucket);
        segs[size_t(k)].blo = nb;
        segs[size_t(k)].bhi = nb + nbk - 1;
        segs[size_t(k)].root = nbk == 1 ? -1 - nb : 0;  // multi-bucket roots come from the tree
        segs[size_t(k)].n = int(b - a);
        segs[size_t(k)].fx = flips[3 * size_t(k)];
        segs[size_t(k)].fy = flips[3 * size_t(k) + 1];
        segs[size_t(k)].fz = flips[3 * size_t(k) + 2];
        segs[size_t(k)].pad = 0;
        nb += nbk;
        np += nbk * bucket;
    }
    off[size_t(S)] = n;
    pad_off[size_t(S)] = np;
    int sbits = 0;
    while ((1 << sbits) < S) sbits++;
    out.nscans = S;
    out.npoints = n;
    out.npadded = np;
    out.nbuckets = nb;
    out.bucket = bucket;
    out.sbits = sbits;
    out.d_off = ws.get<int>(tag + ".off", size_t(S) + 1);
    out.d_pad = ws.get<int>(tag + ".padoff", size_t(S) + 1);
    out.segs = ws.get<SegInfo>(tag + ".segs", size_t(S));
    LVRGB_CUDA(cudaMemcpyAsync(out.d_off, off.data(), sizeof(int) * off.size(), cudaMemcpyHostToDevice, s));
    LVRGB_CUDA(cudaMemcpyAsync(out.d_pad, pad_off.data(), sizeof(int) * pad_off.size(), cudaMemcpyHostToDevice, s));
    LVRGB_CUDA(cudaMemcpyAsync(out.segs, segs.data(), sizeof(SegInfo) * segs.size(), cudaMemcpyHostToDevice, s));
    // the host vectors go out of scope: finish the uploads now
    LVRGB_CUDA(cudaStreamSynchronize(s));
    // size every buffer of the build here so that lbvh_segmented_build allocates nothing
    out.T.pts = ws.get<float4>(tag + ".pts", size_t(np));
    out.T.inv = ws.get<uint32_t>(tag + ".inv", size_t(n));
    out.T.nodes = ws.get<TreeNode>(tag + ".nodes", size_t(nb > 1 ? nb - 1 : 1));
    out.bucket_scan = ws.get<uint16_t>(tag + ".bscan", size_t(nb));
    out.box = ws.get<float>(tag + ".segbox", size_t(S) * 6);
    out.keys = ws.get<uint64_t>(tag + ".keys", size_t(n));
    out.keys2 = ws.get<uint64_t>(tag + ".keys2", size_t(n));
    out.idx = ws.get<uint32_t>(tag + ".idx", size_t(n));
    out.idx2 = ws.get<uint32_t>(tag + ".idx2", size_t(n));
    out.sort_tmp = ws.get<unsigned char>(tag + ".sorttmp", std::max(radix_sort_temp_bytes<uint64_t>(size_t(n)),
                                                                     radix_sort_temp_bytes<uint32_t>(size_t(n))));
    out.sid = ws.get<uint32_t>(tag + ".sid", size_t(n));
    out.sid2 = ws.get<uint32_t>(tag + ".sid2", size_t(n));
    out.perm = ws.get<uint32_t>(tag + ".perm", size_t(n));
    out.perm2 = ws.get<uint32_t>(tag + ".perm2", size_t(n));
    out.pkeys = ws.get<uint64_t>(tag + ".pkeys", size_t(np));
    out.bkeys = ws.get<uint64_t>(tag + ".bkeys", size_t(nb));
    out.bparent = ws.get<int>(tag + ".bparent", size_t(nb));
    out.counters = ws.get<int>(tag + ".counters", size_t(nb > 1 ? nb - 1 : 1));
    out.T.n = np;
    out.T.bucket = bucket;
    out.T.nbuckets = nb;
    out.T.bkeys = nullptr;
}

void lbvh_segmented_build(const float* xyz, SegTree& out, int* d_err, cudaStream_t s) {
    const int S = out.nscans, n = out.npoints, np = out.npadded, nb = out.nbuckets, bucket = out.bucket;
    float4* pts = const_cast<float4*>(out.T.pts);
    uint32_t* inv = const_cast<uint32_t*>(out.T.inv);
    TreeNode* nodes = const_cast<TreeNode*>(out.T.nodes);
    seg_bbox_kernel<<<S, 1024, 0, s>>>(xyz, out.d_off, out.box);
    LVRGB_LAUNCH_CHECK();
    seg_morton_kernel<<<ceil_div(n, 256), 256, 0, s>>>(xyz, n, out.d_off, S, out.box, out.keys, out.idx);
    LVRGB_LAUNCH_CHECK();
    // Morton order over all points, then a stable sort by scan id: each scan
    // contiguous and Morton-ordered within.
    const bool alt = radix_sort_pairs<uint64_t>(out.keys, out.idx, out.keys2, out.idx2, size_t(n), 0, 63,
                                                out.sort_tmp, s);
    const uint64_t* scodes = alt ? out.keys2 : out.keys;
    const uint32_t* sidx = alt ? out.idx2 : out.idx;
    seg_scan_ids_kernel<<<ceil_div(n, 256), 256, 0, s>>>(sidx, n, out.d_off, S, out.sid, out.perm);
    LVRGB_LAUNCH_CHECK();
    const uint32_t* sid = out.sid;
    const uint32_t* perm = nullptr;
    if (out.sbits > 0) {
        const bool alt2 = radix_sort_pairs<uint32_t>(out.sid, out.perm, out.sid2, out.perm2, size_t(n), 0, out.sbits,
                                                     out.sort_tmp, s);
        sid = alt2 ? out.sid2 : out.sid;
        perm = alt2 ? out.perm2 : out.perm;
    }
    seg_pad_kernel<<<ceil_div(np, 256), 256, 0, s>>>(np, out.d_off, out.d_pad, S, pts);
    LVRGB_LAUNCH_CHECK();
    seg_gather_kernel<<<ceil_div(n, 256), 256, 0, s>>>(xyz, scodes, sidx, sid, perm, n, out.d_off, out.d_pad, pts,
                                                      inv, out.pkeys);
    LVRGB_LAUNCH_CHECK();
    seg_bucket_keys_kernel<<<ceil_div(nb, 256), 256, 0, s>>>(out.pkeys, bucket, nb, out.d_pad, S, out.bkeys,
                                                            out.bucket_scan);
    LVRGB_LAUNCH_CHECK();
    if (nb == 1) {
        LVRGB_CUDA(cudaMemsetAsync(out.bparent, 0xff, sizeof(int), s));
        return;
    }
    LVRGB_CUDA(cudaMemsetAsync(out.counters, 0, sizeof(int) * size_t(nb - 1), s));
    karras_kernel<<<ceil_div(nb - 1, 256), 256, 0, s>>>(out.bkeys, out.bucket_scan, out.sbits, nb, nodes,
                                                        out.bparent, out.segs);
    LVRGB_LAUNCH_CHECK();
    bounds_kernel<<<ceil_div(size_t(nb) * 32, 256), 256, 0, s>>>(pts, np, bucket, nb, nodes, out.bparent,
                                                                 out.counters, d_err);
    LVRGB_LAUNCH_CHECK();
}

}  // namespace lvrgb
