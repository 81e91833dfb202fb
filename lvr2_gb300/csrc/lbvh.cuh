// lbvh.cuh -- linear BVH over Morton-sorted point buckets, and the
// warp-cooperative k-nearest-neighbour traversal shared by the normal,
// interpolation, signed-distance and kNN kernels.
//
// Layout in HBM
//   pts    float4[n]      points in Morton order: x, y, z, original index (bits)
//   inv    uint32[n]      original index -> Morton position
//   nodes  TreeNode[nb-1] Karras radix tree over the nb = ceil(n / B) buckets
//                         of B consecutive Morton-ordered points; each node
//                         holds both children's boxes (one 64-byte fetch per
//                         visit) and the child links.
//
// Traversal: one warp serves 32 consecutive queries.  Child boxes are tested
// per lane against that lane's current k-th distance; a child is entered when
// any lane needs it (ballot), so control flow is warp-uniform.  A bucket is
// loaded once (one coalesced float4 per lane), staged in shared memory and
// broadcast to all lanes.  The warp's traversal stack is kept in registers,
// one entry per lane (shuffle to pop).  Each lane keeps its own max-heap of
// (squared distance, original index) keys.
#pragma once
#include "common.cuh"

namespace lvrgb {

struct __align__(16) TreeNode {
    float4 a;  // child0 lo.x lo.y lo.z hi.x
    float4 b;  // child0 hi.y hi.z, child1 lo.x lo.y
    float4 c;  // child1 lo.z hi.x hi.y hi.z
    int4 d;    // child0, child1 (>= 0 internal node, < 0 bucket -1-b), parent word, unused
};

// One scan of a segmented tree: its subtree root (< 0: single bucket -1-root),
// its bucket range and its flip point.
struct SegInfo {
    int root;
    int blo, bhi;
    int n;
    float fx, fy, fz;
    int pad;
};

struct Lbvh {
    const float4* pts = nullptr;
    const uint32_t* inv = nullptr;
    const TreeNode* nodes = nullptr;
    const uint64_t* bkeys = nullptr;  // Morton code of each bucket's first point
    int n = 0;
    int nbuckets = 0;
    int bucket = 32;
    float mn[3] = {0, 0, 0};  // Morton frame: code axis = (x - mn) * scale
    float scale = 0;
    int seed_radius = 1;      // buckets scanned on each side of the seed bucket
};

// Morton codes of the point LBVH: 21 bits per axis (63-bit codes) over the
// cube of the longest bounding-box side.  Scans are far denser near the
// scanner than at range; 10 bits per axis would put hundreds of thousands of
// points of one scan into one code and their buckets would overlap.
constexpr float kMortonCells = 2097152.0f;  // 2^21
__host__ __device__ inline float morton_scale(float extent) { return extent > 0.0f ? kMortonCells / extent : 0.0f; }
__device__ __forceinline__ uint64_t morton63(float x, float y, float z, float mnx, float mny, float mnz, float scale) {
    const float top = kMortonCells - 1.0f;
    const uint32_t cx = uint32_t(fminf(fmaxf(__fmul_rn(__fsub_rn(x, mnx), scale), 0.0f), top));
    const uint32_t cy = uint32_t(fminf(fmaxf(__fmul_rn(__fsub_rn(y, mny), scale), 0.0f), top));
    const uint32_t cz = uint32_t(fminf(fmaxf(__fmul_rn(__fsub_rn(z, mnz), scale), 0.0f), top));
    return spread20(cx) | (spread20(cy) << 1) | (spread20(cz) << 2);
}

// Traversal stack: three register entries per lane.  A root-to-leaf path of a
// Karras tree over 63-bit codes with 32-bit index tie-breaks has fewer than
// 63 + 32 = 95 nodes, and the stack never holds more entries than that depth.
constexpr int kStackMax = 96;
constexpr int kErrStack = 1;   // traversal stack would overflow (never for depth <= 95)
constexpr int kErrWalk = 2;    // more node visits than a tree over nbuckets can have
constexpr int kErrRows = 4;    // a neighbour row shorter than the RANSAC schedule reads
constexpr int kErrTma = 8;     // a TMA tile copy did not complete within its wait bound
constexpr int kErrTable = 16;  // a hash table had no free slot (sized to stay at most half full)

// Traversal counters of one warp (nodes, buckets) and one lane (heap
// insertions); kernels that do not report them let the compiler drop them.
struct TravStats {
    unsigned nodes = 0, buckets = 0, chunks = 0, pushes = 0, rounds = 0, retries = 0;
};

// Per-lane max-heap of uint64 keys, lane-interleaved (entry s of lane l at
// base[s * 32 + l]) so that the 32 lanes of a warp hit distinct banks.  The
// heap is kA-ary: a sift-down is a chain of dependent shared-memory loads, one
// level per step, and the children of a level are independent loads, so a
// wider node shortens the chain (k = 40: 3 levels instead of 5 for a binary
// heap).  kComplete: every internal node has all kA children, (K - 1) % kA ==
// 0 (the launcher guarantees it), so replacements need no bounds tests; k = 40
// is such a 3-ary heap (1 + 3 + 9 + 27 entries).  kFixedK: the launcher
// guarantees K == kFixedK, and a replacement walks the levels below the root's
// children unrolled, with only the bounds tests that size needs (k = 40, 20,
// 5; see kLevelsBelow).  The first K keys are stored without sifting and
// heapified once; until then the bound is +inf.
constexpr int kHeapArity = 4;

template <int kA, bool kComplete, int kFixedK = 0>
struct LaneHeapT {
    // levels below the root's children that a replacement can walk, for the
    // fixed sizes: k = 40 as a perfect 3-ary tree (two, no leaf tests), k = 20
    // as a 4-ary tree whose last internal node (4) lacks its fourth child
    // (one, that child tested)
    static constexpr int kLevelsBelow = (kA == 3 && kFixedK == 40) ? 2 : (kA == 4 && kFixedK == 20) ? 1 : 0;
    static constexpr bool kPerfect = kA == 3 && kFixedK == 40;
    // k = 5: the root's four children are leaves
    static constexpr bool kFlat = kA == 4 && kFixedK == 5;
    unsigned long long* h;
    int K;
    int fill;
    int real;  // real (non-sentinel) entries once finished
    unsigned long long top;

    __device__ __forceinline__ void init(unsigned long long* lane_base, int k) {
        h = lane_base;
        K = k;
        fill = 0;
        real = 0;
        top = kKeyEmpty;
    }
    __device__ __forceinline__ float tau() const { return key_d2(top); }
    // Largest child of a node whose first child is c0 (< end); kChecked: some
    // children may lie at or past end.
    template <bool kChecked>
    __device__ __forceinline__ void max_child(int c0, int end, unsigned long long& best, int& bc) const {
        best = h[c0 * 32];
        bc = c0;
#pragma unroll
        for (int t = 1; t < kA; t++) {
            const int c = c0 + t;
            if (!kChecked || c < end) {
                const unsigned long long v = h[c * 32];
                if (v > best) {
                    best = v;
                    bc = c;
                }
            }
        }
    }
    template <bool kChecked>
    __device__ __forceinline__ void sift_down(int i, int end, unsigned long long key) {
        while (true) {
            const int c0 = kA * i + 1;
            if (c0 >= end) break;
            unsigned long long best;
            int bc;
            max_child<kChecked>(c0, end, best, bc);
            if (best <= key) break;
            h[i * 32] = best;
            i = bc;
        }
        h[i * 32] = key;
    }
    __device__ __forceinline__ void heapify() {
        for (int i = (K - 2) / kA; i >= 0; i--) sift_down<true>(i, K, h[i * 32]);
        top = h[0];
    }
    // Replace the maximum by key (caller guarantees key < top).
    __device__ __forceinline__ void push(unsigned long long key) {
        if (fill < K) {
            h[(fill++) * 32] = key;
            if (fill == K) heapify();
            return;
        }
        // the root's level is peeled so that the new maximum is known without
        // reading it back
        if (!kComplete && kFixedK == 0 && K == 1) {
            h[0] = key;
            top = key;
            return;
        }
        unsigned long long best;
        int bc;
        max_child<!(kComplete || kFixedK > kA)>(1, K, best, bc);
        if (best <= key) {
            h[0] = key;
            top = key;
            return;
        }
        h[0] = best;
        top = best;
        if constexpr (kLevelsBelow > 0) {
            int i = bc;
#pragma unroll
            for (int lev = 0; lev < kLevelsBelow; lev++) {
                const int c0 = kA * i + 1;
                unsigned long long b2 = h[c0 * 32];
                int c2 = c0;
#pragma unroll
                for (int t = 1; t < kA; t++) {
                    if (kPerfect || t < kA - 1 || c0 + t < kFixedK) {
                        const unsigned long long v = h[(c0 + t) * 32];
                        if (v > b2) {
                            b2 = v;
                            c2 = c0 + t;
                        }
                    }
                }
                if (b2 <= key) break;
                h[i * 32] = b2;
                i = c2;
            }
            h[i * 32] = key;
        } else if constexpr (kFlat) {
            h[bc * 32] = key;
        } else {
            sift_down<!kComplete>(bc, K, key);
        }
    }
    // Completes the heap when fewer than K keys were offered (sentinels).
    __device__ __forceinline__ void finish() {
        real = fill;
        if (fill < K) {
            for (int s = fill; s < K; s++) h[s * 32] = kKeyEmpty;
            fill = K;
            heapify();
        }
    }
    // In-place heap sort: afterwards h[0..K) is ascending.
    __device__ __forceinline__ void sort_ascending() {
        for (int end = K - 1; end > 0; end--) {
            unsigned long long mx = h[0];
            unsigned long long key = h[end * 32];
            h[end * 32] = mx;
            sift_down<true>(0, end, key);
        }
    }
    __device__ __forceinline__ unsigned long long at(int s) const { return h[s * 32]; }
};
using LaneHeap = LaneHeapT<kHeapArity, false>;
// complete 3-ary heaps (K = 1 + 3m: 37, 43, ... with five resident blocks),
// and the fixed sizes: k = 40 (kn = 20's first adaptive round), k = 20 (kd =
// 20, kn = 10's first round), k = 5 (the planar pass, kd = 5)
using LaneHeap3 = LaneHeapT<3, true>;
using LaneHeap40 = LaneHeapT<3, true, 40>;
using LaneHeap20 = LaneHeapT<4, false, 20>;
using LaneHeap5 = LaneHeapT<4, true, 5>;
__host__ __device__ constexpr bool complete_3ary(int K) { return K >= 4 && (K - 1) % 3 == 0; }

// Per-warp candidate buffer (64 float4 in shared memory, NaN padded) and the
// warp's query box.  Bucket points pass a cheap warp-level filter (one point
// per lane: distance to the box of the warp's queries against the largest
// k-th bound of the warp, a conservative test) and are compacted into the
// buffer; every 32 buffered candidates are scanned by all lanes with their
// own exact bound.
struct WarpCand {
    float4* buf;
    int count;  // warp-uniform
    float lo[3], hi[3];
};

// Scans buf[0..32) for every lane (entries past `count` are NaN and never
// accepted), pushes accepted candidates, and drops the scanned entries.
template <class Heap>
__device__ __forceinline__ void flush_chunk(WarpCand& W, float qx, float qy, float qz, bool active, Heap& heap,
                                            TravStats& st) {
    const int lane = threadIdx.x & 31;
    st.chunks++;
    unsigned mask = 0;
    if (active) {
        const float tau = heap.tau();
        const unsigned valid = W.count >= 32 ? kFull : (1u << W.count) - 1u;
        if (tau == INFINITY) {
            mask = valid;  // a heap still filling takes every entry
        } else {
            // d2 <= tau exactly when d2 - tau_up < 0, tau_up the float above
            // tau (tau >= 0 is finite): the sign bit of the difference is
            // the acceptance bit, shifted in from the top so that entry j
            // ends at bit j.
            const float tau_up = __uint_as_float(__float_as_uint(tau) + 1u);
#pragma unroll
            for (int j = 31; j >= 0; j--) {
                const float4 c = W.buf[j];
                const float d2 = dist2(qx, qy, qz, c.x, c.y, c.z);
                mask = __funnelshift_l(__float_as_uint(__fsub_rn(d2, tau_up)), mask, 1);
            }
            mask &= valid;
        }
    }
    st.rounds += __reduce_max_sync(kFull, unsigned(__popc(mask)));
    while (mask) {
        const int j = __ffs(mask) - 1;
        mask &= mask - 1;
        const float4 c = W.buf[j];
        const float d2 = dist2(qx, qy, qz, c.x, c.y, c.z);
        const unsigned long long key = make_key(d2, __float_as_uint(c.w));
        if (key < heap.top) {
            heap.push(key);
            st.pushes++;
        }
    }
    __syncwarp();
    const float nan = __int_as_float(0x7fffffff);
    const float4 tail = W.buf[32 + lane];
    __syncwarp();
    W.buf[lane] = tail;
    W.buf[32 + lane] = make_float4(nan, nan, nan, 0.0f);
    __syncwarp();
    W.count = W.count > 32 ? W.count - 32 : 0;
}

// Adds the points of bucket b that may be within some lane's bound.
template <class Heap>
__device__ __forceinline__ void add_bucket(const Lbvh& T, int b, WarpCand& W, float qx, float qy, float qz,
                                           bool active, Heap& heap, TravStats& st) {
    const int lane = threadIdx.x & 31;
    st.buckets++;
    const int first = b * T.bucket;
    int cnt = T.n - first;
    if (cnt > T.bucket) cnt = T.bucket;
    const float tmax = __uint_as_float(__reduce_max_sync(kFull, active ? __float_as_uint(heap.tau()) : 0u));
    bool keep = false;
    float4 p = make_float4(0, 0, 0, 0);
    if (lane < cnt) {
        p = __ldg(T.pts + first + lane);
        keep = box_dist2(p.x, p.y, p.z, W.lo[0], W.lo[1], W.lo[2], W.hi[0], W.hi[1], W.hi[2]) <= tmax;
    }
    const unsigned m = __ballot_sync(kFull, keep);
    if (keep) W.buf[W.count + __popc(m & ((1u << lane) - 1u))] = p;
    W.count += __popc(m);
    __syncwarp();
    if (W.count >= 32) flush_chunk(W, qx, qy, qz, active, heap, st);
}

// Bucket whose first Morton code is the largest <= the code of (x, y, z):
// a 32-ary search by the whole warp over the sorted bucket keys (warp-uniform
// inputs and result).
__device__ __forceinline__ int seed_bucket_for(const Lbvh& T, float x, float y, float z) {
    const int lane = threadIdx.x & 31;
    const uint64_t code = morton63(x, y, z, T.mn[0], T.mn[1], T.mn[2], T.scale);
    int lo = 0, hi = T.nbuckets;  // answer in [lo, hi)
    while (hi - lo > 1) {
        const int step = (hi - lo + 31) / 32;
        const int probe = lo + lane * step;
        const bool le = probe < hi && __ldg(T.bkeys + probe) <= code;
        const int c = __popc(__ballot_sync(kFull, le));
        if (c == 0) return lo;  // code below the first key of the range
        lo = lo + (c - 1) * step;
        hi = min(hi, lo + step);
    }
    return lo;
}

// k-nearest-neighbour search of one query per lane.  On return each lane's
// heap holds its K smallest (d2, original index) keys (unordered).  The
// warp-uniform seed bucket (and seed_radius buckets on each side, which are
// Morton neighbours) are scanned first so that the k-th distance bound is
// small before the tree walk; the walk skips them.
template <class Heap>
__device__ __forceinline__ void knn_traverse(const Lbvh& T, float qx, float qy, float qz, bool active_in,
                                             Heap& heap, float4* stage, int* err, TravStats& st,
                                             int seed = -1, int root = 0, int blo = 0, int bhi = 0x7fffffff) {
    const int lane = threadIdx.x & 31;
    // A query with a non-finite coordinate has no neighbours (every distance
    // is NaN); it takes no part in the walk, where its NaN box distances
    // would open every node.
    const bool active = active_in && isfinite(qx) && isfinite(qy) && isfinite(qz);
    if (T.nbuckets <= 0) {
        if (active_in) heap.finish();
        return;
    }
    // warp query box and an empty, NaN-padded candidate buffer
    WarpCand W;
    W.buf = stage;
    W.count = 0;
    {
        const float nan = __int_as_float(0x7fffffff);
        stage[lane] = make_float4(nan, nan, nan, 0.0f);
        stage[32 + lane] = make_float4(nan, nan, nan, 0.0f);
        const float big = FLT_MAX;
        float v[6] = {active ? qx : big, active ? qy : big, active ? qz : big,
                      active ? qx : -big, active ? qy : -big, active ? qz : -big};
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
            for (int a = 0; a < 3; a++) {
                v[a] = fminf(v[a], __shfl_xor_sync(kFull, v[a], o));
                v[3 + a] = fmaxf(v[3 + a], __shfl_xor_sync(kFull, v[3 + a], o));
            }
        }
        for (int a = 0; a < 3; a++) { W.lo[a] = v[a]; W.hi[a] = v[3 + a]; }
        __syncwarp();
    }
    // A root < 0 is a single bucket (-1 - root): a one-bucket tree or segment.
    if (T.nbuckets == 1) root = -1;
    bhi = min(bhi, T.nbuckets - 1);
    int skip_lo = 1, skip_hi = 0;  // empty range
    if (seed >= 0) {
        skip_lo = max(blo, seed - T.seed_radius);
        skip_hi = min(bhi, seed + T.seed_radius);
        for (int b = skip_lo; b <= skip_hi; b++) add_bucket(T, b, W, qx, qy, qz, active, heap, st);
    }
    if (root < 0) {
        const int b = -1 - root;
        if (b < skip_lo || b > skip_hi) add_bucket(T, b, W, qx, qy, qz, active, heap, st);
        if (W.count) flush_chunk(W, qx, qy, qz, active, heap, st);
        if (active_in) heap.finish();
        return;
    }
    int stk0 = 0, stk1 = 0, stk2 = 0;  // lane l holds stack entries l, l + 32, l + 64
    int sp = 0;
    int node = root;
    // A tree over nb buckets has nb - 1 internal nodes; each is expanded at
    // most once per warp.  The bound only guards against a malformed tree.
    int budget = T.nbuckets + 1;
    bool done = false;
    while (!done) {
        if (--budget < 0) {
            if (lane == 0) atomicOr(err, kErrWalk);
            break;
        }
        st.nodes++;
        // ---- expand an internal node -----------------------------------
        const TreeNode* nd = T.nodes + node;
        const float4 a = __ldg(&nd->a);
        const float4 b = __ldg(&nd->b);
        const float4 c = __ldg(&nd->c);
        const int4 d = __ldg(&nd->d);
        const float tau = heap.tau();
        const float d0 = box_dist2(qx, qy, qz, a.x, a.y, a.z, a.w, b.x, b.y);
        const float d1 = box_dist2(qx, qy, qz, b.z, b.w, c.x, c.y, c.z, c.w);
        const bool n0 = active && d0 <= tau;
        const bool n1 = active && d1 <= tau;
        const unsigned m0 = __ballot_sync(kFull, n0);
        const unsigned m1 = __ballot_sync(kFull, n1);
        int next = 0;
        unsigned need = 0;
        if (m0 && m1) {
            const unsigned p1 = __ballot_sync(kFull, n1 && (!n0 || d1 < d0));
            const bool first1 = 2 * __popc(p1) > __popc(m0 | m1);
            next = first1 ? d.y : d.x;
            need = first1 ? m1 : m0;
            const int ref = (node << 1) | (first1 ? 0 : 1);
            if (sp >= kStackMax) {
                if (lane == 0) atomicOr(err, kErrStack);
                break;
            }
            if (lane == (sp & 31)) {
                if (sp < 32) stk0 = ref; else if (sp < 64) stk1 = ref; else stk2 = ref;
            }
            sp++;
        } else if (m0) {
            next = d.x;
            need = m0;
        } else if (m1) {
            next = d.y;
            need = m1;
        }
        // ---- resolve: scan buckets, pop until an internal node to expand --
        while (true) {
            if (need) {
                if (next >= 0) {
                    node = next;
                    break;
                }
                const int bk = -1 - next;
                if (bk < skip_lo || bk > skip_hi) add_bucket(T, bk, W, qx, qy, qz, active, heap, st);
                need = 0;
            }
            if (sp == 0) {
                done = true;
                break;
            }
            sp--;
            const int ref = __shfl_sync(kFull, sp < 32 ? stk0 : (sp < 64 ? stk1 : stk2), sp & 31);
            const TreeNode* pn = T.nodes + (ref >> 1);
            const int side = ref & 1;
            float lx, ly, lz, hx, hy, hz;
            int child;
            if (side == 0) {
                const float4 pa = __ldg(&pn->a);
                const float4 pb = __ldg(&pn->b);
                lx = pa.x; ly = pa.y; lz = pa.z; hx = pa.w; hy = pb.x; hz = pb.y;
                child = __ldg(&pn->d.x);
            } else {
                const float4 pb = __ldg(&pn->b);
                const float4 pc = __ldg(&pn->c);
                lx = pb.z; ly = pb.w; lz = pc.x; hx = pc.y; hy = pc.z; hz = pc.w;
                child = __ldg(&pn->d.y);
            }
            const float dd = box_dist2(qx, qy, qz, lx, ly, lz, hx, hy, hz);
            need = __ballot_sync(kFull, active && dd <= heap.tau());
            next = child;
        }
    }
    if (W.count) flush_chunk(W, qx, qy, qz, active, heap, st);
    if (active_in) heap.finish();
}

template <class Heap>
__device__ __forceinline__ void knn_traverse(const Lbvh& T, float qx, float qy, float qz, bool active,
                                             Heap& heap, float4* stage, int* err, int seed = -1) {
    TravStats st;
    knn_traverse(T, qx, qy, qz, active, heap, stage, err, st, seed);
}

// Tile order of the per-lane kNN kernels.  With a counter (zeroed before the
// launch) a warp takes the next 32-query tile in ascending order whenever it
// becomes free, so no warp idles until the other warps of its block finish
// and the tiles in flight stay neighbours in Morton order; without one, warp
// w of the grid takes tiles w, w + W, w + 2W, ... (W warps in the grid).
__device__ __forceinline__ int take_tile(int* counter) {
    int t = 0;
    if ((threadIdx.x & 31) == 0) t = atomicAdd(counter, 1);
    return __shfl_sync(kFull, t, 0);
}
template <int kWarps>
__device__ __forceinline__ int first_tile(int* counter) {
    return counter ? take_tile(counter) : int(blockIdx.x) * kWarps + int(threadIdx.x >> 5);
}
template <int kWarps>
__device__ __forceinline__ int next_tile(int* counter, int tile) {
    return counter ? take_tile(counter) : tile + int(gridDim.x) * kWarps;
}

// Shared-memory carving of a kNN kernel block: kWarps candidate buffers of 64
// float4, then (when gheap == nullptr) kWarps lane-interleaved heaps of K keys.
// With a global heap buffer, each resident warp owns K*32 keys of it.
struct WarpCtx {
    float4* stage;
    unsigned long long* heap;  // this lane's heap base (stride 32)
};
template <int kWarps>
__device__ __forceinline__ WarpCtx warp_ctx(unsigned char* smem, unsigned long long* gheap, int K) {
    const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
    WarpCtx c;
    c.stage = reinterpret_cast<float4*>(smem) + wib * 64;
    if (gheap)
        c.heap = gheap + (size_t(blockIdx.x) * kWarps + wib) * size_t(K) * 32 + lane;
    else
        c.heap = reinterpret_cast<unsigned long long*>(smem + kWarps * 64 * sizeof(float4)) +
                 size_t(wib) * K * 32 + lane;
    return c;
}

__device__ __forceinline__ float4 neighbour_point(const Lbvh& T, unsigned long long key) {
    return __ldg(T.pts + __ldg(T.inv + key_idx(key)));
}

}  // namespace lvrgb
