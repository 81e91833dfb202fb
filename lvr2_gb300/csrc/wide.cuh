// wide.cuh -- k-nearest-neighbour search for large k (k > the per-lane heap
// limit): one warp serves one query.
//
// lvr2's adaptive normal estimation doubles k up to 32 * kn
// (AdaptiveKSearchSurface.tcc:218-268), and points on axis-aligned planes
// (floors, walls) fail the neighbourhood-box test in every round before the
// last, so a real scan sends a few percent of its points through k = 160 and
// k = 320 searches.  Per-lane heaps of that size do not fit in shared memory;
// here the whole warp works on one query instead:
//
//   * a bucket is one coalesced float4 load, one candidate per lane; the
//     candidates whose key is below the current bound are appended to a
//     per-warp key buffer (ballot + popc),
//   * when the buffer fills, a warp radix select finds the k-th smallest key,
//     the buffer is compacted to the k keys at or below it and that key
//     becomes the bound (exact: keys are unique (d2, index) pairs),
//   * the search starts with the Morton window of buckets around the query's
//     own bucket (enough points for a finite bound), then walks the tree
//     nearest child first, skipping nodes whose box is beyond the bound.
//
// The result is the same canonical set as the per-lane search: the k smallest
// keys (float d2 without FMA, original index).
#pragma once
#include "lbvh.cuh"

namespace lvrgb {

// Per-warp state of a wide search.  keys: cap entries (shared or global
// memory); hist: 256 counters in shared memory (16-byte aligned) for the
// radix select.
struct WideState {
    unsigned long long* keys;
    uint32_t* hist;
    int cap;
    int K;
    int cnt;                   // keys in the buffer, all below thr
    unsigned long long thr;    // candidates must be below this key
    float tau;                 // d2 part of thr (box pruning bound)
};

// Buffer capacity for a wide search of K: room for K kept keys, (slack - 1) K
// more before each compaction, and one bucket of slack (slack >= 2; a larger
// buffer compacts less often but takes more memory per warp).
__host__ __device__ inline int wide_capacity(int K, int slack = 2) { return ((slack * K + 64) + 31) / 32 * 32; }

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
    return __shfl_sync(kFull, v, 0);
}
__device__ __forceinline__ float warp_min_f(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(kFull, v, o));
    return v;
}
__device__ __forceinline__ float warp_max_f(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(kFull, v, o));
    return v;
}

// The r-th smallest (1-based, 1 <= r <= cnt) of cnt distinct keys, by a warp
// most-significant-digit radix select with 8-bit digits.  Stops as soon as the
// digit prefix identifies a single key.  Not inlined: the search calls it from
// several places, and one copy keeps the kernel within the instruction cache.
__device__ __noinline__ unsigned long long warp_select(const unsigned long long* keys, int cnt, int r,
                                                          uint32_t* hist) {
    const int lane = threadIdx.x & 31;
    unsigned long long prefix = 0, mask = 0;
    __syncwarp();
    for (int shift = 56; shift >= 0; shift -= 8) {
        for (int i = lane; i < 256; i += 32) hist[i] = 0;
        __syncwarp();
        for (int base = 0; base < cnt; base += 32) {
            const int i = base + lane;
            bool in = false;
            unsigned bin = 0;
            if (i < cnt) {
                const unsigned long long k = keys[i];
                in = (k & mask) == prefix;
                bin = unsigned(k >> shift) & 255u;
            }
            const unsigned act = __ballot_sync(kFull, in);
            if (in) {
                const unsigned peers = __match_any_sync(act, bin);
                if (lane == __ffs(peers) - 1) atomicAdd(hist + bin, unsigned(__popc(peers)));
            }
        }
        __syncwarp();
        // bins [8 lane, 8 lane + 8) per lane; find the bin that holds rank r
        const uint4 h0 = reinterpret_cast<const uint4*>(hist)[2 * lane];
        const uint4 h1 = reinterpret_cast<const uint4*>(hist)[2 * lane + 1];
        const unsigned c[8] = {h0.x, h0.y, h0.z, h0.w, h1.x, h1.y, h1.z, h1.w};
        unsigned local = 0;
#pragma unroll
        for (int j = 0; j < 8; j++) local += c[j];
        unsigned incl = local;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned v = __shfl_up_sync(kFull, incl, o);
            if (lane >= o) incl += v;
        }
        const unsigned excl = incl - local;
        const bool mine = excl < unsigned(r) && unsigned(r) <= incl;
        int bin = 0;
        unsigned before = excl, binc = 0;
        if (mine) {
            bool found = false;
#pragma unroll
            for (int j = 0; j < 8; j++) {
                if (!found) {
                    if (before + c[j] >= unsigned(r)) {
                        bin = lane * 8 + j;
                        binc = c[j];
                        found = true;
                    } else {
                        before += c[j];
                    }
                }
            }
        }
        const int owner = __ffs(__ballot_sync(kFull, mine)) - 1;
        bin = __shfl_sync(kFull, bin, owner);
        before = __shfl_sync(kFull, before, owner);
        binc = __shfl_sync(kFull, binc, owner);
        r -= int(before);
        prefix |= (unsigned long long)(unsigned(bin)) << shift;
        mask |= 0xffull << shift;
        if (binc == 1) {
            for (int base = 0; base < cnt; base += 32) {
                const int i = base + lane;
                const unsigned long long k = i < cnt ? keys[i] : 0ull;
                const unsigned hit = __ballot_sync(kFull, i < cnt && (k & mask) == prefix);
                if (hit) return __shfl_sync(kFull, k, __ffs(hit) - 1);
            }
            return prefix;  // not reached for distinct keys
        }
        __syncwarp();
    }
    return prefix;
}

// Keeps the keys <= kth (order preserved), in place; returns their number.
__device__ __noinline__ int warp_compact_le(unsigned long long* keys, int cnt, unsigned long long kth) {
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    int out = 0;
    __syncwarp();
    for (int base = 0; base < cnt; base += 32) {
        const int i = base + lane;
        const unsigned long long k = i < cnt ? keys[i] : 0ull;
        const bool keep = i < cnt && k <= kth;
        const unsigned m = __ballot_sync(kFull, keep);
        __syncwarp();
        if (keep) keys[out + __popc(m & lt)] = k;
        out += __popc(m);
        __syncwarp();
    }
    return out;
}

// Cuts the buffer to its K smallest keys and tightens the bound.
__device__ __forceinline__ void wide_shrink(WideState& W, TravStats& st) {
    if (W.cnt <= W.K) return;
    st.chunks++;
    const unsigned long long kth = warp_select(W.keys, W.cnt, W.K, W.hist);
    W.cnt = warp_compact_le(W.keys, W.cnt, kth);
    W.thr = kth;
    W.tau = key_d2(kth);
}

__device__ __forceinline__ void wide_add_bucket(const Lbvh& T, int b, WideState& W, float qx, float qy, float qz,
                                                TravStats& st) {
    const int lane = threadIdx.x & 31;
    st.buckets++;
    const int first = b * T.bucket;
    const int nb = min(T.n - first, T.bucket);
    bool acc = false;
    unsigned long long key = 0;
    if (lane < nb) {
        const float4 p = __ldg(T.pts + first + lane);
        const float d2 = dist2(qx, qy, qz, p.x, p.y, p.z);
        key = make_key(d2, __float_as_uint(p.w));
        acc = d2 <= W.tau && key < W.thr;  // NaN padding fails the first test
    }
    const unsigned m = __ballot_sync(kFull, acc);
    if (acc) W.keys[W.cnt + __popc(m & ((1u << lane) - 1u))] = key;
    W.cnt += __popc(m);
    st.pushes += __popc(m);
    if (W.cnt > W.cap - 32) wide_shrink(W, st);
}

// The K nearest keys of one query (warp-uniform arguments).  On return
// W.keys[0, W.cnt) holds them (unordered).  seed: the query's bucket.
// bound: squared radius that limits the search (+inf: none); W.cnt < K when
// fewer than K points lie within it, or when the tree (or the segment
// [blo, bhi]) has fewer points.
__device__ __forceinline__ void wide_knn(const Lbvh& T, float qx, float qy, float qz, WideState& W, int* err,
                                         TravStats& st, int seed, int root, int blo, int bhi, float bound) {
    const int lane = threadIdx.x & 31;
    W.cnt = 0;
    W.tau = bound;
    W.thr = bound < __int_as_float(0x7f800000) ? make_key(bound, 0xffffffffu) : kKeyEmpty;
    // a query with a non-finite coordinate has no neighbours (warp-uniform)
    if (T.nbuckets <= 0 || !(isfinite(qx) && isfinite(qy) && isfinite(qz))) return;
    if (T.nbuckets == 1) root = -1;
    bhi = min(bhi, T.nbuckets - 1);
    // Morton window around the query's bucket holding at least K points
    const int half = ((W.K + T.bucket - 1) / T.bucket + 1) / 2;
    const int skip_lo = max(blo, seed - half), skip_hi = min(bhi, seed + half);
    for (int b = skip_lo; b <= skip_hi; b++) wide_add_bucket(T, b, W, qx, qy, qz, st);
    wide_shrink(W, st);
    if (root < 0) {
        const int b = -1 - root;
        if (b < skip_lo || b > skip_hi) wide_add_bucket(T, b, W, qx, qy, qz, st);
        wide_shrink(W, st);
        return;
    }
    int stk0 = 0, stk1 = 0, stk2 = 0;  // lane l holds stack entries l, l + 32, l + 64
    int sp = 0;
    int node = root;
    int budget = T.nbuckets + 1;
    bool done = false;
    while (!done) {
        if (--budget < 0) {
            if (lane == 0) atomicOr(err, kErrWalk);
            break;
        }
        st.nodes++;
        const TreeNode* nd = T.nodes + node;
        const float4 a = __ldg(&nd->a);
        const float4 b = __ldg(&nd->b);
        const float4 c = __ldg(&nd->c);
        const int4 d = __ldg(&nd->d);
        const float d0 = box_dist2(qx, qy, qz, a.x, a.y, a.z, a.w, b.x, b.y);
        const float d1 = box_dist2(qx, qy, qz, b.z, b.w, c.x, c.y, c.z, c.w);
        const bool n0 = d0 <= W.tau, n1 = d1 <= W.tau;
        int next = 0;
        bool need = false;
        if (n0 && n1) {
            const bool first1 = d1 < d0;
            next = first1 ? d.y : d.x;
            need = true;
            if (sp >= kStackMax) {
                if (lane == 0) atomicOr(err, kErrStack);
                break;
            }
            const int ref = (node << 1) | (first1 ? 0 : 1);
            if (lane == (sp & 31)) {
                if (sp < 32) stk0 = ref; else if (sp < 64) stk1 = ref; else stk2 = ref;
            }
            sp++;
        } else if (n0) {
            next = d.x;
            need = true;
        } else if (n1) {
            next = d.y;
            need = true;
        }
        while (true) {
            if (need) {
                if (next >= 0) {
                    node = next;
                    break;
                }
                const int bk = -1 - next;
                if (bk < skip_lo || bk > skip_hi) wide_add_bucket(T, bk, W, qx, qy, qz, st);
                need = false;
            }
            if (sp == 0) {
                done = true;
                break;
            }
            sp--;
            const int ref = __shfl_sync(kFull, sp < 32 ? stk0 : (sp < 64 ? stk1 : stk2), sp & 31);
            const TreeNode* pn = T.nodes + (ref >> 1);
            float lx, ly, lz, hx, hy, hz;
            int child;
            if ((ref & 1) == 0) {
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
            need = box_dist2(qx, qy, qz, lx, ly, lz, hx, hy, hz) <= W.tau;
            next = child;
        }
    }
    wide_shrink(W, st);
}

// Sorts keys[0, cnt) ascending in place by a warp bitonic network over the
// next power of two, padding with ~0 (the buffer holds at least that many:
// cnt <= K and the capacity exceeds 2K).
__device__ __noinline__ void warp_bitonic_sort(unsigned long long* keys, int cnt) {
    const int lane = threadIdx.x & 31;
    int P = 1;
    while (P < cnt) P <<= 1;
    for (int i = cnt + lane; i < P; i += 32) keys[i] = ~0ull;
    __syncwarp();
    for (int k = 2; k <= P; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = lane; i < P; i += 32) {
                const int ixj = i ^ j;
                if (ixj > i) {
                    const unsigned long long a = keys[i], b = keys[ixj];
                    const bool up = (i & k) == 0;
                    if ((a > b) == up) {
                        keys[i] = b;
                        keys[ixj] = a;
                    }
                }
            }
            __syncwarp();
        }
    }
}

// Hands the m smallest of the W.cnt buffered keys to emit(rank, key), rank
// 0 = nearest; 1 <= m <= W.cnt.  The selected keys are staged in the histogram
// area (m <= 128) and ranked among themselves; for larger m the buffer is
// sorted.
template <typename F>
__device__ __forceinline__ void wide_sorted_prefix(WideState& W, int m, F&& emit) {
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    if (m <= 0) return;
    if (m <= 128) {
        const unsigned long long mth = m == W.cnt ? ~0ull : warp_select(W.keys, W.cnt, m, W.hist);
        __syncwarp();
        unsigned long long* stage = reinterpret_cast<unsigned long long*>(W.hist);
        int c = 0;
        for (int base = 0; base < W.cnt; base += 32) {
            const int i = base + lane;
            const unsigned long long k = i < W.cnt ? W.keys[i] : 0ull;
            const bool sel = i < W.cnt && k <= mth;
            const unsigned bm = __ballot_sync(kFull, sel);
            if (sel) stage[c + __popc(bm & lt)] = k;
            c += __popc(bm);
        }
        __syncwarp();
        for (int i = lane; i < m; i += 32) {
            const unsigned long long k = stage[i];
            int rank = 0;
            for (int j = 0; j < m; j++) rank += stage[j] < k ? 1 : 0;
            emit(rank, k);
        }
    } else {
        // sort the whole buffer (the k-th selection above is not needed)
        warp_bitonic_sort(W.keys, W.cnt);
        for (int i = lane; i < m; i += 32) emit(i, W.keys[i]);
    }
    __syncwarp();
}

}  // namespace lvrgb
