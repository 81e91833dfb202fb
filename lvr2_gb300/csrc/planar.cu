// planar.cu -- BilinearFastBox::optimizePlanarFaces (BilinearFastBox.tcc:140-212),
// the post-pass FastReconstruction::getMesh runs on every cell with kc = 5 for
// PMC (FastReconstruction.tcc:158-168), on the whole mesh at once:
//   1. every face edge as an undirected key (min vertex, max vertex) goes
//      into an open-addressing table (linear probing, at most half full);
//      the second insertion of a key marks its slot.  An edge whose slot is
//      unmarked occurs once: it belongs to one face, a border edge,
//   2. one thread per valid cell counts the border edges of its faces and,
//      for 1 or 2, marks both end vertices of each,
//   3. the marked vertices, compacted and Morton-sorted, take the centroid of
//      their kc nearest points (sums in ascending (d2, index) order, then a
//      division by the count, as BaseVector::operator/=).
// lvr2 moves vertices in place while iterating its cell hash map, so a vertex
// on several such edges can move more than once, in a map-dependent order;
// here every marked vertex moves once, from its marching-cubes position.
#include <algorithm>

#include "planar.h"
#include "primitives.cuh"
#include "surface.h"

namespace lvrgb {

namespace {

constexpr unsigned long long kSlotEmpty = ~0ull;
constexpr unsigned long long kSlotTwice = 1ull << 63;  // set by a key's second insertion

// Undirected key of edge e (0..2) of face f: (min vertex) << 32 | max vertex;
// vertex ids are below 2^31, so bit 63 is free for kSlotTwice.
__device__ __forceinline__ unsigned long long edge_key(const uint32_t* __restrict__ faces, int f, int e) {
    const unsigned long long a = faces[3 * size_t(f) + e], b = faces[3 * size_t(f) + (e == 2 ? 0 : e + 1)];
    return a < b ? (a << 32) | b : (b << 32) | a;
}
// 64-bit finaliser of splitmix64 (Steele, Lea, Flood 2014)
__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

__global__ void edge_insert_kernel(const uint32_t* __restrict__ faces, int nf, unsigned long long* __restrict__ table,
                                   unsigned long long slot_mask, int* __restrict__ err) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 3 * nf) return;
    const int f = i / 3;
    const unsigned long long key = edge_key(faces, f, i - 3 * f);
    unsigned long long h = mix64(key) & slot_mask;
    for (unsigned long long probe = 0; probe <= slot_mask; probe++) {
        const unsigned long long old = atomicCAS(table + h, kSlotEmpty, key);
        if (old == kSlotEmpty) return;
        if ((old & ~kSlotTwice) == key) {
            if (!(old & kSlotTwice)) atomicOr(table + h, kSlotTwice);
            return;
        }
        h = (h + 1) & slot_mask;
    }
    atomicOr(err, kErrTable);  // a full table: cannot happen at load <= 1/2
}

__global__ void border_kernel(const uint32_t* __restrict__ faces, int nf, const unsigned long long* __restrict__ table,
                              unsigned long long slot_mask, uint8_t* __restrict__ border) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 3 * nf) return;
    const int f = i / 3;
    const unsigned long long key = edge_key(faces, f, i - 3 * f);
    unsigned long long h = mix64(key) & slot_mask;
    uint8_t b = 1;
    for (unsigned long long probe = 0; probe <= slot_mask; probe++) {
        const unsigned long long v = table[h];
        if ((v & ~kSlotTwice) == key) {
            b = (v & kSlotTwice) ? 0 : 1;
            break;
        }
        if (v == kSlotEmpty) break;
        h = (h + 1) & slot_mask;
    }
    border[i] = b;
}

__global__ void mark_kernel(const uint32_t* __restrict__ faces, const uint8_t* __restrict__ border,
                            const uint32_t* __restrict__ off, int ncells, uint32_t* __restrict__ vmark) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncells) return;
    const uint32_t f0 = off[c], f1 = off[c + 1];
    int cnt = 0;
    for (uint32_t r = 3 * f0; r < 3 * f1; r++) cnt += border[r];
    if (cnt != 1 && cnt != 2) return;
    for (uint32_t f = f0; f < f1; f++)
        for (int e = 0; e < 3; e++)
            if (border[3 * size_t(f) + e]) {
                vmark[faces[3 * size_t(f) + e]] = 1u;
                vmark[faces[3 * size_t(f) + (e == 2 ? 0 : e + 1)]] = 1u;
            }
}

__global__ void gather_marked_kernel(const float* __restrict__ verts, const uint32_t* __restrict__ list, int m,
                                     float* __restrict__ q) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= m) return;
    const size_t v = list[r];
    q[3 * size_t(r)] = verts[3 * v];
    q[3 * size_t(r) + 1] = verts[3 * v + 1];
    q[3 * size_t(r) + 2] = verts[3 * v + 2];
}

__global__ void centroid_kernel(const uint32_t* __restrict__ list, const uint32_t* __restrict__ idx,
                                const int32_t* __restrict__ count, int m, int kc, Lbvh T, float* __restrict__ verts) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= m) return;
    const int c = count[r];
    if (c <= 0) return;  // lvr2 keeps the vertex when the search finds nothing
    float x = 0.0f, y = 0.0f, z = 0.0f;
    for (int s = 0; s < c; s++) {
        const float4 p = __ldg(T.pts + __ldg(T.inv + idx[size_t(r) * kc + s]));
        x = __fadd_rn(x, p.x);
        y = __fadd_rn(y, p.y);
        z = __fadd_rn(z, p.z);
    }
    const float n = float(c);
    const size_t v = list[r];
    verts[3 * v] = __fdiv_rn(x, n);
    verts[3 * v + 1] = __fdiv_rn(y, n);
    verts[3 * v + 2] = __fdiv_rn(z, n);
}

uint32_t read_u32(Workspace& ws, const uint32_t* d, cudaStream_t s) {
    uint64_t* h = ws.pinned();
    h[0] = 0;
    LVRGB_CUDA(cudaMemcpyAsync(h, d, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    LVRGB_CUDA(cudaStreamSynchronize(s));
    return uint32_t(h[0]);
}

}  // namespace

long long optimize_planar_faces(const Lbvh& T, const float* d_box, GridResult& R, int kc, Workspace& ws,
                                int* d_err, cudaStream_t s) {
    const int nf = int(R.nfaces), nv = int(R.nverts), ncells = int(R.ncells_valid);
    if (nf == 0 || nv == 0 || T.n == 0) return 0;
    const int m3 = 3 * nf;
    // 1. border edges
    size_t slots = 1024;
    while (slots < 2 * size_t(m3)) slots *= 2;
    unsigned long long* table = ws.get<unsigned long long>("planar.edges", slots);
    LVRGB_CUDA(cudaMemsetAsync(table, 0xff, slots * sizeof(unsigned long long), s));
    edge_insert_kernel<<<ceil_div(m3, 256), 256, 0, s>>>(R.faces, nf, table, slots - 1, d_err);
    LVRGB_LAUNCH_CHECK();
    uint8_t* border = ws.get<uint8_t>("planar.border", size_t(m3));
    border_kernel<<<ceil_div(m3, 256), 256, 0, s>>>(R.faces, nf, table, slots - 1, border);
    LVRGB_LAUNCH_CHECK();
    // 2. marked vertices
    uint32_t* vmark = ws.get<uint32_t>("planar.vmark", size_t(nv));
    LVRGB_CUDA(cudaMemsetAsync(vmark, 0, sizeof(uint32_t) * size_t(nv), s));
    if (ncells > 0) {
        mark_kernel<<<ceil_div(ncells, 128), 128, 0, s>>>(R.faces, border, R.face_cell_off, ncells, vmark);
        LVRGB_LAUNCH_CHECK();
    }
    uint32_t* ids = ws.get<uint32_t>("planar.ids", size_t(nv));
    uint32_t* pos = ws.get<uint32_t>("planar.pos", size_t(nv) + 1);
    uint32_t* list = ws.get<uint32_t>("planar.list", size_t(nv));
    iota_u32(ids, size_t(nv), s);
    void* stmp = ws.get<unsigned char>("planar.scantmp", scan_temp_bytes(size_t(nv)));
    exclusive_scan_u32(vmark, pos, size_t(nv), stmp, pos + nv, s);
    scatter_flagged_u32(ids, vmark, pos, size_t(nv), list, s);
    const int m = int(read_u32(ws, pos + nv, s));
    if (m == 0) return 0;
    // 3. centroids of the kc nearest points of the marching-cubes positions
    float* q = ws.get<float>("planar.q", size_t(m) * 3);
    gather_marked_kernel<<<ceil_div(m, 256), 256, 0, s>>>(R.verts, list, m, q);
    LVRGB_LAUNCH_CHECK();
    float4* qs = ws.get<float4>("planar.qs", size_t(m));
    sort_queries(q, m, d_box, qs, ws, s);
    uint32_t* idx = ws.get<uint32_t>("planar.idx", size_t(m) * kc);
    float* dist = ws.get<float>("planar.dist", size_t(m) * kc);
    int32_t* cnt = ws.get<int32_t>("planar.cnt", size_t(m));
    knn_rows(T, qs, m, kc, idx, dist, cnt, ws, d_err, s);
    centroid_kernel<<<ceil_div(m, 256), 256, 0, s>>>(list, idx, cnt, m, kc, T, R.verts);
    LVRGB_LAUNCH_CHECK();
    return m;
}

}  // namespace lvrgb
