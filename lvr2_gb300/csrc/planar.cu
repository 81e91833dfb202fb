// planar.cu -- BilinearFastBox::optimizePlanarFaces (BilinearFastBox.tcc:140-212),
// the post-pass FastReconstruction::getMesh runs on every cell with kc = 5 for
// PMC (FastReconstruction.tcc:158-168), on the whole mesh at once:
//   1. every face edge as an undirected key (min vertex, max vertex), packed
//      into 2 x (bits of the vertex count) bits and sorted; an edge whose key
//      occurs once belongs to one face: a border edge,
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

__global__ void edge_keys_kernel(const uint32_t* __restrict__ faces, int nf, int vbits, uint64_t* __restrict__ keys,
                                 uint32_t* __restrict__ vals) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 3 * nf) return;
    const int f = i / 3, e = i - 3 * f;
    const uint64_t a = faces[3 * size_t(f) + e], b = faces[3 * size_t(f) + (e == 2 ? 0 : e + 1)];
    keys[i] = a < b ? (a << vbits) | b : (b << vbits) | a;
    vals[i] = uint32_t(i);
}

__global__ void border_kernel(const uint64_t* __restrict__ keys, const uint32_t* __restrict__ vals, int m,
                              uint8_t* __restrict__ border) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    const uint64_t k = keys[i];
    const bool single = (i == 0 || keys[i - 1] != k) && (i == m - 1 || keys[i + 1] != k);
    border[vals[i]] = single ? 1 : 0;
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
    uint64_t* keys = ws.get<uint64_t>("planar.keys", size_t(m3));
    uint64_t* keys2 = ws.get<uint64_t>("planar.keys2", size_t(m3));
    uint32_t* vals = ws.get<uint32_t>("planar.vals", size_t(m3));
    uint32_t* vals2 = ws.get<uint32_t>("planar.vals2", size_t(m3));
    int vbits = 1;
    while (vbits < 32 && (uint64_t(1) << vbits) < uint64_t(nv)) vbits++;
    edge_keys_kernel<<<ceil_div(m3, 256), 256, 0, s>>>(R.faces, nf, vbits, keys, vals);
    LVRGB_LAUNCH_CHECK();
    void* tmp = ws.get<unsigned char>("planar.sorttmp", radix_sort_temp_bytes<uint64_t>(size_t(m3)));
    if (radix_sort_pairs<uint64_t>(keys, vals, keys2, vals2, size_t(m3), 0, 2 * vbits, tmp, s)) {
        std::swap(keys, keys2);
        std::swap(vals, vals2);
    }
    uint8_t* border = ws.get<uint8_t>("planar.border", size_t(m3));
    border_kernel<<<ceil_div(m3, 256), 256, 0, s>>>(keys, vals, m3, border);
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
