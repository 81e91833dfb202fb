// meshops.cu -- calcVertexNormals (NormalAlgorithms.tcc:102-152) as called by
// lvr2_reconstruct after the mesh is built (src/tools/lvr2_reconstruct/Main.cpp:855-871):
//   face normal   = normalize((v1 - v2) x (v1 - v3)), or (0, 0, 1) for a
//                   degenerate face (getFaceNormal / calcFaceNormals, :46-72);
//   vertex normal = normalize(sum of the normals of its faces)
//                   (interpolatedVertexNormal, :74-100); a vertex whose sum
//                   is zero takes the normal of its nearest point of the cloud.
// lvr2 sums a vertex's faces in half-edge circulation order; here in
// ascending face order (a stable sort of the face references by vertex), a
// canonical order that gives the same bits on every run.
#include <algorithm>
#include <cstring>
#include <stdexcept>

#include "meshops.h"
#include "primitives.cuh"
#include "surface.h"

namespace lvrgb {

namespace {

__device__ __forceinline__ void normalize3(float& x, float& y, float& z) {
    if (!(x == 0.0f && y == 0.0f && z == 0.0f)) {
        const float len = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y)), __fmul_rn(z, z)));
        x = __fdiv_rn(x, len);
        y = __fdiv_rn(y, len);
        z = __fdiv_rn(z, len);
    }
}

__global__ void face_normals_kernel(const float* __restrict__ verts, const uint32_t* __restrict__ faces, int nf,
                                    float4* __restrict__ fn) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nf) return;
    float v[3][3];
#pragma unroll
    for (int b = 0; b < 3; b++) {
        const size_t i = size_t(faces[3 * size_t(f) + b]) * 3;
        v[b][0] = verts[i]; v[b][1] = verts[i + 1]; v[b][2] = verts[i + 2];
    }
    const float ax = __fsub_rn(v[0][0], v[1][0]), ay = __fsub_rn(v[0][1], v[1][1]), az = __fsub_rn(v[0][2], v[1][2]);
    const float bx = __fsub_rn(v[0][0], v[2][0]), by = __fsub_rn(v[0][1], v[2][1]), bz = __fsub_rn(v[0][2], v[2][2]);
    float x = __fsub_rn(__fmul_rn(ay, bz), __fmul_rn(az, by));
    float y = __fsub_rn(__fmul_rn(az, bx), __fmul_rn(ax, bz));
    float z = __fsub_rn(__fmul_rn(ax, by), __fmul_rn(ay, bx));
    const float len2 = __fadd_rn(__fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y)), __fmul_rn(z, z));
    if (len2 == 0.0f) {
        x = 0.0f; y = 0.0f; z = 1.0f;
    } else {
        normalize3(x, y, z);
    }
    fn[f] = make_float4(x, y, z, 0.0f);
}

// One thread per run of equal vertex ids in the sorted (vertex, reference)
// pairs: the vertex's faces in ascending order.
__global__ void vertex_sum_kernel(const uint32_t* __restrict__ vk, const uint32_t* __restrict__ refs, int m,
                                  const float4* __restrict__ fn, float* __restrict__ out, uint32_t* __restrict__ zero) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    const uint32_t v = vk[i];
    if (i > 0 && vk[i - 1] == v) return;
    float x = 0.0f, y = 0.0f, z = 0.0f;
    for (int j = i; j < m && vk[j] == v; j++) {
        const float4 n = fn[refs[j] / 3];
        x = __fadd_rn(x, n.x);
        y = __fadd_rn(y, n.y);
        z = __fadd_rn(z, n.z);
    }
    const float len2 = __fadd_rn(__fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y)), __fmul_rn(z, z));
    if (len2 == 0.0f) {
        zero[v] = 1u;
        return;
    }
    normalize3(x, y, z);
    out[3 * size_t(v)] = x;
    out[3 * size_t(v) + 1] = y;
    out[3 * size_t(v) + 2] = z;
}

// Vertices without faces keep the zero flag set by the initialisation below.
__global__ void init_zero_kernel(uint32_t* __restrict__ zero, int nv) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v < nv) zero[v] = 1u;
}
__global__ void clear_touched_kernel(const uint32_t* __restrict__ vk, int m, uint32_t* __restrict__ zero) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < m) zero[vk[i]] = 0u;
}

__global__ void gather_vertices_kernel(const float* __restrict__ verts, const uint32_t* __restrict__ list, int m,
                                       float* __restrict__ q) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= m) return;
    const size_t v = list[r];
    q[3 * size_t(r)] = verts[3 * v];
    q[3 * size_t(r) + 1] = verts[3 * v + 1];
    q[3 * size_t(r) + 2] = verts[3 * v + 2];
}

// Fallback: the normal of the nearest point, normalised (Normal ctor).
__global__ void nearest_normal_kernel(const uint32_t* __restrict__ list, const uint32_t* __restrict__ idx,
                                      const int32_t* __restrict__ cnt, int m, Lbvh T,
                                      const float4* __restrict__ normals, float* __restrict__ out) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= m || cnt[r] <= 0) return;
    const float4 n = normals[T.inv[idx[r]]];
    float x = n.x, y = n.y, z = n.z;
    normalize3(x, y, z);
    const size_t v = list[r];
    out[3 * v] = x;
    out[3 * v + 1] = y;
    out[3 * v + 2] = z;
}

__global__ void nearest_color_kernel(const uint32_t* __restrict__ idx, const int32_t* __restrict__ cnt, int nv,
                                     const uint8_t* __restrict__ colors, int width, uint8_t* __restrict__ out) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nv) return;
    const bool ok = cnt[v] > 0;
    const size_t src = ok ? size_t(idx[v]) * width : 0;
    for (int c = 0; c < width; c++) out[size_t(v) * width + c] = ok ? colors[src + c] : uint8_t(0);
}

__global__ void max_index_kernel(const uint32_t* __restrict__ a, size_t n, uint32_t* __restrict__ out) {
    uint32_t m = 0;
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x)
        m = max(m, a[i]);
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

}  // namespace

void mesh_vertex_colors(const Lbvh& T, const float* d_box, const float* verts, int nv, const uint8_t* colors,
                        int width, uint8_t* out, Workspace& ws, int* d_err, cudaStream_t s) {
    if (nv == 0) return;
    float4* qs = ws.get<float4>("vc.qs", size_t(nv));
    sort_queries(verts, nv, d_box, qs, ws, s);
    uint32_t* idx = ws.get<uint32_t>("vc.idx", size_t(nv));
    float* dist = ws.get<float>("vc.dist", size_t(nv));
    int32_t* cnt = ws.get<int32_t>("vc.cnt", size_t(nv));
    knn_rows(T, qs, nv, 1, idx, dist, cnt, ws, d_err, s);
    nearest_color_kernel<<<ceil_div(nv, 256), 256, 0, s>>>(idx, cnt, nv, colors, width, out);
    LVRGB_LAUNCH_CHECK();
}

uint32_t max_index(const uint32_t* a, size_t n, Workspace& ws, cudaStream_t s) {
    if (n == 0) return 0;
    uint32_t* d = ws.get<uint32_t>("vn.max", 1);
    LVRGB_CUDA(cudaMemsetAsync(d, 0, sizeof(uint32_t), s));
    const int blocks = std::min(ceil_div((long long)n, 256), 4096);
    max_index_kernel<<<blocks, 256, 0, s>>>(a, n, d);
    LVRGB_LAUNCH_CHECK();
    uint64_t* h = ws.pinned();
    h[0] = 0;
    LVRGB_CUDA(cudaMemcpyAsync(h, d, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    LVRGB_CUDA(cudaStreamSynchronize(s));
    return uint32_t(h[0]);
}

long long mesh_vertex_normals(const Lbvh& T, const float4* normals, const float* d_box, const float* verts,
                              int nv, const uint32_t* faces, int nf, float* out, Workspace& ws, int* d_err,
                              cudaStream_t s) {
    if (nv == 0) return 0;
    LVRGB_CUDA(cudaMemsetAsync(out, 0, sizeof(float) * 3 * size_t(nv), s));
    uint32_t* zero = ws.get<uint32_t>("vn.zero", size_t(nv));
    init_zero_kernel<<<ceil_div(nv, 256), 256, 0, s>>>(zero, nv);
    LVRGB_LAUNCH_CHECK();
    if (nf > 0) {
        const int m = 3 * nf;
        float4* fn = ws.get<float4>("vn.fn", size_t(nf));
        face_normals_kernel<<<ceil_div(nf, 256), 256, 0, s>>>(verts, faces, nf, fn);
        LVRGB_LAUNCH_CHECK();
        uint32_t* vk = ws.get<uint32_t>("vn.vk", size_t(m));
        uint32_t* vk2 = ws.get<uint32_t>("vn.vk2", size_t(m));
        uint32_t* rv = ws.get<uint32_t>("vn.rv", size_t(m));
        uint32_t* rv2 = ws.get<uint32_t>("vn.rv2", size_t(m));
        LVRGB_CUDA(cudaMemcpyAsync(vk, faces, sizeof(uint32_t) * size_t(m), cudaMemcpyDeviceToDevice, s));
        iota_u32(rv, size_t(m), s);
        int bits = 1;
        while (bits < 32 && (uint64_t(1) << bits) < uint64_t(nv)) bits++;
        void* tmp = ws.get<unsigned char>("vn.sorttmp", radix_sort_temp_bytes<uint32_t>(size_t(m)));
        if (radix_sort_pairs<uint32_t>(vk, rv, vk2, rv2, size_t(m), 0, bits, tmp, s)) {
            std::swap(vk, vk2);
            std::swap(rv, rv2);
        }
        clear_touched_kernel<<<ceil_div(m, 256), 256, 0, s>>>(vk, m, zero);
        LVRGB_LAUNCH_CHECK();
        vertex_sum_kernel<<<ceil_div(m, 256), 256, 0, s>>>(vk, rv, m, fn, out, zero);
        LVRGB_LAUNCH_CHECK();
    }
    // vertices without a usable face-normal sum
    uint32_t* ids = ws.get<uint32_t>("vn.ids", size_t(nv));
    uint32_t* pos = ws.get<uint32_t>("vn.pos", size_t(nv) + 1);
    uint32_t* list = ws.get<uint32_t>("vn.list", size_t(nv));
    iota_u32(ids, size_t(nv), s);
    void* stmp = ws.get<unsigned char>("vn.scantmp", scan_temp_bytes(size_t(nv)));
    exclusive_scan_u32(zero, pos, size_t(nv), stmp, pos + nv, s);
    scatter_flagged_u32(ids, zero, pos, size_t(nv), list, s);
    uint64_t* h = ws.pinned();
    h[0] = 0;
    LVRGB_CUDA(cudaMemcpyAsync(h, pos + nv, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    LVRGB_CUDA(cudaStreamSynchronize(s));
    const int mz = int(uint32_t(h[0]));
    if (mz > 0 && T.n > 0) {
        float* q = ws.get<float>("vn.q", size_t(mz) * 3);
        gather_vertices_kernel<<<ceil_div(mz, 256), 256, 0, s>>>(verts, list, mz, q);
        LVRGB_LAUNCH_CHECK();
        float4* qs = ws.get<float4>("vn.qs", size_t(mz));
        sort_queries(q, mz, d_box, qs, ws, s);
        uint32_t* idx = ws.get<uint32_t>("vn.idx", size_t(mz));
        float* dist = ws.get<float>("vn.dist", size_t(mz));
        int32_t* cnt = ws.get<int32_t>("vn.cnt", size_t(mz));
        knn_rows(T, qs, mz, 1, idx, dist, cnt, ws, d_err, s);
        nearest_normal_kernel<<<ceil_div(mz, 256), 256, 0, s>>>(list, idx, cnt, mz, T, normals, out);
        LVRGB_LAUNCH_CHECK();
    }
    return mz;
}

}  // namespace lvrgb

// ---------------------------------------------------------------------------
// Half-edge connectivity (pmp::SurfaceMesh layout) of the triangle soup.
// pmp's add_face (src/liblvr2/geometry/pmp/SurfaceMesh.cpp:283-460) builds it
// face by face; here the same connectivity comes from sorts:
//   - edges are numbered in the order of their first appearance in the face
//     list (face f, corners 0, 1, 2), as add_face creates them, and halfedge
//     2e points the way the edge first appeared (new_edge(start, end));
//   - face halfedges link corner to corner; face_he = the halfedge of corner
//     2 (add_face's halfedges[n - 1]);
//   - a boundary halfedge links to the boundary halfedge leaving its end
//     vertex; at a vertex with several boundary gaps the incoming and outgoing
//     ones are paired in ascending halfedge order (pmp's pairing depends on
//     the face order there);
//   - vertex_he = the smallest outgoing boundary halfedge on the boundary
//     (pmp keeps a boundary one there), else the smallest outgoing halfedge.
namespace lvrgb {
namespace {

constexpr uint32_t kNone = 0xffffffffu;

__device__ __forceinline__ void corner_pair(const uint32_t* faces, uint32_t r, uint32_t& a, uint32_t& b) {
    const uint32_t f = r / 3, c = r % 3;
    a = faces[3 * size_t(f) + c];
    b = faces[3 * size_t(f) + (c == 2 ? 0 : c + 1)];
}

__global__ void he_keys_kernel(const uint32_t* __restrict__ faces, int m, int vb, uint64_t* __restrict__ keys,
                               uint32_t* __restrict__ vals) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= m) return;
    uint32_t a, b;
    corner_pair(faces, uint32_t(r), a, b);
    const uint64_t lo = min(a, b), hi = max(a, b);
    keys[r] = (lo << vb) | hi;
    vals[r] = uint32_t(r);
}

// Per run of equal undirected edges (head at p): start, first reference.
__global__ void he_runs_kernel(const uint32_t* __restrict__ vals, const uint32_t* __restrict__ flags,
                               const uint32_t* __restrict__ pos, int m, uint32_t* __restrict__ run_start,
                               uint32_t* __restrict__ run_first) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= m || !flags[p]) return;
    run_start[pos[p]] = uint32_t(p);
    run_first[pos[p]] = vals[p];
}

__global__ void scatter_rank_kernel(const uint32_t* __restrict__ order, int n, uint32_t* __restrict__ rank) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) rank[order[i]] = uint32_t(i);
}

// Halfedge of every face corner; edge endpoints; complex-edge count.
__global__ void he_assign_kernel(const uint32_t* __restrict__ faces, const uint32_t* __restrict__ vals,
                                 const uint32_t* __restrict__ flags, const uint32_t* __restrict__ pos, int m,
                                 int nruns, const uint32_t* __restrict__ run_start,
                                 const uint32_t* __restrict__ run_first, const uint32_t* __restrict__ edge_of_run,
                                 uint32_t* __restrict__ he_of_ref, uint32_t* __restrict__ he_vertex,
                                 uint32_t* __restrict__ he_face, uint32_t* __restrict__ edge_faces,
                                 unsigned long long* __restrict__ complex_edges) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= m) return;
    const uint32_t run = pos[p] + flags[p] - 1u;
    const uint32_t start = run_start[run];
    const uint32_t end = run + 1 < uint32_t(nruns) ? run_start[run + 1] : uint32_t(m);
    const uint32_t cnt = end - start;
    const uint32_t e = edge_of_run[run];
    const uint32_t r = vals[p], r0 = run_first[run];
    uint32_t a, b, a0, b0;
    corner_pair(faces, r, a, b);
    corner_pair(faces, r0, a0, b0);
    const uint32_t h = (a == a0) ? 2 * e : 2 * e + 1;
    he_of_ref[r] = h;
    he_face[h] = r / 3;
    if (flags[p]) {
        he_vertex[2 * e] = b0;
        he_vertex[2 * e + 1] = a0;
        edge_faces[e] = cnt;
        const bool complex_edge = cnt > 2 || a0 == b0 ||
                                  (cnt == 2 && [&] {
                                      uint32_t a1, b1;
                                      corner_pair(faces, vals[p + 1], a1, b1);
                                      return a1 == a0;  // the same orientation twice
                                  }());
        if (complex_edge) atomicAdd(complex_edges, 1ull);
    }
}

__global__ void he_face_links_kernel(const uint32_t* __restrict__ he_of_ref, int nf, uint32_t* __restrict__ he_next,
                                     uint32_t* __restrict__ face_he) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nf) return;
    const uint32_t h0 = he_of_ref[3 * size_t(f)], h1 = he_of_ref[3 * size_t(f) + 1],
                   h2 = he_of_ref[3 * size_t(f) + 2];
    he_next[h0] = h1;
    he_next[h1] = h2;
    he_next[h2] = h0;
    face_he[f] = h2;
}

// Boundary halfedges (of edges with one face: 2e + 1) keyed by their start
// and end vertices, in ascending halfedge order.
__global__ void he_boundary_kernel(const uint32_t* __restrict__ edge_faces, const uint32_t* __restrict__ flags,
                                   const uint32_t* __restrict__ pos, int ne, const uint32_t* __restrict__ he_vertex,
                                   uint64_t* __restrict__ from_key, uint32_t* __restrict__ from_val,
                                   uint64_t* __restrict__ to_key, uint32_t* __restrict__ to_val) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne || !flags[e]) return;
    const uint32_t b = 2 * uint32_t(e) + 1, i = pos[e];
    from_key[i] = he_vertex[b ^ 1u];  // b leaves the end of its opposite
    to_key[i] = he_vertex[b];
    from_val[i] = b;
    to_val[i] = b;
}

__global__ void edge_flag_kernel(const uint32_t* __restrict__ edge_faces, int ne, uint32_t* __restrict__ flags) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e < ne) flags[e] = edge_faces[e] == 1 ? 1u : 0u;
}

// Group start and size per vertex of a sorted (vertex, halfedge) list.
__global__ void vertex_groups_kernel(const uint64_t* __restrict__ keys, int nb, uint32_t* __restrict__ start,
                                     uint32_t* __restrict__ count) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nb) return;
    const uint32_t v = uint32_t(keys[p]);
    if (p == 0 || keys[p - 1] != keys[p]) {
        int q = p;
        while (q < nb && keys[q] == keys[p]) q++;
        start[v] = uint32_t(p);
        count[v] = uint32_t(q - p);
    }
}

// next of the k-th incoming boundary halfedge of a vertex = its k-th outgoing one.
__global__ void he_boundary_links_kernel(const uint64_t* __restrict__ to_key, const uint32_t* __restrict__ to_val,
                                         int nb, const uint32_t* __restrict__ in_start,
                                         const uint32_t* __restrict__ out_start,
                                         const uint32_t* __restrict__ out_count,
                                         const uint32_t* __restrict__ from_val, uint32_t* __restrict__ he_next,
                                         unsigned long long* __restrict__ bad) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nb) return;
    const uint32_t v = uint32_t(to_key[p]);
    const uint32_t k = uint32_t(p) - in_start[v];
    if (out_start[v] == kNone || k >= out_count[v]) {
        atomicAdd(bad, 1ull);
        return;
    }
    he_next[to_val[p]] = from_val[out_start[v] + k];
}

__global__ void he_prev_kernel(const uint32_t* __restrict__ he_next, int nh, uint32_t* __restrict__ he_prev) {
    const int h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= nh) return;
    const uint32_t n = he_next[h];
    if (n != kNone) he_prev[n] = uint32_t(h);
}

__global__ void he_vertex_min_kernel(const uint32_t* __restrict__ he_vertex, const uint32_t* __restrict__ he_face,
                                     int nh, uint32_t* __restrict__ vmin_all, uint32_t* __restrict__ vmin_b) {
    const int h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= nh) return;
    const uint32_t v = he_vertex[uint32_t(h) ^ 1u];  // h leaves v
    atomicMin(vmin_all + v, uint32_t(h));
    if (he_face[h] == kNone) atomicMin(vmin_b + v, uint32_t(h));
}

__global__ void he_vertex_pick_kernel(const uint32_t* __restrict__ vmin_all, const uint32_t* __restrict__ vmin_b,
                                      const uint32_t* __restrict__ out_count, int nv,
                                      uint32_t* __restrict__ vertex_he, unsigned long long* __restrict__ complex_v) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nv) return;
    vertex_he[v] = vmin_b[v] != kNone ? vmin_b[v] : vmin_all[v];
    if (out_count[v] > 1 && out_count[v] != kNone) atomicAdd(complex_v, 1ull);
}

template <typename T>
__global__ void fill_kernel(T* __restrict__ a, size_t n, T v) {
    const size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
    if (i < n) a[i] = v;
}

template <typename T>
void fill(T* a, size_t n, T v, cudaStream_t s) {
    if (n == 0) return;
    fill_kernel<<<ceil_div((long long)n, 256), 256, 0, s>>>(a, n, v);
    LVRGB_LAUNCH_CHECK();
}

uint64_t read_count(Workspace& ws, const void* d, size_t bytes, cudaStream_t s) {
    uint64_t* h = ws.pinned();
    h[0] = 0;
    LVRGB_CUDA(cudaMemcpyAsync(h, d, bytes, cudaMemcpyDeviceToHost, s));
    LVRGB_CUDA(cudaStreamSynchronize(s));
    return h[0];
}

}  // namespace

void build_halfedges(const uint32_t* faces, int nf, int nv, Workspace& ws, HalfedgeMesh& H, cudaStream_t s) {
    H = HalfedgeMesh();
    H.nverts = nv;
    H.nfaces = nf;
    const int m = 3 * nf;
    unsigned long long* counters = ws.get<unsigned long long>("he.counters", 4);
    LVRGB_CUDA(cudaMemsetAsync(counters, 0, 4 * sizeof(unsigned long long), s));
    uint32_t* vertex_he = ws.get<uint32_t>("he.vertex_he", std::max(nv, 1));
    uint32_t* face_he = ws.get<uint32_t>("he.face_he", std::max(nf, 1));
    H.vertex_he = vertex_he;
    H.face_he = face_he;
    if (m == 0) {
        fill<uint32_t>(vertex_he, size_t(nv), kNone, s);
        H.he_vertex = H.he_next = H.he_prev = H.he_face = ws.get<uint32_t>("he.empty", 1);
        return;
    }
    int vb = 1;
    while (vb < 32 && (uint64_t(1) << vb) < uint64_t(nv)) vb++;
    // (undirected edge, corner reference), sorted: runs are edges
    uint64_t* k = ws.get<uint64_t>("he.k", m);
    uint64_t* k2 = ws.get<uint64_t>("he.k2", m);
    uint32_t* v = ws.get<uint32_t>("he.v", m);
    uint32_t* v2 = ws.get<uint32_t>("he.v2", m);
    he_keys_kernel<<<ceil_div(m, 256), 256, 0, s>>>(faces, m, vb, k, v);
    LVRGB_LAUNCH_CHECK();
    void* tmp = ws.get<unsigned char>("he.sorttmp", radix_sort_temp_bytes<uint64_t>(size_t(m)));
    if (radix_sort_pairs<uint64_t>(k, v, k2, v2, size_t(m), 0, 2 * vb, tmp, s)) {
        std::swap(k, k2);
        std::swap(v, v2);
    }
    uint32_t* flags = ws.get<uint32_t>("he.flags", m);
    uint32_t* pos = ws.get<uint32_t>("he.pos", size_t(m) + 1);
    head_flags_u64(k, size_t(m), flags, s);
    void* stmp = ws.get<unsigned char>("he.scantmp", scan_temp_bytes(size_t(m)));
    exclusive_scan_u32(flags, pos, size_t(m), stmp, pos + m, s);
    const int ne = int(read_count(ws, pos + m, sizeof(uint32_t), s));
    H.nedges = ne;
    const int nh = 2 * ne;
    uint32_t* run_start = ws.get<uint32_t>("he.run_start", ne);
    uint32_t* run_first = ws.get<uint32_t>("he.run_first", ne);
    he_runs_kernel<<<ceil_div(m, 256), 256, 0, s>>>(v, flags, pos, m, run_start, run_first);
    LVRGB_LAUNCH_CHECK();
    // edge ids: runs in order of their first appearance
    uint32_t* fk = ws.get<uint32_t>("he.fk", ne);
    uint32_t* fk2 = ws.get<uint32_t>("he.fk2", ne);
    uint32_t* order = ws.get<uint32_t>("he.order", ne);
    uint32_t* order2 = ws.get<uint32_t>("he.order2", ne);
    LVRGB_CUDA(cudaMemcpyAsync(fk, run_first, sizeof(uint32_t) * size_t(ne), cudaMemcpyDeviceToDevice, s));
    iota_u32(order, size_t(ne), s);
    void* tmp32 = ws.get<unsigned char>("he.sorttmp32", radix_sort_temp_bytes<uint32_t>(size_t(ne)));
    int rb = 1;
    while (rb < 32 && (uint64_t(1) << rb) < uint64_t(m)) rb++;
    if (radix_sort_pairs<uint32_t>(fk, order, fk2, order2, size_t(ne), 0, rb, tmp32, s)) std::swap(order, order2);
    uint32_t* edge_of_run = ws.get<uint32_t>("he.edge_of_run", ne);
    scatter_rank_kernel<<<ceil_div(ne, 256), 256, 0, s>>>(order, ne, edge_of_run);
    LVRGB_LAUNCH_CHECK();
    // halfedges of the face corners
    uint32_t* he_of_ref = ws.get<uint32_t>("he.of_ref", m);
    uint32_t* he_vertex = ws.get<uint32_t>("he.vertex", nh);
    uint32_t* he_face = ws.get<uint32_t>("he.face", nh);
    uint32_t* he_next = ws.get<uint32_t>("he.next", nh);
    uint32_t* he_prev = ws.get<uint32_t>("he.prev", nh);
    uint32_t* edge_faces = ws.get<uint32_t>("he.edge_faces", ne);
    fill<uint32_t>(he_face, size_t(nh), kNone, s);
    fill<uint32_t>(he_next, size_t(nh), kNone, s);
    fill<uint32_t>(he_prev, size_t(nh), kNone, s);
    he_assign_kernel<<<ceil_div(m, 256), 256, 0, s>>>(faces, v, flags, pos, m, ne, run_start, run_first, edge_of_run,
                                                      he_of_ref, he_vertex, he_face, edge_faces, counters);
    LVRGB_LAUNCH_CHECK();
    H.he_vertex = he_vertex;
    H.he_face = he_face;
    H.he_next = he_next;
    H.he_prev = he_prev;
    H.complex_edges = (long long)read_count(ws, counters, sizeof(unsigned long long), s);
    if (H.complex_edges > 0) return;
    he_face_links_kernel<<<ceil_div(nf, 256), 256, 0, s>>>(he_of_ref, nf, he_next, face_he);
    LVRGB_LAUNCH_CHECK();
    // boundary halfedges and their links
    uint32_t* bflags = ws.get<uint32_t>("he.bflags", ne);
    uint32_t* bpos = ws.get<uint32_t>("he.bpos", size_t(ne) + 1);
    edge_flag_kernel<<<ceil_div(ne, 256), 256, 0, s>>>(edge_faces, ne, bflags);
    LVRGB_LAUNCH_CHECK();
    void* stmp2 = ws.get<unsigned char>("he.scantmp2", scan_temp_bytes(size_t(ne)));
    exclusive_scan_u32(bflags, bpos, size_t(ne), stmp2, bpos + ne, s);
    const int nb = int(read_count(ws, bpos + ne, sizeof(uint32_t), s));
    H.boundary = nb;
    uint32_t* out_start = ws.get<uint32_t>("he.out_start", std::max(nv, 1));
    uint32_t* out_count = ws.get<uint32_t>("he.out_count", std::max(nv, 1));
    fill<uint32_t>(out_start, size_t(nv), kNone, s);
    fill<uint32_t>(out_count, size_t(nv), 0u, s);
    if (nb > 0) {
        uint64_t* fk64 = ws.get<uint64_t>("he.bfk", nb);
        uint64_t* fk64b = ws.get<uint64_t>("he.bfk2", nb);
        uint32_t* fv = ws.get<uint32_t>("he.bfv", nb);
        uint32_t* fvb = ws.get<uint32_t>("he.bfv2", nb);
        uint64_t* tk64 = ws.get<uint64_t>("he.btk", nb);
        uint64_t* tk64b = ws.get<uint64_t>("he.btk2", nb);
        uint32_t* tv = ws.get<uint32_t>("he.btv", nb);
        uint32_t* tvb = ws.get<uint32_t>("he.btv2", nb);
        he_boundary_kernel<<<ceil_div(ne, 256), 256, 0, s>>>(edge_faces, bflags, bpos, ne, he_vertex, fk64, fv, tk64,
                                                             tv);
        LVRGB_LAUNCH_CHECK();
        void* btmp = ws.get<unsigned char>("he.bsorttmp", radix_sort_temp_bytes<uint64_t>(size_t(nb)));
        if (radix_sort_pairs<uint64_t>(fk64, fv, fk64b, fvb, size_t(nb), 0, vb, btmp, s)) {
            std::swap(fk64, fk64b);
            std::swap(fv, fvb);
        }
        if (radix_sort_pairs<uint64_t>(tk64, tv, tk64b, tvb, size_t(nb), 0, vb, btmp, s)) {
            std::swap(tk64, tk64b);
            std::swap(tv, tvb);
        }
        uint32_t* in_start = ws.get<uint32_t>("he.in_start", std::max(nv, 1));
        uint32_t* in_count = ws.get<uint32_t>("he.in_count", std::max(nv, 1));
        vertex_groups_kernel<<<ceil_div(nb, 256), 256, 0, s>>>(fk64, nb, out_start, out_count);
        LVRGB_LAUNCH_CHECK();
        vertex_groups_kernel<<<ceil_div(nb, 256), 256, 0, s>>>(tk64, nb, in_start, in_count);
        LVRGB_LAUNCH_CHECK();
        he_boundary_links_kernel<<<ceil_div(nb, 256), 256, 0, s>>>(tk64, tv, nb, in_start, out_start, out_count, fv,
                                                                   he_next, counters + 1);
        LVRGB_LAUNCH_CHECK();
    }
    he_prev_kernel<<<ceil_div(nh, 256), 256, 0, s>>>(he_next, nh, he_prev);
    LVRGB_LAUNCH_CHECK();
    uint32_t* vmin_all = ws.get<uint32_t>("he.vmin_all", std::max(nv, 1));
    uint32_t* vmin_b = ws.get<uint32_t>("he.vmin_b", std::max(nv, 1));
    fill<uint32_t>(vmin_all, size_t(nv), kNone, s);
    fill<uint32_t>(vmin_b, size_t(nv), kNone, s);
    he_vertex_min_kernel<<<ceil_div(nh, 256), 256, 0, s>>>(he_vertex, he_face, nh, vmin_all, vmin_b);
    LVRGB_LAUNCH_CHECK();
    he_vertex_pick_kernel<<<ceil_div(nv, 256), 256, 0, s>>>(vmin_all, vmin_b, out_count, nv, vertex_he, counters + 2);
    LVRGB_LAUNCH_CHECK();
    uint64_t c[4] = {0, 0, 0, 0};
    uint64_t* h = ws.pinned();
    LVRGB_CUDA(cudaMemcpyAsync(h, counters, 4 * sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
    LVRGB_CUDA(cudaStreamSynchronize(s));
    std::memcpy(c, h, sizeof(c));
    if (c[1] != 0) throw std::runtime_error("inconsistent boundary: a vertex has more incoming than outgoing boundary halfedges");
    H.complex_vertices = (long long)c[2];
}

}  // namespace lvrgb
