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
