// adjoint.cu -- reverse-mode gradients of AdaptiveKSearchSurface::distance
// (AdaptiveKSearchSurface.tcc:414-457) and Newton projection onto its zero
// level.
//
// For a position q with kd nearest points p_j and normals n_j (the
// neighbourhood is held fixed: it is piecewise constant in q):
//   c = mean(p_j), m = mean(n_j), nh = m / |m|, r = q - c,
//   d = r . nh (projected distance), e = |r| (Euclidean distance).
// With upstream gradients gd (of d) and ge (of e):
//   dL/dq   = gd nh + ge r / e
//   dL/dp_j = -(dL/dq) / kd                       for every neighbour j
//   dL/dn_j = gd (r - d nh) / (kd |m|)             for every neighbour j
// The per-neighbour terms are scatter-added with float4 atomics (sums of
// float atomics: the last bits depend on the order of the additions).
#include <stdexcept>

#include "adjoint.h"
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

// The signed distance of one position from its sorted heap: the sums in
// ascending (d2, index) order with the operations of the forward kernel.
struct SdfEval {
    int cnt;
    float r[3];   // q - mean point
    float nh[3];  // normalised mean normal
    float mlen;   // |mean normal| before normalisation
    float proj, eucl;
};

template <class Heap>
__device__ __forceinline__ SdfEval eval_sdf(const Lbvh& T, const float4* __restrict__ normals, const Heap& heap,
                                            float qx, float qy, float qz) {
    SdfEval E;
    float px = 0, py = 0, pz = 0, nx = 0, ny = 0, nz = 0;
    E.cnt = heap.real;
#pragma unroll 4
    for (int s = 0; s < E.cnt; s++) {
        const uint32_t j = __ldg(T.inv + key_idx(heap.at(s)));
        const float4 p = __ldg(T.pts + j);
        const float4 nn = __ldg(normals + j);
        px = __fadd_rn(px, p.x); py = __fadd_rn(py, p.y); pz = __fadd_rn(pz, p.z);
        nx = __fadd_rn(nx, nn.x); ny = __fadd_rn(ny, nn.y); nz = __fadd_rn(nz, nn.z);
    }
    if (E.cnt == 0) {
        E.proj = E.eucl = FLT_MAX;
        E.mlen = 0.0f;
        for (int a = 0; a < 3; a++) E.r[a] = E.nh[a] = 0.0f;
        return E;
    }
    const float c = float(E.cnt);
    nx = __fdiv_rn(nx, c); ny = __fdiv_rn(ny, c); nz = __fdiv_rn(nz, c);
    px = __fdiv_rn(px, c); py = __fdiv_rn(py, c); pz = __fdiv_rn(pz, c);
    E.mlen = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(nx, nx), __fmul_rn(ny, ny)), __fmul_rn(nz, nz)));
    normalize3(nx, ny, nz);
    E.nh[0] = nx; E.nh[1] = ny; E.nh[2] = nz;
    E.r[0] = __fsub_rn(qx, px); E.r[1] = __fsub_rn(qy, py); E.r[2] = __fsub_rn(qz, pz);
    E.proj = __fadd_rn(__fadd_rn(__fmul_rn(E.r[0], nx), __fmul_rn(E.r[1], ny)), __fmul_rn(E.r[2], nz));
    E.eucl = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(E.r[0], E.r[0]), __fmul_rn(E.r[1], E.r[1])),
                                  __fmul_rn(E.r[2], E.r[2])));
    return E;
}

struct GradArgs {
    Lbvh T;
    int K;
    const float4* normals;
    const float4* qs;
    int nq;
    AdjointOut out;
    unsigned long long* gheap;
    int* err;
    int* tiles = nullptr;  // tile counter of a persistent launch
};

template <class Heap>
__global__ void __launch_bounds__(kWarpsPerBlock * 32) sdf_adjoint_kernel(GradArgs A) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31;
    const WarpCtx ctx = warp_ctx<kWarpsPerBlock>(smem, A.gheap, A.K);
    for (int tile = first_tile<kWarpsPerBlock>(A.tiles); tile * 32 < A.nq;
         tile = next_tile<kWarpsPerBlock>(A.tiles, tile)) {
        const int qi = tile * 32 + lane;
        const bool active = qi < A.nq;
        const float4 q = active ? A.qs[qi] : make_float4(0, 0, 0, 0);
        Heap heap;
        heap.init(ctx.heap, A.K);
        const float4 q0 = A.qs[tile * 32];
        knn_traverse(A.T, q.x, q.y, q.z, active, heap, ctx.stage, A.err, seed_bucket_for(A.T, q0.x, q0.y, q0.z));
        if (!active) continue;
        heap.sort_ascending();
        const SdfEval E = eval_sdf(A.T, A.normals, heap, q.x, q.y, q.z);
        const size_t row = __float_as_uint(q.w);
        if (A.out.dist) A.out.dist[row] = E.proj;
        if (A.out.eucl) A.out.eucl[row] = E.eucl;
        if (E.cnt == 0) {
            if (A.out.gq) A.out.gq[3 * row] = A.out.gq[3 * row + 1] = A.out.gq[3 * row + 2] = 0.0f;
            continue;
        }
        const float gd = A.out.gdist ? A.out.gdist[row] : 0.0f;
        const float ge = A.out.geucl ? A.out.geucl[row] : 0.0f;
        float g[3];
        const float ger = E.eucl > 0.0f ? ge / E.eucl : 0.0f;
#pragma unroll
        for (int a = 0; a < 3; a++) g[a] = gd * E.nh[a] + ger * E.r[a];
        if (A.out.gq) {
            A.out.gq[3 * row] = g[0];
            A.out.gq[3 * row + 1] = g[1];
            A.out.gq[3 * row + 2] = g[2];
        }
        const float inv_k = 1.0f / float(E.cnt);
        const float4 gp = make_float4(-g[0] * inv_k, -g[1] * inv_k, -g[2] * inv_k, 0.0f);
        float4 gn = make_float4(0, 0, 0, 0);
        const bool has_gn = A.out.gn && E.mlen > 0.0f && gd != 0.0f;
        if (has_gn) {
            const float w = gd * inv_k / E.mlen;
            gn = make_float4(w * (E.r[0] - E.proj * E.nh[0]), w * (E.r[1] - E.proj * E.nh[1]),
                             w * (E.r[2] - E.proj * E.nh[2]), 0.0f);
        }
        if (A.out.gp || has_gn) {
            for (int s = 0; s < E.cnt; s++) {
                const uint32_t j = __ldg(A.T.inv + key_idx(heap.at(s)));
                if (A.out.gp) atomicAdd(A.out.gp + j, gp);
                if (has_gn) atomicAdd(A.out.gn + j, gn);
            }
        }
    }
}

struct ProjectArgs {
    Lbvh T;
    int K;
    const float4* normals;
    const float4* qs;
    int nq;
    int steps;
    float* out_pos;
    float* out_normal;
    unsigned long long* gheap;
    int* err;
    int* tiles = nullptr;  // tile counter of a persistent launch
};

// Newton steps toward the zero level: x <- x - d(x) nh(x), a new kd
// neighbourhood at every step.
template <class Heap>
__global__ void __launch_bounds__(kWarpsPerBlock * 32) project_kernel(ProjectArgs A) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31;
    const WarpCtx ctx = warp_ctx<kWarpsPerBlock>(smem, A.gheap, A.K);
    for (int tile = first_tile<kWarpsPerBlock>(A.tiles); tile * 32 < A.nq;
         tile = next_tile<kWarpsPerBlock>(A.tiles, tile)) {
        const int qi = tile * 32 + lane;
        const bool active = qi < A.nq;
        const float4 q = active ? A.qs[qi] : make_float4(0, 0, 0, 0);
        float x = q.x, y = q.y, z = q.z;
        float nh[3] = {0, 0, 0};
        for (int step = 0; step < A.steps; step++) {
            Heap heap;
            heap.init(ctx.heap, A.K);
            const float sx = __shfl_sync(kFull, x, 0), sy = __shfl_sync(kFull, y, 0), sz = __shfl_sync(kFull, z, 0);
            knn_traverse(A.T, x, y, z, active, heap, ctx.stage, A.err, seed_bucket_for(A.T, sx, sy, sz));
            if (active) {
                heap.sort_ascending();
                const SdfEval E = eval_sdf(A.T, A.normals, heap, x, y, z);
                if (E.cnt > 0) {
                    nh[0] = E.nh[0]; nh[1] = E.nh[1]; nh[2] = E.nh[2];
                    x = __fsub_rn(x, __fmul_rn(E.proj, nh[0]));
                    y = __fsub_rn(y, __fmul_rn(E.proj, nh[1]));
                    z = __fsub_rn(z, __fmul_rn(E.proj, nh[2]));
                }
            }
            __syncwarp();
        }
        if (!active) continue;
        const size_t row = __float_as_uint(q.w);
        if (A.out_pos) {
            A.out_pos[3 * row] = x;
            A.out_pos[3 * row + 1] = y;
            A.out_pos[3 * row + 2] = z;
        }
        if (A.out_normal) {
            A.out_normal[3 * row] = nh[0];
            A.out_normal[3 * row + 1] = nh[1];
            A.out_normal[3 * row + 2] = nh[2];
        }
    }
}

template <typename Kernel>
void set_smem(Kernel k, size_t bytes) {
    if (bytes > 48 * 1024) LVRGB_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(bytes)));
}

}  // namespace

void distance_adjoint(const Lbvh& T, const float4* normals, int kd, const float4* qs, int nq, const AdjointOut& out,
                      Workspace& ws, int* d_err, cudaStream_t s) {
    if (nq == 0) return;
    GradArgs A;
    A.T = T;
    A.K = kd > 0 ? kd : 1;
    A.normals = normals;
    A.qs = qs;
    A.nq = nq;
    A.out = out;
    A.err = d_err;
    HeapPlan P = plan_heap(nq, A.K, ws);
    A.gheap = P.gheap;
    if (complete_3ary(A.K)) {
        set_smem(sdf_adjoint_kernel<LaneHeap3>, P.smem);
        A.tiles = persistent_tiles(sdf_adjoint_kernel<LaneHeap3>, P, ws, s);
        sdf_adjoint_kernel<LaneHeap3><<<P.blocks, kWarpsPerBlock * 32, P.smem, s>>>(A);
    } else {
        set_smem(sdf_adjoint_kernel<LaneHeap>, P.smem);
        A.tiles = persistent_tiles(sdf_adjoint_kernel<LaneHeap>, P, ws, s);
        sdf_adjoint_kernel<LaneHeap><<<P.blocks, kWarpsPerBlock * 32, P.smem, s>>>(A);
    }
    LVRGB_LAUNCH_CHECK();
}

void project_to_surface(const Lbvh& T, const float4* normals, int kd, const float4* qs, int nq, int steps,
                        float* out_pos, float* out_normal, Workspace& ws, int* d_err, cudaStream_t s) {
    if (nq == 0) return;
    if (steps < 1 || steps > 64) throw std::invalid_argument("steps must be in 1..64");
    ProjectArgs A;
    A.T = T;
    A.K = kd > 0 ? kd : 1;
    A.normals = normals;
    A.qs = qs;
    A.nq = nq;
    A.steps = steps;
    A.out_pos = out_pos;
    A.out_normal = out_normal;
    A.err = d_err;
    HeapPlan P = plan_heap(nq, A.K, ws);
    A.gheap = P.gheap;
    if (complete_3ary(A.K)) {
        set_smem(project_kernel<LaneHeap3>, P.smem);
        A.tiles = persistent_tiles(project_kernel<LaneHeap3>, P, ws, s);
        project_kernel<LaneHeap3><<<P.blocks, kWarpsPerBlock * 32, P.smem, s>>>(A);
    } else {
        set_smem(project_kernel<LaneHeap>, P.smem);
        A.tiles = persistent_tiles(project_kernel<LaneHeap>, P, ws, s);
        project_kernel<LaneHeap><<<P.blocks, kWarpsPerBlock * 32, P.smem, s>>>(A);
    }
    LVRGB_LAUNCH_CHECK();
}

}  // namespace lvrgb
