// grid.cu -- PointsetGrid on the GPU: cell discovery and extrusion as sorted
// lattice keys, grid vertices deduplicated by key, the kd-weighted signed
// distance at every vertex, invalid-cell culling, and marching cubes with
// edge-key vertex deduplication and compacted face output.
//
// Lattice keys are 3-D Morton codes of (coordinate - base), 20 bits per axis,
// so that sorted cells and vertices are spatially coherent: consecutive grid
// vertices form the 32-query groups of the signed-distance kNN.
#include <algorithm>
#include <climits>
#include <cmath>
#include <mutex>
#include <optional>
#include <stdexcept>

#include <cuda.h>  // CUtensorMap and its enums (the encoder is fetched from the driver at run time)

#include "grid.h"
#include "nvtx.h"
#include "primitives.cuh"
#include "surface.h"

namespace lvrgb {

namespace {

// Cell corner offsets (box_creation_table of FastReconstructionTables.hpp:86,
// mapped from -1/+1 to 0/1) and corner pairs of the 12 cell edges
// (vertex_edge_table of FastBoxTables.hpp:71).
__constant__ int c_corner[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                                   {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
__constant__ int c_edge[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {4, 5}, {5, 6},
                                  {6, 7}, {7, 4}, {0, 4}, {1, 5}, {3, 7}, {2, 6}};
__constant__ unsigned long long c_mc[256] = {
#include "mc_table.inc"
};

constexpr uint64_t kNoKey = ~0ull;

struct Frame {
    float vs;
    int bx, by, bz;  // base
    float lo[3], hi[3];
};

__device__ __forceinline__ float cell_center(int idx, float vs) { return __fmul_rn(__fadd_rn(float(idx), 0.5f), vs); }
// Grid vertex coordinate: the centre of the cell whose lowest corner it is,
// plus (-1) * (vs / 2) (HashGrid::addBox, HashGrid.tcc:235-259).
__device__ __forceinline__ float lattice_coord(int L, float vs) {
    return __fadd_rn(cell_center(L, vs), -__fdiv_rn(vs, 2.0f));
}
__device__ __forceinline__ bool inside(const Frame& F, float x, float y, float z) {
    return (F.lo[0] <= x && F.hi[0] >= x) && (F.lo[1] <= y && F.hi[1] >= y) && (F.lo[2] <= z && F.hi[2] >= z);
}

__global__ void point_cells_kernel(const float4* __restrict__ pts, int n, Frame F, uint64_t* __restrict__ keys) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 p = pts[i];
    // HashGrid::calcIndex (HashGrid.hpp:263-268)
    int ix = int(floorf(__fdiv_rn(p.x, F.vs)));
    int iy = int(floorf(__fdiv_rn(p.y, F.vs)));
    int iz = int(floorf(__fdiv_rn(p.z, F.vs)));
    bool ok = inside(F, cell_center(ix, F.vs), cell_center(iy, F.vs), cell_center(iz, F.vs));
    keys[i] = ok ? lattice_key(uint32_t(ix - F.bx), uint32_t(iy - F.by), uint32_t(iz - F.bz)) : kNoKey;
}

__global__ void extrude_kernel(const uint64_t* __restrict__ cells, int nc, Frame F, uint64_t* __restrict__ out) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nc * 27) return;
    int c = t / 27, o = t % 27;
    uint32_t x, y, z;
    lattice_decode(cells[c], x, y, z);
    int dx = o / 9 - 1, dy = (o / 3) % 3 - 1, dz = o % 3 - 1;
    int ix = int(x) + F.bx + dx, iy = int(y) + F.by + dy, iz = int(z) + F.bz + dz;
    bool ok = inside(F, cell_center(ix, F.vs), cell_center(iy, F.vs), cell_center(iz, F.vs));
    out[t] = ok ? lattice_key(uint32_t(int(x) + dx), uint32_t(int(y) + dy), uint32_t(int(z) + dz)) : kNoKey;
}

__global__ void corner_pairs_kernel(const uint64_t* __restrict__ cells, int nc, uint64_t* __restrict__ keys,
                                    uint32_t* __restrict__ vals) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nc * 8) return;
    int c = t >> 3, k = t & 7;
    uint32_t x, y, z;
    lattice_decode(cells[c], x, y, z);
    keys[t] = lattice_key(x + c_corner[k][0], y + c_corner[k][1], z + c_corner[k][2]);
    vals[t] = uint32_t(t);
}

// After sorting (key, slot) pairs: vertex id of every slot and the unique keys.
__global__ void assign_ids_kernel(const uint64_t* __restrict__ keys, const uint32_t* __restrict__ vals,
                                  const uint32_t* __restrict__ flags, const uint32_t* __restrict__ pos, int n,
                                  uint32_t* __restrict__ slot_id, uint64_t* __restrict__ ukeys,
                                  uint32_t* __restrict__ first_slot) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t id = pos[i] + flags[i] - 1u;
    slot_id[vals[i]] = id;
    if (flags[i]) {
        ukeys[id] = keys[i];
        if (first_slot) first_slot[id] = vals[i];
    }
}

// ---- dense form: when the lattice key space is small, a flag per key and a
// scan replace sort + unique; the compacted keys come out sorted and a key's
// scan position is its id.
__global__ void mark_point_cells_kernel(const float4* __restrict__ pts, int n, Frame F, uint32_t* __restrict__ flags) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 p = pts[i];
    int ix = int(floorf(__fdiv_rn(p.x, F.vs)));
    int iy = int(floorf(__fdiv_rn(p.y, F.vs)));
    int iz = int(floorf(__fdiv_rn(p.z, F.vs)));
    if (inside(F, cell_center(ix, F.vs), cell_center(iy, F.vs), cell_center(iz, F.vs)))
        flags[lattice_key(uint32_t(ix - F.bx), uint32_t(iy - F.by), uint32_t(iz - F.bz))] = 1u;
}

__global__ void mark_extrude_kernel(const uint64_t* __restrict__ cells, int nc, Frame F, uint32_t* __restrict__ flags) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nc * 27) return;
    int c = t / 27, o = t % 27;
    uint32_t x, y, z;
    lattice_decode(cells[c], x, y, z);
    int dx = o / 9 - 1, dy = (o / 3) % 3 - 1, dz = o % 3 - 1;
    int ix = int(x) + F.bx + dx, iy = int(y) + F.by + dy, iz = int(z) + F.bz + dz;
    if (inside(F, cell_center(ix, F.vs), cell_center(iy, F.vs), cell_center(iz, F.vs)))
        flags[lattice_key(uint32_t(int(x) + dx), uint32_t(int(y) + dy), uint32_t(int(z) + dz))] = 1u;
}

__global__ void mark_corners_kernel(const uint64_t* __restrict__ cells, int nc, uint32_t* __restrict__ flags) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nc * 8) return;
    int c = t >> 3, k = t & 7;
    uint32_t x, y, z;
    lattice_decode(cells[c], x, y, z);
    flags[lattice_key(x + c_corner[k][0], y + c_corner[k][1], z + c_corner[k][2])] = 1u;
}

__global__ void corner_ids_kernel(const uint64_t* __restrict__ cells, int nc, const uint32_t* __restrict__ pos,
                                  uint32_t* __restrict__ cell_corner) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nc * 8) return;
    int c = t >> 3, k = t & 7;
    uint32_t x, y, z;
    lattice_decode(cells[c], x, y, z);
    cell_corner[t] = pos[lattice_key(x + c_corner[k][0], y + c_corner[k][1], z + c_corner[k][2])];
}

__global__ void dense_compact_kernel(const uint32_t* __restrict__ flags, const uint32_t* __restrict__ pos, size_t N,
                                     uint64_t* __restrict__ out) {
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= N) return;
    if (flags[i]) out[pos[i]] = uint64_t(i);
}

__global__ void mark_refs_kernel(const uint64_t* __restrict__ rk, size_t nref, uint32_t* __restrict__ flags) {
    size_t r = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (r < nref) flags[rk[r]] = 1u;
}

// Face vertex ids and vertex positions from the dense edge map (every
// reference to an edge computes the same position, so the writes agree).
__global__ void dense_refs_kernel(const uint64_t* __restrict__ rk, const float4* __restrict__ rp, size_t nref,
                                  const uint32_t* __restrict__ pos, uint32_t* __restrict__ faces,
                                  float* __restrict__ verts) {
    size_t r = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (r >= nref) return;
    const uint32_t id = pos[rk[r]];
    faces[r] = id;
    const float4 p = rp[r];
    verts[3 * size_t(id)] = p.x;
    verts[3 * size_t(id) + 1] = p.y;
    verts[3 * size_t(id) + 2] = p.z;
}

__global__ void qp_pos_kernel(const uint64_t* __restrict__ keys, int n, Frame F, float4* __restrict__ pos) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t x, y, z;
    lattice_decode(keys[i], x, y, z);
    pos[i] = make_float4(lattice_coord(int(x) + F.bx, F.vs), lattice_coord(int(y) + F.by, F.vs),
                         lattice_coord(int(z) + F.bz, F.vs), __uint_as_float(uint32_t(i)));
}

struct SdfArgs {
    Lbvh T;
    int K;
    const float4* normals;
    const float4* qs;
    int nq;
    double limit;  // 1.75 * voxelsize
    int* tiles = nullptr;  // tile counter of a persistent launch
    unsigned long long* stats = nullptr;  // optional search counters (GridConfig::sdf_stats)
    float* dist;
    float* eucl;
    uint8_t* invalid;
    unsigned long long* gheap;
    int* err;
};

__device__ __forceinline__ void normalize_ieee(float& x, float& y, float& z) {
    if (!(x == 0.0f && y == 0.0f && z == 0.0f)) {
        float len = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y)), __fmul_rn(z, z)));
        x = __fdiv_rn(x, len);
        y = __fdiv_rn(y, len);
        z = __fdiv_rn(z, len);
    }
}

// AdaptiveKSearchSurface::distance (AdaptiveKSearchSurface.tcc:414-457) for
// one query per lane, neighbours summed in ascending (d2, index) order, plus
// the invalid rule of PointsetGrid::calcDistanceValues (PointsetGrid.tcc:133-140).
// Nine resident blocks is what the shared memory allows at kd = 20; at that
// bound the kernel may use 56 registers.
template <class Heap>
__global__ void __launch_bounds__(kWarpsPerBlock * 32, 9) sdf_kernel(SdfArgs A) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31;
    const WarpCtx ctx = warp_ctx<kWarpsPerBlock>(smem, A.gheap, A.K);
    TravStats st;
    for (int tile = first_tile<kWarpsPerBlock>(A.tiles); tile * 32 < A.nq;
         tile = next_tile<kWarpsPerBlock>(A.tiles, tile)) {
        const int qi = tile * 32 + lane;
        const bool active = qi < A.nq;
        const float4 q = active ? A.qs[qi] : make_float4(0, 0, 0, 0);
        Heap heap;
        heap.init(ctx.heap, A.K);
        const float4 q0 = A.qs[tile * 32];
        const int seed = seed_bucket_for(A.T, q0.x, q0.y, q0.z);
        knn_traverse(A.T, q.x, q.y, q.z, active, heap, ctx.stage, A.err, st, seed);
        if (active) {
            heap.sort_ascending();
            float px = 0, py = 0, pz = 0, nx = 0, ny = 0, nz = 0;
            const int cnt = heap.real;
#pragma unroll 4
            for (int s = 0; s < cnt; s++) {
                const unsigned long long key = heap.at(s);
                const uint32_t j = __ldg(A.T.inv + key_idx(key));
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
                normalize_ieee(nx, ny, nz);
                const float dx = __fsub_rn(q.x, px), dy = __fsub_rn(q.y, py), dz = __fsub_rn(q.z, pz);
                proj = __fadd_rn(__fadd_rn(__fmul_rn(dx, nx), __fmul_rn(dy, ny)), __fmul_rn(dz, nz));
                eu = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz)));
            }
            const uint32_t row = __float_as_uint(q.w);
            A.dist[row] = proj;
            if (A.eucl) A.eucl[row] = eu;
            if (A.invalid) A.invalid[row] = double(eu) > A.limit ? 1 : 0;
        }
    }
    if (A.stats) {
        unsigned pushes = st.pushes;
        for (int o = 16; o > 0; o >>= 1) pushes += __shfl_xor_sync(kFull, pushes, o);
        if (lane == 0 && st.nodes) {
            atomicAdd(A.stats + 0, (unsigned long long)st.buckets);
            atomicAdd(A.stats + 1, (unsigned long long)st.nodes);
            atomicAdd(A.stats + 2, (unsigned long long)pushes);
            atomicAdd(A.stats + 3, (unsigned long long)st.chunks);
            atomicAdd(A.stats + 4, (unsigned long long)st.rounds);
        }
    }
}

__global__ void cell_valid_kernel(const uint32_t* __restrict__ corner, int nc, const uint8_t* __restrict__ invalid,
                                  uint32_t* __restrict__ flags) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    bool ok = true;
#pragma unroll
    for (int k = 0; k < 8; k++) ok &= invalid[corner[size_t(c) * 8 + k]] == 0;
    flags[c] = ok ? 1u : 0u;
}

// FastBox::calcIntersection (FastBox.tcc:134-158)
__device__ __forceinline__ float calc_intersection(float x1, float x2, float d1, float d2) {
    if (d1 == 0.0f) return x1;
    if (d2 == 0.0f) return x2;
    if ((d1 < 0.0f && d2 > 0.0f) || (d2 < 0.0f && d1 > 0.0f))
        return __fsub_rn(x2, __fdiv_rn(__fmul_rn(d2, __fsub_rn(x1, x2)), __fsub_rn(d1, d2)));
    return 0.0f;
}

struct McCell {
    int L[3];       // lattice of corner 0
    uint32_t rel[3];
    float d[8];
    int index;
};

__device__ __forceinline__ void load_cell(const uint64_t* cell_keys, const uint32_t* corner, const float* qp_dist,
                                          uint32_t c, const Frame& F, McCell& C) {
    lattice_decode(cell_keys[c], C.rel[0], C.rel[1], C.rel[2]);
    C.L[0] = int(C.rel[0]) + F.bx;
    C.L[1] = int(C.rel[1]) + F.by;
    C.L[2] = int(C.rel[2]) + F.bz;
    C.index = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) {
        C.d[k] = qp_dist[corner[size_t(c) * 8 + k]];
        if (C.d[k] > 0.0f) C.index |= 1 << k;
    }
}

// Position and key of cell edge e (low corner -> high corner along its axis).
__device__ __forceinline__ void edge_vertex(const McCell& C, const Frame& F, int e, float p[3], uint64_t& key) {
    const int a = c_edge[e][0], b = c_edge[e][1];
    int axis = 0;
    if (c_corner[a][1] != c_corner[b][1]) axis = 1;
    if (c_corner[a][2] != c_corner[b][2]) axis = 2;
    const int lo = c_corner[a][axis] < c_corner[b][axis] ? a : b;
    const int hi = lo == a ? b : a;
#pragma unroll
    for (int t = 0; t < 3; t++) p[t] = lattice_coord(C.L[t] + c_corner[lo][t], F.vs);
    const float x2 = lattice_coord(C.L[axis] + 1, F.vs);
    p[axis] = calc_intersection(p[axis], x2, C.d[lo], C.d[hi]);
    key = (lattice_key(C.rel[0] + c_corner[lo][0], C.rel[1] + c_corner[lo][1], C.rel[2] + c_corner[lo][2]) << 2) |
          uint64_t(axis);
}

__device__ __forceinline__ bool same3(const float* a, const float* b) { return a[0] == b[0] && a[1] == b[1] && a[2] == b[2]; }

// FastBox::getSurface / BilinearFastBox::getSurface: count (emit == false)
// or write (emit == true) the faces of valid cell t (index into the valid list).
template <bool kEmit>
__device__ __forceinline__ void mc_cell(const McCell& C, const Frame& F, int pmc, uint32_t t,
                                        uint32_t* __restrict__ counts, const uint32_t* __restrict__ offsets,
                                        uint64_t* __restrict__ ref_key, uint32_t* __restrict__ ref_val,
                                        float4* __restrict__ ref_pos) {
    const unsigned long long word = c_mc[C.index];
    const int ntri = int(word >> 60);
    uint32_t f = kEmit ? offsets[t] : 0u;
    int count = 0;
    for (int tri = 0; tri < ntri; tri++) {
        float p[3][3];
        uint64_t k[3];
#pragma unroll
        for (int b = 0; b < 3; b++) edge_vertex(C, F, int((word >> (4 * (3 * tri + b))) & 0xf), p[b], k[b]);
        if (pmc && (same3(p[0], p[1]) || same3(p[0], p[2]) || same3(p[2], p[1]))) continue;
        count++;
        if (kEmit) {
#pragma unroll
            for (int b = 0; b < 3; b++) {
                const size_t r = size_t(f) * 3 + b;
                ref_key[r] = k[b];
                ref_val[r] = uint32_t(r);
                ref_pos[r] = make_float4(p[b][0], p[b][1], p[b][2], 0.0f);
            }
            f++;
        }
    }
    if (!kEmit) counts[t] = uint32_t(count);
}

template <bool kEmit>
__global__ void mc_kernel(const uint64_t* __restrict__ cell_keys, const uint32_t* __restrict__ corner,
                          const float* __restrict__ qp_dist, const uint32_t* __restrict__ valid, int nvalid, Frame F,
                          int pmc, uint32_t* __restrict__ counts, const uint32_t* __restrict__ offsets,
                          uint64_t* __restrict__ ref_key, uint32_t* __restrict__ ref_val, float4* __restrict__ ref_pos) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nvalid) return;
    McCell C;
    load_cell(cell_keys, corner, qp_dist, valid[t], F, C);
    mc_cell<kEmit>(C, F, pmc, uint32_t(t), counts, offsets, ref_key, ref_val, ref_pos);
}

// ---- marching cubes over TMA-staged distance slabs ------------------------
// When the box of grid vertices is small enough, their distances are
// scattered into a dense volume D[z][y][x] (x padded to a multiple of 4, so
// every row starts on a 16-byte boundary).  The valid cells of one 8x8x8
// brick are a contiguous run of the valid list (lattice keys are Morton
// codes, so key >> 9 names the brick); one CTA takes a run: a 3-D TMA tile
// copy (cp.async.bulk.tensor, box 12 x 9 x 9 floats: the 9 x 9 x 9 corners of
// the brick, the inner extent rounded up to a multiple of 16 bytes) brings its
// corner distances into shared memory, completion is signalled on an
// mbarrier, and every cell reads its eight corners from there instead of
// gathering them through the corner-id array.  The faces are those of
// mc_kernel, at the same places (counts and offsets by valid-list index).
constexpr int kSlabX = 12, kSlabY = 9, kSlabZ = 9;
constexpr uint32_t kSlabBytes = uint32_t(kSlabX * kSlabY * kSlabZ * sizeof(float));
// try_wait polls (each may suspend for a while in hardware) before the copy
// is reported as lost; a 3.9 KB tile copy needs a few microseconds.
constexpr int kTmaWaitIters = 1 << 20;

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return uint32_t(__cvta_generic_to_shared(p)); }

__device__ __forceinline__ bool mbar_wait_parity(uint32_t bar, uint32_t parity, int max_iters) {
    for (int it = 0; it < max_iters; it++) {
        uint32_t done;
        asm volatile(
            "{\n"
            " .reg .pred P;\n"
            " mbarrier.try_wait.parity.shared::cta.b64 P, [%1], %2;\n"
            " selp.u32 %0, 1, 0, P;\n"
            "}\n"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

template <bool kEmit>
__global__ void __launch_bounds__(128) mc_tma_kernel(const __grid_constant__ CUtensorMap tmap,
                                                     const uint64_t* __restrict__ cell_keys,
                                                     const uint32_t* __restrict__ valid,
                                                     const uint32_t* __restrict__ runs, Frame F, int pmc,
                                                     uint32_t* __restrict__ counts,
                                                     const uint32_t* __restrict__ offsets,
                                                     uint64_t* __restrict__ ref_key, uint32_t* __restrict__ ref_val,
                                                     float4* __restrict__ ref_pos, int* __restrict__ err) {
    __shared__ __align__(128) float slab[kSlabZ * kSlabY * kSlabX];
    __shared__ __align__(8) unsigned long long bar;
    const uint32_t t0 = runs[blockIdx.x], t1 = runs[blockIdx.x + 1];
    uint32_t bx, by, bz;
    lattice_decode(cell_keys[valid[t0]], bx, by, bz);
    bx &= ~7u;
    by &= ~7u;
    bz &= ~7u;
    const uint32_t sbar = smem_addr(&bar), sdst = smem_addr(slab);
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(sbar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(sbar), "r"(kSlabBytes)
                     : "memory");
        // x = bx is a multiple of 8 floats: the copy starts on a 32-byte boundary
        asm volatile(
            "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, "
            "%4}], [%5];" ::"r"(sdst),
            "l"(reinterpret_cast<uint64_t>(&tmap)), "r"(int(bx)), "r"(int(by)), "r"(int(bz)), "r"(sbar)
            : "memory");
    }
    if (!mbar_wait_parity(sbar, 0, kTmaWaitIters)) {
        if (threadIdx.x == 0) atomicOr(err, kErrTma);
        // one more bounded wait for the copy in flight before the block leaves
        mbar_wait_parity(sbar, 0, kTmaWaitIters);
        return;
    }
    for (uint32_t t = t0 + threadIdx.x; t < t1; t += blockDim.x) {
        McCell C;
        lattice_decode(cell_keys[valid[t]], C.rel[0], C.rel[1], C.rel[2]);
        C.L[0] = int(C.rel[0]) + F.bx;
        C.L[1] = int(C.rel[1]) + F.by;
        C.L[2] = int(C.rel[2]) + F.bz;
        const int lx = int(C.rel[0] - bx), ly = int(C.rel[1] - by), lz = int(C.rel[2] - bz);
        C.index = 0;
#pragma unroll
        for (int k = 0; k < 8; k++) {
            C.d[k] = slab[((lz + c_corner[k][2]) * kSlabY + (ly + c_corner[k][1])) * kSlabX + lx + c_corner[k][0]];
            if (C.d[k] > 0.0f) C.index |= 1 << k;
        }
        mc_cell<kEmit>(C, F, pmc, t, counts, offsets, ref_key, ref_val, ref_pos);
    }
}

// Distances of the grid vertices into the dense volume (x fastest).
__global__ void dense_volume_kernel(const uint64_t* __restrict__ qp_keys, const float* __restrict__ qp_dist, int n,
                                    int X, int Y, int Z, float* __restrict__ D, int* __restrict__ err) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t x, y, z;
    lattice_decode(qp_keys[i], x, y, z);
    if (x >= uint32_t(X) || y >= uint32_t(Y) || z >= uint32_t(Z)) {  // outside the planned box: not written
        atomicOr(err, kErrTma);
        return;
    }
    D[(size_t(z) * Y + y) * X + x] = qp_dist[i];
}

// Brick runs of the valid list: run r covers valid[runs[r], runs[r + 1]).
__global__ void brick_flags_kernel(const uint64_t* __restrict__ cell_keys, const uint32_t* __restrict__ valid, int n,
                                   uint32_t* __restrict__ flags) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    flags[t] = (t == 0 || (cell_keys[valid[t]] >> 9) != (cell_keys[valid[t - 1]] >> 9)) ? 1u : 0u;
}
__global__ void brick_runs_kernel(const uint32_t* __restrict__ flags, const uint32_t* __restrict__ pos, int n,
                                  uint32_t* __restrict__ runs) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t > n) return;
    if (t == n) runs[pos[n]] = uint32_t(n);
    else if (flags[t]) runs[pos[t]] = uint32_t(t);
}

using TensorMapEncodeTiled = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                          const cuuint64_t*, const cuuint32_t*, const cuuint32_t*,
                                          CUtensorMapInterleave, CUtensorMapSwizzle, CUtensorMapL2promotion,
                                          CUtensorMapFloatOOBfill);

// cuTensorMapEncodeTiled from the driver (null when it is not available, in
// which case marching cubes gathers its corners as before).
TensorMapEncodeTiled tensor_map_encoder() {
    static std::once_flag once;
    static TensorMapEncodeTiled fn = nullptr;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<TensorMapEncodeTiled>(p);
        cudaGetLastError();
    });
    return fn;
}

// The dense-slab plan of mc_stage: volume extents and the TMA descriptor.
struct SlabPlan {
    bool on = false;
    int X = 0, Y = 0, Z = 0;
    float* D = nullptr;
    uint32_t* runs = nullptr;
    int nruns = 0;
    CUtensorMap map;
};

__global__ void vertex_out_kernel(const uint32_t* __restrict__ first_ref, int nv, const float4* __restrict__ ref_pos,
                                  float* __restrict__ verts) {
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nv) return;
    float4 p = ref_pos[first_ref[v]];
    verts[3 * size_t(v)] = p.x;
    verts[3 * size_t(v) + 1] = p.y;
    verts[3 * size_t(v) + 2] = p.z;
}

template <typename Kernel>
void set_smem(Kernel k, size_t bytes) {
    if (bytes > 48 * 1024) LVRGB_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(bytes)));
}

uint64_t read_u64(Workspace& ws, const void* dptr, size_t bytes, cudaStream_t s) {
    uint64_t* h = ws.pinned();
    h[0] = 0;
    LVRGB_CUDA(cudaMemcpyAsync(h, dptr, bytes, cudaMemcpyDeviceToHost, s));
    LVRGB_CUDA(cudaStreamSynchronize(s));
    return h[0];
}

// Sorts keys in place (result pointer returned), removes duplicates and a
// trailing kNoKey; returns the unique count.
size_t sort_unique(Workspace& ws, const std::string& tag, uint64_t*& keys, size_t n, int bits, cudaStream_t s) {
    if (n == 0) return 0;
    uint64_t* alt = ws.get<uint64_t>(tag + ".alt", n);
    void* tmp = ws.get<unsigned char>("grid.sorttmp", radix_sort_temp_bytes<uint64_t>(n));
    if (radix_sort_pairs<uint64_t>(keys, nullptr, alt, nullptr, n, 0, bits, tmp, s)) std::swap(keys, alt);
    uint32_t* flags = ws.get<uint32_t>("grid.flags", n);
    uint32_t* pos = ws.get<uint32_t>("grid.pos", n + 1);
    head_flags_u64(keys, n, flags, s);
    void* stmp = ws.get<unsigned char>("grid.scantmp", scan_temp_bytes(n));
    exclusive_scan_u32(flags, pos, n, stmp, pos + n, s);
    scatter_flagged_u64(keys, flags, pos, n, alt, s);
    size_t u = size_t(uint32_t(read_u64(ws, pos + n, sizeof(uint32_t), s)));
    std::swap(keys, alt);
    if (u > 0 && read_u64(ws, keys + (u - 1), sizeof(uint64_t), s) == kNoKey) u--;
    return u;
}

// The dense form pays a scan over the whole key space; it replaces sorts of
// at least `nkeys` keys.
bool use_dense(int bits, size_t nkeys) {
    return bits <= 30 && (size_t(1) << bits) <= std::max<size_t>(size_t(1) << 24, 8 * nkeys);
}

// Scan of a dense flag map (N entries); returns the number of set flags and
// leaves the positions in pos (N + 1 entries).
size_t dense_scan(Workspace& ws, const uint32_t* flags, uint32_t* pos, size_t N, cudaStream_t s) {
    void* stmp = ws.get<unsigned char>("grid.densescan", scan_temp_bytes(N));
    exclusive_scan_u32(flags, pos, N, stmp, pos + N, s);
    return size_t(uint32_t(read_u64(ws, pos + N, sizeof(uint32_t), s)));
}

struct StageTimer {
    cudaEvent_t ev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    bool on = false;
    explicit StageTimer(bool enable) : on(enable) {
        if (on)
            for (auto& e : ev) LVRGB_CUDA(cudaEventCreate(&e));
    }
    void mark(int i, cudaStream_t s) {
        if (on) LVRGB_CUDA(cudaEventRecord(ev[i], s));
    }
    void finish(GridTimings* t, cudaStream_t s) {
        if (!on) return;
        LVRGB_CUDA(cudaStreamSynchronize(s));
        for (int i = 0; i < 4; i++) LVRGB_CUDA(cudaEventElapsedTime(&t->ms[i], ev[i], ev[i + 1]));
    }
    ~StageTimer() {
        for (auto& e : ev)
            if (e) cudaEventDestroy(e);
    }
};

}  // namespace

void signed_distance_rows(const Lbvh& T, const float4* normals, int kd, const float4* qs, int nq, float vs,
                          float* dist, float* eucl, uint8_t* invalid, Workspace& ws, int* d_err, cudaStream_t s,
                          unsigned long long* stats) {
    if (nq == 0) return;
    SdfArgs A;
    A.T = T;
    A.K = kd > 0 ? kd : 1;
    A.normals = normals;
    A.qs = qs;
    A.nq = nq;
    A.limit = 1.75 * double(vs);
    A.dist = dist;
    A.eucl = eucl;
    A.invalid = invalid;
    A.err = d_err;
    A.stats = stats;
    HeapPlan P = plan_heap(nq, A.K, ws);
    A.gheap = P.gheap;
    if (A.K == 5) {
        set_smem(sdf_kernel<LaneHeap5>, P.smem);
        A.tiles = persistent_tiles(sdf_kernel<LaneHeap5>, P, ws, s);
        sdf_kernel<LaneHeap5><<<P.blocks, kWarpsPerBlock * 32, P.smem, s>>>(A);
    } else if (A.K == 20) {
        set_smem(sdf_kernel<LaneHeap20>, P.smem);
        A.tiles = persistent_tiles(sdf_kernel<LaneHeap20>, P, ws, s);
        sdf_kernel<LaneHeap20><<<P.blocks, kWarpsPerBlock * 32, P.smem, s>>>(A);
    } else if (complete_3ary(A.K)) {
        set_smem(sdf_kernel<LaneHeap3>, P.smem);
        A.tiles = persistent_tiles(sdf_kernel<LaneHeap3>, P, ws, s);
        sdf_kernel<LaneHeap3><<<P.blocks, kWarpsPerBlock * 32, P.smem, s>>>(A);
    } else {
        set_smem(sdf_kernel<LaneHeap>, P.smem);
        A.tiles = persistent_tiles(sdf_kernel<LaneHeap>, P, ws, s);
        sdf_kernel<LaneHeap><<<P.blocks, kWarpsPerBlock * 32, P.smem, s>>>(A);
    }
    LVRGB_LAUNCH_CHECK();
}

namespace {
// Marching cubes over the valid cells of R (FastReconstruction::getMesh with
// FastBox / BilinearFastBox): count, scan, emit, deduplicate the vertices.
// The dense volume, the brick runs and the TMA descriptor of the slab path,
// when the box of grid vertices (ext: vertices per axis, relative to the
// base) holds at most 16 volume entries per vertex (plus 1M) and 2^28 in all,
// spans at least one slab in every direction, and the driver encodes
// tensor maps.  Otherwise on = false and marching cubes gathers its corners.
SlabPlan plan_slabs(const GridResult& R, const int ext[3], size_t nvalid, Workspace& ws, int* d_err, cudaStream_t s) {
    SlabPlan P;
    if (nvalid == 0 || R.nqp == 0) return P;
    const TensorMapEncodeTiled enc = tensor_map_encoder();
    if (!enc) return P;
    const size_t X = (size_t(std::max(ext[0], 1)) + 3) & ~size_t(3), Y = size_t(std::max(ext[1], 1)),
                 Z = size_t(std::max(ext[2], 1));
    const size_t vol = X * Y * Z;
    if (X < size_t(kSlabX) || Y < size_t(kSlabY) || Z < size_t(kSlabZ)) return P;
    if (vol > (size_t(1) << 28) || vol > 16 * size_t(R.nqp) + (size_t(1) << 20)) return P;
    float* D = ws.get<float>("mc.dense", vol);
    cuuint64_t dims[3] = {cuuint64_t(X), cuuint64_t(Y), cuuint64_t(Z)};
    cuuint64_t strides[2] = {cuuint64_t(X * sizeof(float)), cuuint64_t(X * Y * sizeof(float))};
    cuuint32_t box[3] = {cuuint32_t(kSlabX), cuuint32_t(kSlabY), cuuint32_t(kSlabZ)};
    cuuint32_t elem[3] = {1, 1, 1};
    if (enc(&P.map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, D, dims, strides, box, elem, CU_TENSOR_MAP_INTERLEAVE_NONE,
            CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) !=
        CUDA_SUCCESS)
        return SlabPlan();
    // entries that are no grid vertex keep whatever the buffer held: they are
    // never read, since the eight corners of a valid cell are grid vertices
    dense_volume_kernel<<<ceil_div(size_t(R.nqp), 256), 256, 0, s>>>(R.qp_keys, R.qp_dist, int(R.nqp), int(X),
                                                                      int(Y), int(Z), D, d_err);
    LVRGB_LAUNCH_CHECK();
    uint32_t* flags = ws.get<uint32_t>("mc.bflags", nvalid);
    uint32_t* pos = ws.get<uint32_t>("mc.bpos", nvalid + 1);
    brick_flags_kernel<<<ceil_div(nvalid, 256), 256, 0, s>>>(R.cell_keys, R.valid_cells, int(nvalid), flags);
    LVRGB_LAUNCH_CHECK();
    void* stmp = ws.get<unsigned char>("grid.scantmp", scan_temp_bytes(nvalid));
    exclusive_scan_u32(flags, pos, nvalid, stmp, pos + nvalid, s);
    P.nruns = int(uint32_t(read_u64(ws, pos + nvalid, sizeof(uint32_t), s)));
    P.runs = ws.get<uint32_t>("mc.runs", size_t(P.nruns) + 1);
    brick_runs_kernel<<<ceil_div(nvalid + 1, 256), 256, 0, s>>>(flags, pos, int(nvalid), P.runs);
    LVRGB_LAUNCH_CHECK();
    P.X = int(X);
    P.Y = int(Y);
    P.Z = int(Z);
    P.D = D;
    P.on = true;
    return P;
}

void mc_stage(GridResult& R, const Frame& F, int kbits, const int ext[3], int decomposition, Workspace& ws,
              int* d_err, cudaStream_t s) {
    const uint64_t* ck = R.cell_keys;
    const uint32_t* cell_corner = R.cell_corner;
    const uint32_t* valid = R.valid_cells;
    const size_t nvalid = size_t(R.ncells_valid);
    GridConfig cfg;
    cfg.decomposition = decomposition;
    size_t nf = 0;
    uint32_t* fcount = ws.get<uint32_t>("mc.count", nvalid);
    uint32_t* foff = ws.get<uint32_t>("mc.off", nvalid + 1);
    const SlabPlan slabs = plan_slabs(R, ext, nvalid, ws, d_err, s);
    // count (kEmit false) or emit the faces of every valid cell
    auto mc_pass = [&](bool emit, uint64_t* rk, uint32_t* rv, float4* rp) {
        if (slabs.on) {
            if (emit)
                mc_tma_kernel<true><<<slabs.nruns, 128, 0, s>>>(slabs.map, ck, valid, slabs.runs, F,
                                                                 cfg.decomposition == 1, nullptr, foff, rk, rv, rp,
                                                                 d_err);
            else
                mc_tma_kernel<false><<<slabs.nruns, 128, 0, s>>>(slabs.map, ck, valid, slabs.runs, F,
                                                                  cfg.decomposition == 1, fcount, nullptr, nullptr,
                                                                  nullptr, nullptr, d_err);
        } else if (emit) {
            mc_kernel<true><<<ceil_div(nvalid, 128), 128, 0, s>>>(ck, cell_corner, R.qp_dist, valid, int(nvalid), F,
                                                                  cfg.decomposition == 1, nullptr, foff, rk, rv, rp);
        } else {
            mc_kernel<false><<<ceil_div(nvalid, 128), 128, 0, s>>>(ck, cell_corner, R.qp_dist, valid, int(nvalid),
                                                                   F, cfg.decomposition == 1, fcount, nullptr,
                                                                   nullptr, nullptr, nullptr);
        }
        LVRGB_LAUNCH_CHECK();
    };
    if (nvalid) {
        mc_pass(false, nullptr, nullptr, nullptr);
        void* stmp = ws.get<unsigned char>("grid.scantmp", scan_temp_bytes(nvalid));
        exclusive_scan_u32(fcount, foff, nvalid, stmp, foff + nvalid, s);
        nf = size_t(uint32_t(read_u64(ws, foff + nvalid, sizeof(uint32_t), s)));
    }
    const size_t nref = nf * 3;
    uint64_t* rk = ws.get<uint64_t>("mc.rk", nref);
    uint32_t* rv = ws.get<uint32_t>("mc.rv", nref);
    float4* rp = ws.get<float4>("mc.rp", nref);
    uint32_t* faces = ws.get<uint32_t>("mc.faces", nref);
    uint64_t* vkeys = ws.get<uint64_t>("mc.vkeys", nref);
    size_t nv = 0;
    const bool dense_edges = use_dense(kbits + 2, nref);
    float* verts = nullptr;
    if (nf && dense_edges) {
        mc_pass(true, rk, rv, rp);
        const size_t NE = size_t(1) << (kbits + 2);
        uint32_t* eflags = ws.get<uint32_t>("mc.dflags", NE);
        uint32_t* epos = ws.get<uint32_t>("mc.dpos", NE + 1);
        LVRGB_CUDA(cudaMemsetAsync(eflags, 0, NE * sizeof(uint32_t), s));
        mark_refs_kernel<<<ceil_div(nref, 256), 256, 0, s>>>(rk, nref, eflags);
        LVRGB_LAUNCH_CHECK();
        nv = dense_scan(ws, eflags, epos, NE, s);
        dense_compact_kernel<<<ceil_div(NE, 256), 256, 0, s>>>(eflags, epos, NE, vkeys);
        LVRGB_LAUNCH_CHECK();
        verts = ws.get<float>("mc.verts", nv * 3);
        dense_refs_kernel<<<ceil_div(nref, 256), 256, 0, s>>>(rk, rp, nref, epos, faces, verts);
        LVRGB_LAUNCH_CHECK();
    } else if (nf) {
        uint64_t* rk2 = ws.get<uint64_t>("mc.rk2", nref);
        uint32_t* rv2 = ws.get<uint32_t>("mc.rv2", nref);
        uint32_t* first = ws.get<uint32_t>("mc.first", nref);
        mc_pass(true, rk, rv, rp);
        void* tmp = ws.get<unsigned char>("grid.sorttmp", radix_sort_temp_bytes<uint64_t>(nref));
        if (radix_sort_pairs<uint64_t>(rk, rv, rk2, rv2, nref, 0, kbits + 2, tmp, s)) {
            std::swap(rk, rk2);
            std::swap(rv, rv2);
        }
        uint32_t* flags = ws.get<uint32_t>("grid.flags", nref);
        uint32_t* pos = ws.get<uint32_t>("grid.pos", nref + 1);
        head_flags_u64(rk, nref, flags, s);
        void* stmp = ws.get<unsigned char>("grid.scantmp", scan_temp_bytes(nref));
        exclusive_scan_u32(flags, pos, nref, stmp, pos + nref, s);
        assign_ids_kernel<<<ceil_div(nref, 256), 256, 0, s>>>(rk, rv, flags, pos, int(nref), faces, vkeys, first);
        LVRGB_LAUNCH_CHECK();
        nv = size_t(uint32_t(read_u64(ws, pos + nref, sizeof(uint32_t), s)));
        verts = ws.get<float>("mc.verts", nv * 3);
        if (nv) {
            vertex_out_kernel<<<ceil_div(nv, 256), 256, 0, s>>>(first, int(nv), rp, verts);
            LVRGB_LAUNCH_CHECK();
        }
    }
    if (!verts) verts = ws.get<float>("mc.verts", 1);
    R.nfaces = (long long)nf;
    R.nverts = (long long)nv;
    R.faces = faces;
    R.face_cell_off = foff;
    R.vert_keys = vkeys;
    R.verts = verts;
}

}  // namespace

void grid_reconstruct(const Lbvh& T, const float4* normals, const float bb[6], const GridConfig& cfg, Workspace& ws,
                      GridResult& R, int* d_err, cudaStream_t s, GridTimings* timings) {
    StageTimer timer(timings != nullptr);
    timer.mark(0, s);
    std::optional<NvtxRange> stage;
    stage.emplace("lvrgb.grid_build");
    R = GridResult();
    // HashGrid ctor (HashGrid.tcc:48-52)
    const float longest = std::max({bb[3] - bb[0], bb[4] - bb[1], bb[5] - bb[2]});
    const float vs = cfg.is_voxelsize ? cfg.resolution : longest / cfg.resolution;
    if (!(vs > 0.0f) || !std::isfinite(vs)) throw std::invalid_argument("voxel size must be positive");
    R.vs = vs;
    Frame F;
    F.vs = vs;
    int top[3];
    for (int a = 0; a < 3; a++) {
        F.lo[a] = bb[a];
        F.hi[a] = bb[3 + a];
        const double lo = std::floor(double(bb[a] / vs));
        const double hi = std::floor(double(bb[3 + a] / vs));
        if (std::fabs(lo) > 1e9 || std::fabs(hi) > 1e9) throw std::invalid_argument("grid index out of range");
        R.base[a] = int(lo) - 2;
        top[a] = int(hi) - R.base[a] + 3;
    }
    F.bx = R.base[0]; F.by = R.base[1]; F.bz = R.base[2];
    int nbits = 1;
    while ((1 << nbits) <= std::max({top[0], top[1], top[2]}) + 1) nbits++;
    if (nbits > 20) throw std::invalid_argument("grid extent exceeds 2^20 cells per axis");
    R.nbits = nbits;
    const int kbits = 3 * nbits;
    const int n = T.n;

    // ---- cells of the points, then extrusion (PointsetGrid.tcc:61-106) ----
    const bool dense = use_dense(kbits, size_t(n));
    const size_t NK = dense ? size_t(1) << kbits : 0;
    uint32_t* dflags = dense ? ws.get<uint32_t>("grid.dflags", NK) : nullptr;
    uint32_t* dpos = dense ? ws.get<uint32_t>("grid.dpos", NK + 1) : nullptr;
    uint64_t* ck;
    size_t nc;
    if (dense) {
        LVRGB_CUDA(cudaMemsetAsync(dflags, 0, NK * sizeof(uint32_t), s));
        mark_point_cells_kernel<<<ceil_div(n, 256), 256, 0, s>>>(T.pts, n, F, dflags);
        LVRGB_LAUNCH_CHECK();
        nc = dense_scan(ws, dflags, dpos, NK, s);
        ck = ws.get<uint64_t>("grid.cellsA", std::max<size_t>(nc, 1));
        dense_compact_kernel<<<ceil_div(NK, 256), 256, 0, s>>>(dflags, dpos, NK, ck);
        LVRGB_LAUNCH_CHECK();
        if (cfg.extrude && nc > 0) {
            // the point cells stay marked; their neighbours join them
            mark_extrude_kernel<<<ceil_div(nc * 27, 256), 256, 0, s>>>(ck, int(nc), F, dflags);
            LVRGB_LAUNCH_CHECK();
            nc = dense_scan(ws, dflags, dpos, NK, s);
            ck = ws.get<uint64_t>("grid.cellsB", std::max<size_t>(nc, 1));
            dense_compact_kernel<<<ceil_div(NK, 256), 256, 0, s>>>(dflags, dpos, NK, ck);
            LVRGB_LAUNCH_CHECK();
        }
    } else {
        ck = ws.get<uint64_t>("grid.cellsA", size_t(n));
        point_cells_kernel<<<ceil_div(n, 256), 256, 0, s>>>(T.pts, n, F, ck);
        LVRGB_LAUNCH_CHECK();
        nc = sort_unique(ws, "grid.cellsA", ck, size_t(n), kbits, s);
        if (cfg.extrude && nc > 0) {
            uint64_t* ek = ws.get<uint64_t>("grid.cellsB", nc * 27);
            extrude_kernel<<<ceil_div(nc * 27, 256), 256, 0, s>>>(ck, int(nc), F, ek);
            LVRGB_LAUNCH_CHECK();
            nc = sort_unique(ws, "grid.cellsB", ek, nc * 27, kbits, s);
            ck = ek;
        }
    }
    R.ncells_all = (long long)nc;
    R.cell_keys = ck;

    // ---- grid vertices: the 8 corners of every cell, deduplicated --------
    const size_t ncorner = nc * 8;
    uint32_t* cell_corner = ws.get<uint32_t>("grid.cell_corner", ncorner);
    uint64_t* qk = ws.get<uint64_t>("grid.qp_keys", ncorner);
    size_t nqp = 0;
    if (nc > 0 && dense) {
        LVRGB_CUDA(cudaMemsetAsync(dflags, 0, NK * sizeof(uint32_t), s));
        mark_corners_kernel<<<ceil_div(ncorner, 256), 256, 0, s>>>(ck, int(nc), dflags);
        LVRGB_LAUNCH_CHECK();
        nqp = dense_scan(ws, dflags, dpos, NK, s);
        dense_compact_kernel<<<ceil_div(NK, 256), 256, 0, s>>>(dflags, dpos, NK, qk);
        LVRGB_LAUNCH_CHECK();
        corner_ids_kernel<<<ceil_div(ncorner, 256), 256, 0, s>>>(ck, int(nc), dpos, cell_corner);
        LVRGB_LAUNCH_CHECK();
    } else if (nc > 0) {
        uint64_t* pk = ws.get<uint64_t>("grid.cornerk", ncorner);
        uint32_t* pv = ws.get<uint32_t>("grid.cornerv", ncorner);
        uint64_t* pk2 = ws.get<uint64_t>("grid.cornerk2", ncorner);
        uint32_t* pv2 = ws.get<uint32_t>("grid.cornerv2", ncorner);
        corner_pairs_kernel<<<ceil_div(ncorner, 256), 256, 0, s>>>(ck, int(nc), pk, pv);
        LVRGB_LAUNCH_CHECK();
        void* tmp = ws.get<unsigned char>("grid.sorttmp", radix_sort_temp_bytes<uint64_t>(ncorner));
        if (radix_sort_pairs<uint64_t>(pk, pv, pk2, pv2, ncorner, 0, kbits, tmp, s)) {
            std::swap(pk, pk2);
            std::swap(pv, pv2);
        }
        uint32_t* flags = ws.get<uint32_t>("grid.flags", ncorner);
        uint32_t* pos = ws.get<uint32_t>("grid.pos", ncorner + 1);
        head_flags_u64(pk, ncorner, flags, s);
        void* stmp = ws.get<unsigned char>("grid.scantmp", scan_temp_bytes(ncorner));
        exclusive_scan_u32(flags, pos, ncorner, stmp, pos + ncorner, s);
        assign_ids_kernel<<<ceil_div(ncorner, 256), 256, 0, s>>>(pk, pv, flags, pos, int(ncorner), cell_corner, qk,
                                                                   nullptr);
        LVRGB_LAUNCH_CHECK();
        nqp = size_t(uint32_t(read_u64(ws, pos + ncorner, sizeof(uint32_t), s)));
    }
    R.nqp = (long long)nqp;
    R.qp_keys = qk;
    R.cell_corner = cell_corner;
    float4* qpos = ws.get<float4>("grid.qp_pos", nqp);
    R.qp_pos = qpos;
    if (nqp) {
        qp_pos_kernel<<<ceil_div(nqp, 256), 256, 0, s>>>(qk, int(nqp), F, qpos);
        LVRGB_LAUNCH_CHECK();
    }
    timer.mark(1, s);
    stage.emplace("lvrgb.signed_distance");

    // ---- signed distance at every grid vertex (calcDistanceValues) -------
    R.qp_dist = ws.get<float>("grid.qp_dist", nqp);
    R.qp_eucl = ws.get<float>("grid.qp_eucl", nqp);
    R.qp_invalid = ws.get<uint8_t>("grid.qp_invalid", nqp);
    signed_distance_rows(T, normals, cfg.kd, qpos, int(nqp), vs, R.qp_dist, R.qp_eucl, R.qp_invalid, ws, d_err, s,
                         cfg.sdf_stats);
    timer.mark(2, s);
    stage.emplace("lvrgb.culling");

    // ---- remove cells with an invalid corner (PointsetGrid.tcc:153-184) --
    uint32_t* vflags = ws.get<uint32_t>("grid.vflags", nc);
    uint32_t* vpos = ws.get<uint32_t>("grid.vpos", nc + 1);
    uint32_t* valid = ws.get<uint32_t>("grid.valid", nc);
    size_t nvalid = 0;
    if (nc) {
        cell_valid_kernel<<<ceil_div(nc, 256), 256, 0, s>>>(cell_corner, int(nc), R.qp_invalid, vflags);
        LVRGB_LAUNCH_CHECK();
        uint32_t* ids = ws.get<uint32_t>("grid.ids", nc);
        iota_u32(ids, nc, s);
        void* stmp = ws.get<unsigned char>("grid.scantmp", scan_temp_bytes(nc));
        exclusive_scan_u32(vflags, vpos, nc, stmp, vpos + nc, s);
        scatter_flagged_u32(ids, vflags, vpos, nc, valid, s);
        nvalid = size_t(uint32_t(read_u64(ws, vpos + nc, sizeof(uint32_t), s)));
    }
    R.ncells_valid = (long long)nvalid;
    R.valid_cells = valid;
    timer.mark(3, s);
    stage.emplace("lvrgb.marching_cubes");

    const int ext[3] = {top[0] + 1, top[1] + 1, top[2] + 1};
    mc_stage(R, F, kbits, ext, cfg.decomposition, ws, d_err, s);
    timer.mark(4, s);
    stage.reset();
    timer.finish(timings, s);
}

namespace {

// Merged grid of stored chunk cells (HashGrid(chunks, innerBoxes, bb, voxelsize),
// HashGrid.tcc:136-193).
__global__ void merge_index_kernel(const float* __restrict__ centers, int n, const int64_t* __restrict__ off,
                                   int nchunks, const float* __restrict__ boxes, float vs, int4* __restrict__ idx,
                                   uint32_t* __restrict__ keep, int* __restrict__ range) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float x = centers[3 * size_t(i)], y = centers[3 * size_t(i) + 1], z = centers[3 * size_t(i) + 2];
    bool ok = true;
    if (boxes) {
        int lo = 0, hi = nchunks - 1;  // chunk c holds cells [off[c], off[c + 1])
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (off[mid] <= i) lo = mid; else hi = mid - 1;
        }
        const float* b = boxes + 6 * size_t(lo);
        // BoundingBox::contains (BoundingBox.tcc:166-171)
        ok = (b[0] <= x && b[3] >= x) && (b[1] <= y && b[4] >= y) && (b[2] <= z && b[5] >= z);
    }
    // HashGrid::calcIndex (HashGrid.hpp:263-268)
    const float fx = floorf(__fdiv_rn(x, vs)), fy = floorf(__fdiv_rn(y, vs)), fz = floorf(__fdiv_rn(z, vs));
    ok = ok && fabsf(fx) < 1e9f && fabsf(fy) < 1e9f && fabsf(fz) < 1e9f;  // NaN fails too
    keep[i] = ok ? 1u : 0u;
    if (!ok) return;
    const int ix = int(fx), iy = int(fy), iz = int(fz);
    idx[i] = make_int4(ix, iy, iz, 0);
    atomicMin(range + 0, ix); atomicMin(range + 1, iy); atomicMin(range + 2, iz);
    atomicMax(range + 3, ix); atomicMax(range + 4, iy); atomicMax(range + 5, iz);
}

__global__ void merge_keys_kernel(const int4* __restrict__ idx, const uint32_t* __restrict__ keep,
                                  const uint32_t* __restrict__ pos, int n, int bx, int by, int bz,
                                  uint64_t* __restrict__ keys, uint32_t* __restrict__ rank) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || !keep[i]) return;
    const int4 c = idx[i];
    keys[pos[i]] = lattice_key(uint32_t(c.x - bx), uint32_t(c.y - by), uint32_t(c.z - bz));
    rank[pos[i]] = uint32_t(i);
}

// Unique cells (the first of each run of equal keys: the earliest input cell).
__global__ void merge_unique_kernel(const uint64_t* __restrict__ keys, const uint32_t* __restrict__ rank,
                                    const uint32_t* __restrict__ flags, const uint32_t* __restrict__ pos, int n,
                                    uint64_t* __restrict__ ukeys, uint32_t* __restrict__ urank) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || !flags[i]) return;
    ukeys[pos[i]] = keys[i];
    urank[pos[i]] = rank[i];
}

// Corner slots j * 8 + k, generated cell by cell in input order so that a
// stable sort by corner key puts the earliest cell's slot first.
__global__ void merge_corner_kernel(const uint64_t* __restrict__ ukeys, const uint32_t* __restrict__ order, int nc,
                                    uint64_t* __restrict__ keys, uint32_t* __restrict__ vals) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nc * 8) return;
    const uint32_t j = order[t >> 3];
    const int k = t & 7;
    uint32_t x, y, z;
    lattice_decode(ukeys[j], x, y, z);
    keys[t] = lattice_key(x + c_corner[k][0], y + c_corner[k][1], z + c_corner[k][2]);
    vals[t] = j * 8u + uint32_t(k);
}

// A grid vertex takes the distance the earliest cell holding it gave
// (HashGrid::addBox keeps a shared corner found by findQueryPoint).
__global__ void merge_dist_kernel(const uint32_t* __restrict__ first, int nqp, const uint32_t* __restrict__ urank,
                                  const float* __restrict__ tsdf, float* __restrict__ dist) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nqp) return;
    const uint32_t slot = first[q];
    dist[q] = tsdf[size_t(urank[slot >> 3]) * 8 + (slot & 7u)];
}

}  // namespace

void grid_from_cells(const float* centers, const float* tsdf, int n, const int64_t* chunk_off, int nchunks,
                     const float* boxes, float vs, int decomposition, Workspace& ws, GridResult& R, int* d_err,
                     cudaStream_t s) {
    (void)d_err;
    R = GridResult();
    if (!(vs > 0.0f) || !std::isfinite(vs)) throw std::invalid_argument("voxel size must be positive");
    R.vs = vs;
    Frame F;
    F.vs = vs;
    for (int a = 0; a < 3; a++) {
        F.lo[a] = -INFINITY;
        F.hi[a] = INFINITY;
    }
    int4* idx = ws.get<int4>("merge.idx", size_t(std::max(n, 1)));
    uint32_t* keep = ws.get<uint32_t>("merge.keep", size_t(std::max(n, 1)));
    uint32_t* kpos = ws.get<uint32_t>("merge.kpos", size_t(n) + 1);
    int* range = ws.get<int>("merge.range", 6);
    const int init[6] = {INT_MAX, INT_MAX, INT_MAX, INT_MIN, INT_MIN, INT_MIN};
    LVRGB_CUDA(cudaMemcpyAsync(range, init, sizeof(init), cudaMemcpyHostToDevice, s));
    size_t nk = 0;
    if (n > 0) {
        merge_index_kernel<<<ceil_div(n, 256), 256, 0, s>>>(centers, n, chunk_off, nchunks, boxes, vs, idx, keep, range);
        LVRGB_LAUNCH_CHECK();
        void* stmp = ws.get<unsigned char>("grid.scantmp", scan_temp_bytes(size_t(n)));
        exclusive_scan_u32(keep, kpos, size_t(n), stmp, kpos + n, s);
        nk = size_t(uint32_t(read_u64(ws, kpos + n, sizeof(uint32_t), s)));
    }
    int rng[6] = {0, 0, 0, 0, 0, 0};
    if (nk) {
        LVRGB_CUDA(cudaMemcpyAsync(rng, range, sizeof(rng), cudaMemcpyDeviceToHost, s));
        LVRGB_CUDA(cudaStreamSynchronize(s));
    }
    int top = 1;
    for (int a = 0; a < 3; a++) {
        R.base[a] = rng[a] - 1;
        top = std::max(top, rng[3 + a] - R.base[a] + 2);
    }
    F.bx = R.base[0]; F.by = R.base[1]; F.bz = R.base[2];
    int nbits = 1;
    while ((1 << nbits) <= top + 1) nbits++;
    if (nbits > 20) throw std::invalid_argument("grid extent exceeds 2^20 cells per axis");
    R.nbits = nbits;
    const int kbits = 3 * nbits;

    // kept cells (key, input index), sorted by key; the first of equal keys wins
    uint64_t* ck = ws.get<uint64_t>("merge.keys", std::max<size_t>(nk, 1));
    uint32_t* cr = ws.get<uint32_t>("merge.rank", std::max<size_t>(nk, 1));
    size_t nc = 0;
    uint64_t* uck = ws.get<uint64_t>("grid.cellsA", std::max<size_t>(nk, 1));
    uint32_t* urank = ws.get<uint32_t>("merge.urank", std::max<size_t>(nk, 1));
    if (nk) {
        merge_keys_kernel<<<ceil_div(n, 256), 256, 0, s>>>(idx, keep, kpos, n, R.base[0], R.base[1], R.base[2], ck, cr);
        LVRGB_LAUNCH_CHECK();
        uint64_t* ck2 = ws.get<uint64_t>("merge.keys2", nk);
        uint32_t* cr2 = ws.get<uint32_t>("merge.rank2", nk);
        void* tmp = ws.get<unsigned char>("grid.sorttmp", radix_sort_temp_bytes<uint64_t>(nk));
        if (radix_sort_pairs<uint64_t>(ck, cr, ck2, cr2, nk, 0, kbits, tmp, s)) {
            std::swap(ck, ck2);
            std::swap(cr, cr2);
        }
        uint32_t* flags = ws.get<uint32_t>("grid.flags", nk);
        uint32_t* pos = ws.get<uint32_t>("grid.pos", nk + 1);
        head_flags_u64(ck, nk, flags, s);
        void* stmp = ws.get<unsigned char>("grid.scantmp", scan_temp_bytes(nk));
        exclusive_scan_u32(flags, pos, nk, stmp, pos + nk, s);
        merge_unique_kernel<<<ceil_div(nk, 256), 256, 0, s>>>(ck, cr, flags, pos, int(nk), uck, urank);
        LVRGB_LAUNCH_CHECK();
        nc = size_t(uint32_t(read_u64(ws, pos + nk, sizeof(uint32_t), s)));
    }
    R.ncells_all = (long long)nc;
    R.cell_keys = uck;

    // grid vertices: corners of the cells, taken in input order of the cells
    const size_t ncorner = nc * 8;
    uint32_t* cell_corner = ws.get<uint32_t>("grid.cell_corner", std::max<size_t>(ncorner, 1));
    uint64_t* qk = ws.get<uint64_t>("grid.qp_keys", std::max<size_t>(ncorner, 1));
    size_t nqp = 0;
    uint32_t* first = ws.get<uint32_t>("merge.first", std::max<size_t>(ncorner, 1));
    if (nc) {
        // cells in input order
        uint32_t* rk = ws.get<uint32_t>("merge.rk", nc);
        uint32_t* rk2 = ws.get<uint32_t>("merge.rk2", nc);
        uint32_t* ord = ws.get<uint32_t>("merge.ord", nc);
        uint32_t* ord2 = ws.get<uint32_t>("merge.ord2", nc);
        LVRGB_CUDA(cudaMemcpyAsync(rk, urank, nc * sizeof(uint32_t), cudaMemcpyDeviceToDevice, s));
        iota_u32(ord, nc, s);
        void* tmp = ws.get<unsigned char>("grid.sorttmp", radix_sort_temp_bytes<uint32_t>(nc));
        if (radix_sort_pairs<uint32_t>(rk, ord, rk2, ord2, nc, 0, 32, tmp, s)) std::swap(ord, ord2);
        uint64_t* pk = ws.get<uint64_t>("grid.cornerk", ncorner);
        uint32_t* pv = ws.get<uint32_t>("grid.cornerv", ncorner);
        uint64_t* pk2 = ws.get<uint64_t>("grid.cornerk2", ncorner);
        uint32_t* pv2 = ws.get<uint32_t>("grid.cornerv2", ncorner);
        merge_corner_kernel<<<ceil_div(ncorner, 256), 256, 0, s>>>(uck, ord, int(nc), pk, pv);
        LVRGB_LAUNCH_CHECK();
        void* tmp2 = ws.get<unsigned char>("grid.sorttmp", radix_sort_temp_bytes<uint64_t>(ncorner));
        if (radix_sort_pairs<uint64_t>(pk, pv, pk2, pv2, ncorner, 0, kbits, tmp2, s)) {
            std::swap(pk, pk2);
            std::swap(pv, pv2);
        }
        uint32_t* flags = ws.get<uint32_t>("grid.flags", ncorner);
        uint32_t* pos = ws.get<uint32_t>("grid.pos", ncorner + 1);
        head_flags_u64(pk, ncorner, flags, s);
        void* stmp = ws.get<unsigned char>("grid.scantmp", scan_temp_bytes(ncorner));
        exclusive_scan_u32(flags, pos, ncorner, stmp, pos + ncorner, s);
        assign_ids_kernel<<<ceil_div(ncorner, 256), 256, 0, s>>>(pk, pv, flags, pos, int(ncorner), cell_corner, qk,
                                                                   first);
        LVRGB_LAUNCH_CHECK();
        nqp = size_t(uint32_t(read_u64(ws, pos + ncorner, sizeof(uint32_t), s)));
    }
    R.nqp = (long long)nqp;
    R.qp_keys = qk;
    R.cell_corner = cell_corner;
    float4* qpos = ws.get<float4>("grid.qp_pos", std::max<size_t>(nqp, 1));
    R.qp_pos = qpos;
    R.qp_dist = ws.get<float>("grid.qp_dist", std::max<size_t>(nqp, 1));
    R.qp_eucl = ws.get<float>("grid.qp_eucl", std::max<size_t>(nqp, 1));
    R.qp_invalid = ws.get<uint8_t>("grid.qp_invalid", std::max<size_t>(nqp, 1));
    if (nqp) {
        qp_pos_kernel<<<ceil_div(nqp, 256), 256, 0, s>>>(qk, int(nqp), F, qpos);
        LVRGB_LAUNCH_CHECK();
        merge_dist_kernel<<<ceil_div(nqp, 256), 256, 0, s>>>(first, int(nqp), urank, tsdf, R.qp_dist);
        LVRGB_LAUNCH_CHECK();
        LVRGB_CUDA(cudaMemsetAsync(R.qp_eucl, 0, nqp * sizeof(float), s));
        LVRGB_CUDA(cudaMemsetAsync(R.qp_invalid, 0, nqp, s));
    }
    // every merged cell is valid (the chunks were culled when they were made)
    uint32_t* valid = ws.get<uint32_t>("grid.valid", std::max<size_t>(nc, 1));
    if (nc) iota_u32(valid, nc, s);
    R.ncells_valid = (long long)nc;
    R.valid_cells = valid;
    const int ext[3] = {rng[3] - R.base[0] + 3, rng[4] - R.base[1] + 3, rng[5] - R.base[2] + 3};
    mc_stage(R, F, kbits, ext, decomposition, ws, d_err, s);
}

namespace {
__global__ void cell_tsdf_kernel(const uint64_t* __restrict__ keys, const uint32_t* __restrict__ valid, int n,
                                 int bx, int by, int bz, float vs, const uint32_t* __restrict__ corner,
                                 const float* __restrict__ dist, float* __restrict__ centers,
                                 float* __restrict__ tsdf) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t c = valid[i];
    uint32_t x, y, z;
    lattice_decode(keys[c], x, y, z);
    if (centers) {
        centers[3 * size_t(i)] = cell_center(int(x) + bx, vs);
        centers[3 * size_t(i) + 1] = cell_center(int(y) + by, vs);
        centers[3 * size_t(i) + 2] = cell_center(int(z) + bz, vs);
    }
    if (tsdf) {
#pragma unroll
        for (int k = 0; k < 8; k++) tsdf[8 * size_t(i) + k] = dist[corner[8 * size_t(c) + k]];
    }
}
}  // namespace

void cell_tsdf(const GridResult& R, float* centers, float* tsdf, cudaStream_t s) {
    const int n = int(R.ncells_valid);
    if (n == 0) return;
    cell_tsdf_kernel<<<ceil_div(n, 256), 256, 0, s>>>(R.cell_keys, R.valid_cells, n, R.base[0], R.base[1],
                                                      R.base[2], R.vs, R.cell_corner, R.qp_dist, centers, tsdf);
    LVRGB_LAUNCH_CHECK();
}

}  // namespace lvrgb
