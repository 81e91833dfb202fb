// api.cu -- the C ABI (include/lvrgb.h): handle, input staging, call
// sequencing and error translation.  No exception crosses this file's
// extern "C" functions.
#include <algorithm>
#include <atomic>
#include <climits>
#include <cmath>
#include <cstring>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "lvrgb.h"
#include "batch.h"
#include "chunks.h"
#include "adjoint.h"
#include "grid.h"
#include "meshops.h"
#include "nvtx.h"
#include "planar.h"
#include "lbvh_build.h"
#include "primitives.cuh"
#include "surface.h"

using namespace lvrgb;

struct lvrgb_surface_s {
    lvrgb_surface_config cfg;
    int device = 0;
    Workspace ws;
    Lbvh T;
    float bb[9] = {0};
    float* d_box = nullptr;
    int* d_err = nullptr;
    uint32_t* d_stats = nullptr;
    unsigned long long* d_sdf_stats = nullptr;  // signed-distance search counters of the last reconstruct
    float4* normals = nullptr;      // final normals, Morton order
    float4* raw_normals = nullptr;  // before interpolation
    int32_t* kused = nullptr;
    std::vector<float> poses;  // scan poses (x y z each), empty: none
    bool has_normals = false;
    bool has_raw = false;
    GridResult grid;
    bool has_grid = false;
    // device-time events: LBVH build, normal estimation, interpolation, PMC
    // planar post-pass
    cudaEvent_t ev[8] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    bool ev_used[4] = {false, false, false, false};
    float grid_ms[4] = {0, 0, 0, 0};
    cudaEvent_t copy_ev = nullptr;  // orders lvrgb_get_normals_async's copy stream
    ~lvrgb_surface_s() {
        for (auto& e : ev)
            if (e) cudaEventDestroy(e);
        if (copy_ev) cudaEventDestroy(copy_ev);
    }
};

namespace lvrgb {
static std::atomic<unsigned long long> g_launches{0};
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
}  // namespace lvrgb

namespace {

thread_local std::string g_last_error;

struct ApiError {
    lvrgb_status st;
    std::string msg;
};

lvrgb_status fail(lvrgb_status st, const std::string& msg) {
    g_last_error = msg;
    return st;
}

template <typename F>
lvrgb_status guarded(F&& f) {
    try {
        f();
        return LVRGB_OK;
    } catch (const ApiError& e) {
        return fail(e.st, e.msg);
    } catch (const CudaError& e) {
        std::string m = std::string(cudaGetErrorString(e.err)) + " at " + e.file + ":" + std::to_string(e.line);
        cudaGetLastError();  // clear a sticky launch error where possible
        if (e.err == cudaErrorMemoryAllocation) return fail(LVRGB_ERR_OUT_OF_MEMORY, m);
        return fail(LVRGB_ERR_CUDA, m);
    } catch (const std::invalid_argument& e) {
        return fail(LVRGB_ERR_INVALID_ARGUMENT, e.what());
    } catch (const std::bad_alloc&) {
        return fail(LVRGB_ERR_OUT_OF_MEMORY, "host allocation failed");
    } catch (const std::exception& e) {
        return fail(LVRGB_ERR_CUDA, e.what());
    } catch (...) {
        return fail(LVRGB_ERR_CUDA, "unknown error");
    }
}

void require(bool ok, lvrgb_status st, const char* msg) {
    if (!ok) throw ApiError{st, msg};
}

cudaStream_t as_stream(void* s) { return static_cast<cudaStream_t>(s); }

struct DeviceScope {
    int prev = -1;
    explicit DeviceScope(int dev) {
        LVRGB_CUDA(cudaGetDevice(&prev));
        if (prev != dev) LVRGB_CUDA(cudaSetDevice(dev));
    }
    ~DeviceScope() {
        int cur = -1;
        if (cudaGetDevice(&cur) == cudaSuccess && cur != prev && prev >= 0) cudaSetDevice(prev);
    }
};

// Device view of an input array: device pointers pass through, host arrays
// are copied into a workspace buffer.
template <typename T>
const T* stage_in(Workspace& ws, const char* name, const T* p, size_t count, int on_device, cudaStream_t s) {
    if (on_device) return p;
    T* d = ws.get<T>(name, count);
    if (count) LVRGB_CUDA(cudaMemcpyAsync(d, p, sizeof(T) * count, cudaMemcpyHostToDevice, s));
    return d;
}
// Device destination for an output array; finish_out copies it to the host.
template <typename T>
T* stage_out(Workspace& ws, const char* name, T* p, size_t count, int on_device) {
    return on_device ? p : ws.get<T>(name, count);
}
template <typename T>
void finish_out(T* host, const T* dev, size_t count, int on_device, cudaStream_t s) {
    if (on_device || !host) return;
    if (count) LVRGB_CUDA(cudaMemcpyAsync(host, dev, sizeof(T) * count, cudaMemcpyDeviceToHost, s));
}

void check_kernel_error(lvrgb_surface s, cudaStream_t st) {
    int* h = reinterpret_cast<int*>(s->ws.pinned());
    h[0] = 0;
    LVRGB_CUDA(cudaMemcpyAsync(h, s->d_err, sizeof(int), cudaMemcpyDeviceToHost, st));
    LVRGB_CUDA(cudaStreamSynchronize(st));
    if (h[0]) {
        LVRGB_CUDA(cudaMemsetAsync(s->d_err, 0, sizeof(int), st));
        throw ApiError{LVRGB_ERR_KERNEL, (h[0] & kErrStack)  ? "kNN traversal exceeded its stack depth"
                                         : (h[0] & kErrWalk) ? "tree walk exceeded its bound (malformed tree)"
                                         : (h[0] & kErrTma)  ? "a TMA copy of marching cubes did not complete"
                                         : (h[0] & kErrTable) ? "the planar pass's edge table had no free slot"
                                                              : "a neighbour row was shorter than the RANSAC draws"};
    }
}

// Rows of AoS positions as float4 (xyz, row index bits), in the given order.
__global__ void pack_queries_kernel(const float* __restrict__ q, int nq, float4* __restrict__ qs) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nq) return;
    qs[i] = make_float4(q[3 * size_t(i)], q[3 * size_t(i) + 1], q[3 * size_t(i) + 2], __uint_as_float(uint32_t(i)));
}

__global__ void morton_to_aos_kernel(const float4* __restrict__ v, const float4* __restrict__ pts, int n,
                                     float* __restrict__ out) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    size_t o = __float_as_uint(pts[j].w);
    float4 a = v[j];
    out[3 * o] = a.x;
    out[3 * o + 1] = a.y;
    out[3 * o + 2] = a.z;
}
__global__ void aos_to_morton_kernel(const float* __restrict__ in, const float4* __restrict__ pts, int n,
                                     float4* __restrict__ v) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    size_t o = __float_as_uint(pts[j].w);
    v[j] = make_float4(in[3 * o], in[3 * o + 1], in[3 * o + 2], 0.0f);
}
__global__ void morton_to_orig_i32_kernel(const int32_t* __restrict__ v, const float4* __restrict__ pts, int n,
                                          int32_t* __restrict__ out) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    out[__float_as_uint(pts[j].w)] = v[j];
}
__global__ void decode_lattice_kernel(const uint64_t* __restrict__ keys, const uint32_t* __restrict__ sel, int n,
                                      int bx, int by, int bz, int32_t* __restrict__ out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t x, y, z;
    lattice_decode(keys[sel ? sel[i] : uint32_t(i)], x, y, z);
    out[3 * size_t(i)] = int(x) + bx;
    out[3 * size_t(i) + 1] = int(y) + by;
    out[3 * size_t(i) + 2] = int(z) + bz;
}
__global__ void decode_edges_kernel(const uint64_t* __restrict__ keys, int n, int bx, int by, int bz,
                                    int32_t* __restrict__ out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint64_t k = keys[i];
    uint32_t x, y, z;
    lattice_decode(k >> 2, x, y, z);
    out[4 * size_t(i)] = int(x) + bx;
    out[4 * size_t(i) + 1] = int(y) + by;
    out[4 * size_t(i) + 2] = int(z) + bz;
    out[4 * size_t(i) + 3] = int(k & 3);
}
__global__ void pos3_kernel(const float4* __restrict__ p, int n, float* __restrict__ out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 a = p[i];
    out[3 * size_t(i)] = a.x;
    out[3 * size_t(i) + 1] = a.y;
    out[3 * size_t(i) + 2] = a.z;
}

NormalsConfig normals_config(const lvrgb_surface_s* s) {
    NormalsConfig c;
    c.kn = s->cfg.kn;
    c.nem = s->cfg.nem;
    c.adaptive = s->cfg.adaptive;
    if (s->cfg.flip_set) {
        c.flip[0] = s->cfg.flip[0]; c.flip[1] = s->cfg.flip[1]; c.flip[2] = s->cfg.flip[2];
    } else {
        c.flip[0] = s->bb[6]; c.flip[1] = s->bb[7]; c.flip[2] = s->bb[8];
    }
    c.gap_threshold = s->cfg.gap_threshold > 0 ? s->cfg.gap_threshold : 1e-3f;
    return c;
}

void check_nem(int nem) {
    require(nem >= 0 && nem <= 4, LVRGB_ERR_INVALID_ARGUMENT, "nem must be 0, 1, 2, 3 or 4");
}

// k of the first normal search: 2 kn (adaptive k doubles before every
// search), kn for nem 4 (LBVHIndex::knn_normals searches once with kn).
int first_search_k(int kn, int nem) { return nem == 4 ? kn : 2 * kn; }

void check_lbvh_k(int kn, int nem) {
    require(nem != 4 || kn <= kSmemHeapMax, LVRGB_ERR_INVALID_ARGUMENT, "nem 4 needs kn <= 96");
}

// Sorts host/device query positions into Morton order on the device.
const float4* prepare_queries(lvrgb_surface s, const float* q, int64_t nq, int on_device, cudaStream_t st) {
    const float* dq = stage_in(s->ws, "api.q", q, size_t(nq) * 3, on_device, st);
    float4* qs = s->ws.get<float4>("api.qs", size_t(nq));
    sort_queries(dq, int(nq), s->d_box, qs, s->ws, st);
    return qs;
}

void record(lvrgb_surface s, int i, cudaStream_t st) {
    if (!s->ev[i]) LVRGB_CUDA(cudaEventCreate(&s->ev[i]));
    LVRGB_CUDA(cudaEventRecord(s->ev[i], st));
}

__global__ void first_nonfinite_kernel(const float* __restrict__ xyz, int n, int* __restrict__ first) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float x = xyz[3 * size_t(i)], y = xyz[3 * size_t(i) + 1], z = xyz[3 * size_t(i) + 2];
    if (!(isfinite(x) && isfinite(y) && isfinite(z))) atomicMin(first, i);
}

// lvr2's trees order points by comparisons that NaN breaks: a point with a
// non-finite coordinate is rejected (device array xyz, n x 3).
void require_finite_points(Workspace& ws, const float* xyz, int64_t n, cudaStream_t st) {
    if (n <= 0) return;
    int* d_first = ws.get<int>("api.first_bad", 1);
    const int init = INT_MAX;
    LVRGB_CUDA(cudaMemcpyAsync(d_first, &init, sizeof(int), cudaMemcpyHostToDevice, st));
    first_nonfinite_kernel<<<ceil_div(n, 256), 256, 0, st>>>(xyz, int(n), d_first);
    LVRGB_LAUNCH_CHECK();
    int first = INT_MAX;
    LVRGB_CUDA(cudaMemcpyAsync(&first, d_first, sizeof(int), cudaMemcpyDeviceToHost, st));
    LVRGB_CUDA(cudaStreamSynchronize(st));
    if (first != INT_MAX)
        throw ApiError{LVRGB_ERR_INVALID_ARGUMENT, "point " + std::to_string(first) + " has a non-finite coordinate"};
}

// (Re)builds the search structure and bounding box of a handle.
void build_points(lvrgb_surface s, const float* xyz, int64_t n, int on_device, cudaStream_t st) {
    require(n >= 0 && n < (int64_t(1) << 31), LVRGB_ERR_INVALID_ARGUMENT, "point count must be in [0, 2^31)");
    require(n == 0 || xyz != nullptr, LVRGB_ERR_INVALID_ARGUMENT, "xyz is NULL");
    s->has_normals = s->has_raw = s->has_grid = false;
    const float* dx = stage_in(s->ws, "api.xyz", xyz, size_t(n) * 3, on_device, st);
    require_finite_points(s->ws, dx, n, st);
    record(s, 0, st);
    lbvh_build(dx, int(n), s->cfg.bucket, s->ws, "tree", s->T, s->d_box, s->d_err, st);
    s->T.seed_radius = s->cfg.seed_radius;
    record(s, 1, st);
    s->ev_used[0] = true;
    float h[6] = {0, 0, 0, 0, 0, 0};
    if (n > 0) {
        LVRGB_CUDA(cudaMemcpyAsync(h, s->d_box, 6 * sizeof(float), cudaMemcpyDeviceToHost, st));
        LVRGB_CUDA(cudaStreamSynchronize(st));
    } else {
        // empty BoundingBox: min = FLT_MAX, max = lowest (BoundingBox.tcc:45-53)
        h[0] = h[1] = h[2] = FLT_MAX;
        h[3] = h[4] = h[5] = -FLT_MAX;
    }
    for (int i = 0; i < 6; i++) s->bb[i] = h[i];
    // BoundingBox centroid (BoundingBox.tcc:210-214)
    for (int a = 0; a < 3; a++) s->bb[6 + a] = h[a] + 0.5f * (h[3 + a] - h[a]);
    // Morton frame of the tree (used to seed searches of arbitrary positions)
    const float ext = std::max(std::max(h[3] - h[0], h[4] - h[1]), h[5] - h[2]);
    for (int a = 0; a < 3; a++) s->T.mn[a] = h[a];
    s->T.scale = morton_scale(ext);
    check_kernel_error(s, st);
    s->normals = s->ws.get<float4>("api.normals", size_t(n));
    s->raw_normals = s->ws.get<float4>("api.raw_normals", size_t(n));
    s->kused = s->ws.get<int32_t>("api.kused", size_t(n));
}

}  // namespace

extern "C" {

void lvrgb_surface_config_default(lvrgb_surface_config* cfg) {
    if (!cfg) return;
    std::memset(cfg, 0, sizeof(*cfg));
    cfg->kn = 10;
    cfg->ki = 10;
    cfg->kd = 5;
    cfg->nem = 0;
    cfg->adaptive = 1;
    cfg->flip_set = 1;
    cfg->bucket = 32;
    cfg->gap_threshold = 1e-3f;
    cfg->device = 0;
    cfg->seed_radius = 1;
}

lvrgb_status lvrgb_surface_create(const lvrgb_surface_config* cfg, const float* xyz, int64_t n, int32_t on_device,
                                  void* stream, lvrgb_surface* out) {
    if (!out) return fail(LVRGB_ERR_INVALID_ARGUMENT, "out is NULL");
    *out = nullptr;
    lvrgb_surface s = nullptr;
    lvrgb_status st = guarded([&] {
        require(cfg != nullptr, LVRGB_ERR_INVALID_ARGUMENT, "cfg is NULL");
        require(n >= 0 && n < (int64_t(1) << 31), LVRGB_ERR_INVALID_ARGUMENT, "point count must be in [0, 2^31)");
        require(n == 0 || xyz != nullptr, LVRGB_ERR_INVALID_ARGUMENT, "xyz is NULL");
        require(cfg->kn > 0 && cfg->ki >= 0 && cfg->kd > 0, LVRGB_ERR_INVALID_ARGUMENT, "kn, kd must be > 0, ki >= 0");
        check_nem(cfg->nem);
        require(cfg->bucket >= 0 && cfg->bucket <= 32, LVRGB_ERR_INVALID_ARGUMENT, "bucket must be in 0..32");
        require(cfg->seed_radius >= 0 && cfg->seed_radius <= 16, LVRGB_ERR_INVALID_ARGUMENT,
                "seed_radius must be in 0..16");
        DeviceScope dev(cfg->device);
        cudaStream_t st = as_stream(stream);
        s = new lvrgb_surface_s();
        s->cfg = *cfg;
        if (s->cfg.bucket == 0) s->cfg.bucket = 32;
        if (s->cfg.seed_radius == 0) s->cfg.seed_radius = 1;
        s->device = cfg->device;
        s->d_box = s->ws.get<float>("api.box", 8);
        s->d_err = s->ws.get<int>("api.err", 4);
        s->d_stats = s->ws.get<uint32_t>("api.stats", kNormalStats);
        LVRGB_CUDA(cudaMemsetAsync(s->d_err, 0, 4 * sizeof(int), st));
        LVRGB_CUDA(cudaMemsetAsync(s->d_stats, 0, kNormalStats * sizeof(uint32_t), st));
        build_points(s, xyz, n, on_device, st);
        LVRGB_CUDA(cudaStreamSynchronize(st));
    });
    if (st != LVRGB_OK) {
        delete s;
        return st;
    }
    *out = s;
    return LVRGB_OK;
}

lvrgb_status lvrgb_surface_destroy(lvrgb_surface s) {
    if (!s) return LVRGB_OK;
    return guarded([&] {
        DeviceScope dev(s->device);
        delete s;
    });
}

lvrgb_status lvrgb_surface_set_k(lvrgb_surface s, int32_t kn, int32_t ki, int32_t kd) {
    return guarded([&] {
        require(s != nullptr, LVRGB_ERR_INVALID_ARGUMENT, "surface is NULL");
        require(kn != 0 && kd != 0, LVRGB_ERR_INVALID_ARGUMENT, "kn and kd must be > 0");
        if (kn > 0) s->cfg.kn = kn;
        if (ki >= 0) s->cfg.ki = ki;
        if (kd > 0) s->cfg.kd = kd;
    });
}

lvrgb_status lvrgb_surface_set_flip_point(lvrgb_surface s, float x, float y, float z) {
    return guarded([&] {
        require(s != nullptr, LVRGB_ERR_INVALID_ARGUMENT, "surface is NULL");
        s->cfg.flip_set = 1;
        s->cfg.flip[0] = x; s->cfg.flip[1] = y; s->cfg.flip[2] = z;
    });
}

lvrgb_status lvrgb_surface_set_scan_poses(lvrgb_surface s, const float* poses, int64_t np) {
    return guarded([&] {
        require(s != nullptr, LVRGB_ERR_INVALID_ARGUMENT, "surface is NULL");
        require(np >= 0 && np <= 8192, LVRGB_ERR_INVALID_ARGUMENT, "pose count must be in 0..8192");
        require(np == 0 || poses != nullptr, LVRGB_ERR_INVALID_ARGUMENT, "poses is NULL");
        for (int64_t i = 0; i < 3 * np; i++)
            require(std::isfinite(poses[i]), LVRGB_ERR_INVALID_ARGUMENT, "a pose has a non-finite coordinate");
        s->poses.assign(poses, poses + 3 * np);
        s->has_normals = s->has_raw = false;
    });
}

lvrgb_status lvrgb_surface_set_method(lvrgb_surface s, int32_t nem) {
    return guarded([&] {
        require(s != nullptr, LVRGB_ERR_INVALID_ARGUMENT, "surface is NULL");
        check_nem(nem);
        s->cfg.nem = nem;
    });
}

lvrgb_status lvrgb_surface_bounding_box(lvrgb_surface s, float out9[9]) {
    return guarded([&] {
        require(s != nullptr && out9 != nullptr, LVRGB_ERR_INVALID_ARGUMENT, "NULL argument");
        std::memcpy(out9, s->bb, sizeof(s->bb));
    });
}

lvrgb_status lvrgb_surface_num_points(lvrgb_surface s, int64_t* n) {
    return guarded([&] {
        require(s != nullptr && n != nullptr, LVRGB_ERR_INVALID_ARGUMENT, "NULL argument");
        *n = s->T.n;
    });
}

lvrgb_status lvrgb_calculate_normals(lvrgb_surface s, void* stream) {
    return guarded([&] {
        NvtxRange nvtx_range("lvrgb.calculate_normals");
        require(s != nullptr, LVRGB_ERR_INVALID_ARGUMENT, "surface is NULL");
        DeviceScope dev(s->device);
        cudaStream_t st = as_stream(stream);
        LVRGB_CUDA(cudaMemsetAsync(s->d_stats, 0, kNormalStats * sizeof(uint32_t), st));
        check_lbvh_k(s->cfg.kn, s->cfg.nem);
        require(s->cfg.nem != 1 || s->T.n == 0 || std::min<int64_t>(2 * int64_t(s->cfg.kn), s->T.n) >= 3,
                LVRGB_ERR_INVALID_ARGUMENT, "nem 1 needs at least 3 neighbours (kn >= 2 and 3 points)");
        NormalsConfig c = normals_config(s);
        if (!s->poses.empty() && s->T.n > 0) {
            const int np = int(s->poses.size() / 3);
            float* dp = s->ws.get<float>("api.poses", s->poses.size());
            LVRGB_CUDA(cudaMemcpyAsync(dp, s->poses.data(), s->poses.size() * sizeof(float), cudaMemcpyHostToDevice, st));
            float4* targets = s->ws.get<float4>("api.pose_targets", size_t(s->T.n));
            pose_flip_targets(s->T, dp, np, targets, st);
            c.flip_target = targets;
        }
        // The interpolation's kNN(ki) is the first ki of the estimation's
        // kNN (k >= 2kn, or kn for nem 4): keep those lists instead of searching again.
        const bool lists = s->cfg.ki > 0 && s->cfg.ki <= first_search_k(s->cfg.kn, s->cfg.nem);
        uint32_t* nbr = lists ? s->ws.get<uint32_t>("api.nbr", size_t(s->T.n) * size_t(s->cfg.ki)) : nullptr;
        record(s, 2, st);
        compute_normals(s->T, c, s->raw_normals, s->kused, s->ws, s->d_err, s->d_stats, st, nbr, s->cfg.ki);
        record(s, 3, st);
        s->ev_used[1] = true;
        s->has_raw = true;
        record(s, 4, st);
        if (lists)
            interpolate_from_lists(s->T.n, s->cfg.ki, nbr, s->raw_normals, s->normals, st);
        else if (s->cfg.ki > 0)
            interpolate_normals(s->T, s->cfg.ki, s->raw_normals, s->normals, s->ws, s->d_err, st);
        record(s, 5, st);
        s->ev_used[2] = true;
        if (s->cfg.ki <= 0 && s->T.n)
            LVRGB_CUDA(cudaMemcpyAsync(s->normals, s->raw_normals, sizeof(float4) * size_t(s->T.n),
                                       cudaMemcpyDeviceToDevice, st));
        check_kernel_error(s, st);
        s->has_normals = true;
    });
}

lvrgb_status lvrgb_interpolate_normals(lvrgb_surface s, void* stream) {
    return guarded([&] {
        NvtxRange nvtx_range("lvrgb.interpolate_normals");
        require(s != nullptr, LVRGB_ERR_INVALID_ARGUMENT, "surface is NULL");
        require(s->has_normals, LVRGB_ERR_STATE, "no normals: call lvrgb_calculate_normals or lvrgb_set_normals");
        require(s->cfg.ki > 0, LVRGB_ERR_INVALID_ARGUMENT, "ki must be > 0");
        DeviceScope dev(s->device);
        cudaStream_t st = as_stream(stream);
        float4* tmp = s->ws.get<float4>("api.interp_tmp", size_t(s->T.n));
        interpolate_normals(s->T, s->cfg.ki, s->normals, tmp, s->ws, s->d_err, st);
        if (s->T.n)
            LVRGB_CUDA(cudaMemcpyAsync(s->normals, tmp, sizeof(float4) * size_t(s->T.n), cudaMemcpyDeviceToDevice, st));
        check_kernel_error(s, st);
    });
}

lvrgb_status lvrgb_get_normals(lvrgb_surface s, float* normals, int32_t on_device, void* stream) {
    return guarded([&] {
        require(s != nullptr, LVRGB_ERR_INVALID_ARGUMENT, "surface is NULL");
        require(s->has_normals, LVRGB_ERR_STATE, "no normals: call lvrgb_calculate_normals or lvrgb_set_normals");
        require(normals != nullptr || s->T.n == 0, LVRGB_ERR_INVALID_ARGUMENT, "normals is NULL");
        DeviceScope dev(s->device);
        cudaStream_t st = as_stream(stream);
        const int n = s->T.n;
        float* d = stage_out(s->ws, "api.out3", normals, size_t(n) * 3, on_device);
        if (n) {
            morton_to_aos_kernel<<<ceil_div(n, 256), 256, 0, st>>>(s->normals, s->T.pts, n, d);
            LVRGB_LAUNCH_CHECK();
        }
        finish_out(normals, d, size_t(n) * 3, on_device, st);
        if (!on_device) LVRGB_CUDA(cudaStreamSynchronize(st));
    });
}

lvrgb_status lvrgb_get_normals_async(lvrgb_surface s, float* normals, void* stream, void* copy_stream) {
    return guarded([&] {
        require(s != nullptr, LVRGB_ERR_INVALID_ARGUMENT, "surface is NULL");
        require(s->has_normals, LVRGB_ERR_STATE, "no normals: call lvrgb_calculate_normals or lvrgb_set_normals");
        require(normals != nullptr || s->T.n == 0, LVRGB_ERR_INVALID_ARGUMENT, "normals is NULL");
        DeviceScope dev(s->device);
        const int n = s->T.n;
        if (n == 0) return;
        cudaStream_t st = as_stream(stream), cs = as_stream(copy_stream);
        float* d = s->ws.get<float>("api.normals_async", size_t(n) * 3);
        if (!s->copy_ev) LVRGB_CUDA(cudaEventCreateWithFlags(&s->copy_ev, cudaEventDisableTiming));
        LVRGB_CUDA(cudaEventRecord(s->copy_ev, st));
        LVRGB_CUDA(cudaStreamWaitEvent(cs, s->copy_ev, 0));
        morton_to_aos_kernel<<<ceil_div(n, 256), 256, 0, cs>>>(s->normals, s->T.pts, n, d);
        LVRGB_LAUNCH_CHECK();
        LVRGB_CUDA(cudaMemcpyAsync(normals, d, size_t(n) * 3 * sizeof(float), cudaMemcpyDeviceToHost, cs));
    });
}

lvrgb_status lvrgb_distance_stats(lvrgb_surface s, uint64_t out[8]) {
    return guarded([&] {
        require(s != nullptr && out != nullptr, LVRGB_ERR_INVALID_ARGUMENT, "NULL argument");
        DeviceScope dev(s->device);
        for (int i = 0; i < 8; i++) out[i] = 0;
        if (s->d_sdf_stats)
            LVRGB_CUDA(cudaMemcpy(out, s->d_sdf_stats, 8 * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
    });
}

lvrgb_status lvrgb_get_raw_normals(lvrgb_surface s, float* normals, int32_t* k_used, int32_t on_device,
                                   void* stream) {
    return guarded([&] {
        require(s != nullptr, LVRGB_ERR_INVALID_ARGUMENT, "surface is NULL");
        require(s->has_raw, LVRGB_ERR_STATE, "no estimated normals: call lvrgb_calculate_normals");
        DeviceScope dev(s->device);
        cudaStream_t st = as_stream(stream);
        const int n = s->T.n;
        if (normals) {
            float* d = stage_out(s->ws, "api.out3", normals, size_t(n) * 3, on_device);
            if (n) {
                morton_to_aos_kernel<<<ceil_div(n, 256), 256, 0, st>>>(s->raw_normals, s->T.pts, n, d);
                LVRGB_LAUNCH_CHECK();
            }
            finish_out(normals, d, size_t(n) * 3, on_device, st);
        }
        if (k_used) {
            int32_t* d = stage_out(s->ws, "api.outk", k_used, size_t(n), on_device);
            if (n) {
                morton_to_orig_i32_kernel<<<ceil_div(n, 256), 256, 0, st>>>(s->kused, s->T.pts, n, d);
                LVRGB_LAUNCH_CHECK();
            }
            finish_out(k_used, d, size_t(n), on_device, st);
        }
        if (!on_device) LVRGB_CUDA(cudaStreamSynchronize(st));
    });
}

lvrgb_status lvrgb_set_normals(lvrgb_surface s, const float* normals, int32_t on_device, void* stream) {
    return guarded([&] {
        require(s != nullptr, LVRGB_ERR_INVALID_ARGUMENT, "surface is NULL");
        require(normals != nullptr || s->T.n == 0, LVRGB_ERR_INVALID_ARGUMENT, "normals is NULL");
        DeviceScope dev(s->device);
        cudaStream_t st = as_stream(stream);
        const int n = s->T.n;
        const float* d = stage_in(s->ws, "api.in3", normals, size_t(n) * 3, on_device, st);
        if (n) {
            aos_to_morton_kernel<<<ceil_div(n, 256), 256, 0, st>>>(d, s->T.pts, n, s->normals);
            LVRGB_LAUNCH_CHECK();
        }
        if (!on_device) LVRGB_CUDA(cudaStreamSynchronize(st));
        s->has_normals = true;
    });
}

lvrgb_status lvrgb_normal_stats(lvrgb_surface s, uint32_t out[16]) {
    return guarded([&] {
        require(s != nullptr && out != nullptr, LVRGB_ERR_INVALID_ARGUMENT, "NULL argument");
        DeviceScope dev(s->device);
        LVRGB_CUDA(cudaMemcpy(out, s->d_stats, kNormalStats * sizeof(uint32_t), cudaMemcpyDeviceToHost));
    });
}

lvrgb_status lvrgb_knn(lvrgb_surface s, const float* q, int64_t nq, int32_t k, uint32_t* idx, float* dist,
                       int32_t* count, int32_t on_device, void* stream) {
    return guarded([&] {
        NvtxRange nvtx_range("lvrgb.knn");
        require(s != nullptr, LVRGB_ERR_INVALID_ARGUMENT, "surface is NULL");
        require(nq >= 0 && nq < (int64_t(1) << 31), LVRGB_ERR_INVALID_ARGUMENT, "query count out of range");
        require(k > 0 && k <= (1 << 16), LVRGB_ERR_INVALID_ARGUMENT, "k must be in 1..65536");
        require(nq == 0 || (q && idx && dist), LVRGB_ERR_INVALID_ARGUMENT, "NULL array");
        if (nq == 0) return;
        DeviceScope dev(s->device);
        cudaStream_t st = as_stream(stream);
        const float4* qs = prepare_queries(s, q, nq, on_device, st);
        const size_t rows = size_t(nq) * size_t(k);
        uint32_t* di = stage_out(s->ws, "api.idx", idx, rows, on_device);
        float* dd = stage_out(s->ws, "api.dist", dist, rows, on_device);
        int32_t* dc = count ? stage_out(s->ws, "api.cnt", count, size_t(nq), on_device) : nullptr;
        knn_rows(s->T, qs, int(nq), k, di, dd, dc, s->ws, s->d_err, st);
        finish_out(idx, di, rows, on_device, st);
        finish_out(dist, dd, rows, on_device, st);
        if (count) finish_out(count, dc, size_t(nq), on_device, st);
        if (!on_device) check_kernel_error(s, st);
    });
}

lvrgb_status lvrgb_normals_from_neighbors(lvrgb_surface s, const float* queries, int64_t nq, int32_t k,
                                          const uint32_t* n_neighbors, const uint32_t* indices, float* normals,
                                          int32_t on_device, void* stream) {
    return guarded([&] {
        require(s != nullptr, LVRGB_ERR_INVALID_ARGUMENT, "surface is NULL");
        require(nq >= 0 && nq < (int64_t(1) << 31), LVRGB_ERR_INVALID_ARGUMENT, "query count out of range");
        require(k > 0 && k <= (1 << 16), LVRGB_ERR_INVALID_ARGUMENT, "k must be in 1..65536");
        require(nq == 0 || (queries && n_neighbors && indices && normals), LVRGB_ERR_INVALID_ARGUMENT, "NULL array");
        if (nq == 0) return;
        DeviceScope dev(s->device);
        cudaStream_t st = as_stream(stream);
        const float* dq = stage_in(s->ws, "lists.q", queries, size_t(nq) * 3, on_device, st);
        const uint32_t* dc = stage_in(s->ws, "lists.c", n_neighbors, size_t(nq), on_device, st);
        const uint32_t* di = stage_in(s->ws, "lists.i", indices, size_t(nq) * size_t(k), on_device, st);
        uint32_t ext[2];
        list_extent(dc, di, int(nq), k, s->ws, ext, st);
        require(ext[0] <= uint32_t(k), LVRGB_ERR_INVALID_ARGUMENT, "a neighbour count exceeds k");
        require(ext[1] < uint32_t(s->T.n), LVRGB_ERR_INVALID_ARGUMENT, "a neighbour index is out of range");
        const NormalsConfig c = normals_config(s);
        float* dn = stage_out(s->ws, "lists.n", normals, size_t(nq) * 3, on_device);
        normals_from_lists(s->T, dq, int(nq), k, dc, di, c.flip, dn, st);
        finish_out(normals, dn, size_t(nq) * 3, on_device, st);
        check_kernel_error(s, st);
    });
}

lvrgb_status lvrgb_radius_search(lvrgb_surface s, const float* q, int64_t nq, int32_t k, float radius,
                                 uint32_t* idx, float* dist, int32_t* count, int32_t on_device, void* stream) {
    return guarded([&] {
        NvtxRange nvtx_range("lvrgb.radius_search");
        require(s != nullptr, LVRGB_ERR_INVALID_ARGUMENT, "surface is NULL");
        require(nq >= 0 && nq < (int64_t(1) << 31), LVRGB_ERR_INVALID_ARGUMENT, "query count out of range");
        require(k > 0 && k <= (1 << 16), LVRGB_ERR_INVALID_ARGUMENT, "k must be in 1..65536");
        const float r2 = radius * radius;
        require(radius > 0.0f && r2 > 0.0f && r2 < FLT_MAX, LVRGB_ERR_INVALID_ARGUMENT,
                "radius must be > 0 with a finite, nonzero square");
        require(nq == 0 || (q && idx && dist), LVRGB_ERR_INVALID_ARGUMENT, "NULL array");
        if (nq == 0) return;
        DeviceScope dev(s->device);
        cudaStream_t st = as_stream(stream);
        const float4* qs = prepare_queries(s, q, nq, on_device, st);
        const size_t rows = size_t(nq) * size_t(k);
        uint32_t* di = stage_out(s->ws, "api.idx", idx, rows, on_device);
        float* dd = stage_out(s->ws, "api.dist", dist, rows, on_device);
        int32_t* dc = count ? stage_out(s->ws, "api.cnt", count, size_t(nq), on_device) : nullptr;
        knn_rows(s->T, qs, int(nq), k, di, dd, dc, s->ws, s->d_err, st, r2);
        finish_out(idx, di, rows, on_device, st);
        finish_out(dist, dd, rows, on_device, st);
        if (count) finish_out(count, dc, size_t(nq), on_device, st);
        if (!on_device) check_kernel_error(s, st);
    });
}

lvrgb_status lvrgb_distance(lvrgb_surface s, const float* q, int64_t nq, float* projected, float* euclidean,
                            int32_t on_device, void* stream) {
    return guarded([&] {
        NvtxRange nvtx_range("lvrgb.distance");
        require(s != nullptr, LVRGB_ERR_INVALID_ARGUMENT, "surface is NULL");
        require(s->has_normals, LVRGB_ERR_STATE, "no normals: call lvrgb_calculate_normals or lvrgb_set_normals");
        require(nq >= 0 && nq < (int64_t(1) << 31), LVRGB_ERR_INVALID_ARGUMENT, "query count out of range");
        require(nq == 0 || (q && projected), LVRGB_ERR_INVALID_ARGUMENT, "NULL array");
        if (nq == 0) return;
        DeviceScope dev(s->device);
        cudaStream_t st = as_stream(stream);
        const float4* qs = prepare_queries(s, q, nq, on_device, st);
        float* dp = stage_out(s->ws, "api.d1", projected, size_t(nq), on_device);
        float* de = euclidean ? stage_out(s->ws, "api.d2", euclidean, size_t(nq), on_device) : nullptr;
        signed_distance_rows(s->T, s->normals, s->cfg.kd, qs, int(nq), 1.0f, dp, de, nullptr, s->ws, s->d_err, st);
        finish_out(projected, dp, size_t(nq), on_device, st);
        if (euclidean) finish_out(euclidean, de, size_t(nq), on_device, st);
        if (!on_device) check_kernel_error(s, st);
    });
}

lvrgb_status lvrgb_distance_adjoint(lvrgb_surface s, const float* q, int64_t nq, const float* grad_projected,
                                    const float* grad_euclidean, float* projected, float* euclidean, float* grad_q,
                                    float* grad_points, float* grad_normals, int32_t on_device, void* stream) {
    return guarded([&] {
        NvtxRange nvtx_range("lvrgb.distance_adjoint");
        require(s != nullptr, LVRGB_ERR_INVALID_ARGUMENT, "surface is NULL");
        require(s->has_normals, LVRGB_ERR_STATE, "no normals: call lvrgb_calculate_normals or lvrgb_set_normals");
        require(nq >= 0 && nq < (int64_t(1) << 31), LVRGB_ERR_INVALID_ARGUMENT, "query count out of range");
        require(nq == 0 || q, LVRGB_ERR_INVALID_ARGUMENT, "NULL query array");
        DeviceScope dev(s->device);
        cudaStream_t st = as_stream(stream);
        const int n = s->T.n;
        // gradients w.r.t. points and normals start at zero
        float4* gp = grad_points ? s->ws.get<float4>("adj.gp", size_t(n)) : nullptr;
        float4* gn = grad_normals ? s->ws.get<float4>("adj.gn", size_t(n)) : nullptr;
        if (gp && n) LVRGB_CUDA(cudaMemsetAsync(gp, 0, sizeof(float4) * size_t(n), st));
        if (gn && n) LVRGB_CUDA(cudaMemsetAsync(gn, 0, sizeof(float4) * size_t(n), st));
        AdjointOut o;
        if (nq > 0) {
            const float4* qs = prepare_queries(s, q, nq, on_device, st);
            o.gdist = grad_projected ? stage_in(s->ws, "adj.gd", grad_projected, size_t(nq), on_device, st) : nullptr;
            o.geucl = grad_euclidean ? stage_in(s->ws, "adj.ge", grad_euclidean, size_t(nq), on_device, st) : nullptr;
            o.dist = projected ? stage_out(s->ws, "adj.d", projected, size_t(nq), on_device) : nullptr;
            o.eucl = euclidean ? stage_out(s->ws, "adj.e", euclidean, size_t(nq), on_device) : nullptr;
            o.gq = grad_q ? stage_out(s->ws, "adj.gq", grad_q, size_t(nq) * 3, on_device) : nullptr;
            o.gp = gp;
            o.gn = gn;
            distance_adjoint(s->T, s->normals, s->cfg.kd, qs, int(nq), o, s->ws, s->d_err, st);
            if (projected) finish_out(projected, o.dist, size_t(nq), on_device, st);
            if (euclidean) finish_out(euclidean, o.eucl, size_t(nq), on_device, st);
            if (grad_q) finish_out(grad_q, o.gq, size_t(nq) * 3, on_device, st);
        }
        // Morton order -> input order
        for (int t = 0; t < 2; t++) {
            float* host = t == 0 ? grad_points : grad_normals;
            const float4* acc = t == 0 ? gp : gn;
            if (!host || n == 0) continue;
            float* d = stage_out(s->ws, t == 0 ? "adj.gpo" : "adj.gno", host, size_t(n) * 3, on_device);
            morton_to_aos_kernel<<<ceil_div(n, 256), 256, 0, st>>>(acc, s->T.pts, n, d);
            LVRGB_LAUNCH_CHECK();
            finish_out(host, d, size_t(n) * 3, on_device, st);
        }
        if (!on_device) check_kernel_error(s, st);
    });
}

lvrgb_status lvrgb_project_to_surface(lvrgb_surface s, const float* v, int64_t nv, int32_t steps,
                                      float* out_positions, float* out_normals, int32_t on_device, void* stream) {
    return guarded([&] {
        NvtxRange nvtx_range("lvrgb.project_to_surface");
        require(s != nullptr, LVRGB_ERR_INVALID_ARGUMENT, "surface is NULL");
        require(s->has_normals, LVRGB_ERR_STATE, "no normals: call lvrgb_calculate_normals or lvrgb_set_normals");
        require(nv >= 0 && nv < (int64_t(1) << 31), LVRGB_ERR_INVALID_ARGUMENT, "position count out of range");
        require(steps >= 1 && steps <= 64, LVRGB_ERR_INVALID_ARGUMENT, "steps must be in 1..64");
        require(nv == 0 || v, LVRGB_ERR_INVALID_ARGUMENT, "NULL position array");
        if (nv == 0) return;
        DeviceScope dev(s->device);
        cudaStream_t st = as_stream(stream);
        const float* dv = stage_in(s->ws, "proj.v", v, size_t(nv) * 3, on_device, st);
        float4* qs = s->ws.get<float4>("proj.qs", size_t(nv));
        pack_queries_kernel<<<ceil_div(nv, 256), 256, 0, st>>>(dv, int(nv), qs);
        LVRGB_LAUNCH_CHECK();
        float* op = out_positions ? stage_out(s->ws, "proj.op", out_positions, size_t(nv) * 3, on_device) : nullptr;
        float* on = out_normals ? stage_out(s->ws, "proj.on", out_normals, size_t(nv) * 3, on_device) : nullptr;
        project_to_surface(s->T, s->normals, s->cfg.kd, qs, int(nv), steps, op, on, s->ws, s->d_err, st);
        if (op) finish_out(out_positions, op, size_t(nv) * 3, on_device, st);
        if (on) finish_out(out_normals, on, size_t(nv) * 3, on_device, st);
        if (!on_device) check_kernel_error(s, st);
    });
}

lvrgb_status lvrgb_grid_distances(lvrgb_surface s, const float* q, int64_t nq, float voxel_size, float* distance,
                                  uint8_t* invalid, int32_t on_device, void* stream) {
    return guarded([&] {
        NvtxRange nvtx_range("lvrgb.grid_distances");
        require(s != nullptr, LVRGB_ERR_INVALID_ARGUMENT, "surface is NULL");
        require(s->has_normals, LVRGB_ERR_STATE, "no normals: call lvrgb_calculate_normals or lvrgb_set_normals");
        require(nq >= 0 && nq < (int64_t(1) << 31), LVRGB_ERR_INVALID_ARGUMENT, "query count out of range");
        require(voxel_size > 0, LVRGB_ERR_INVALID_ARGUMENT, "voxel_size must be > 0");
        require(nq == 0 || (q && distance && invalid), LVRGB_ERR_INVALID_ARGUMENT, "NULL array");
        if (nq == 0) return;
        DeviceScope dev(s->device);
        cudaStream_t st = as_stream(stream);
        const float4* qs = prepare_queries(s, q, nq, on_device, st);
        float* dp = stage_out(s->ws, "api.d1", distance, size_t(nq), on_device);
        uint8_t* di = stage_out(s->ws, "api.inv", invalid, size_t(nq), on_device);
        signed_distance_rows(s->T, s->normals, s->cfg.kd, qs, int(nq), voxel_size, dp, nullptr, di, s->ws, s->d_err,
                             st);
        finish_out(distance, dp, size_t(nq), on_device, st);
        finish_out(invalid, di, size_t(nq), on_device, st);
        if (!on_device) check_kernel_error(s, st);
    });
}

lvrgb_status lvrgb_interpolated_normal(lvrgb_surface s, const float* q, int64_t nq, float* out, int32_t on_device,
                                       void* stream) {
    return guarded([&] {
        require(s != nullptr, LVRGB_ERR_INVALID_ARGUMENT, "surface is NULL");
        require(s->has_normals, LVRGB_ERR_STATE, "no normals: call lvrgb_calculate_normals or lvrgb_set_normals");
        require(nq >= 0 && nq < (int64_t(1) << 31), LVRGB_ERR_INVALID_ARGUMENT, "query count out of range");
        require(s->cfg.ki > 0, LVRGB_ERR_INVALID_ARGUMENT, "ki must be > 0");
        require(nq == 0 || (q && out), LVRGB_ERR_INVALID_ARGUMENT, "NULL array");
        if (nq == 0) return;
        DeviceScope dev(s->device);
        cudaStream_t st = as_stream(stream);
        const float4* qs = prepare_queries(s, q, nq, on_device, st);
        float* d = stage_out(s->ws, "api.out3q", out, size_t(nq) * 3, on_device);
        interpolated_normal_rows(s->T, s->normals, s->cfg.ki, qs, int(nq), d, s->ws, s->d_err, st);
        finish_out(out, d, size_t(nq) * 3, on_device, st);
        if (!on_device) check_kernel_error(s, st);
    });
}

lvrgb_status lvrgb_reconstruct(lvrgb_surface s, const lvrgb_grid_config* g, lvrgb_mesh_info* info, void* stream) {
    return guarded([&] {
        NvtxRange nvtx_range("lvrgb.reconstruct");
        require(s != nullptr && g != nullptr, LVRGB_ERR_INVALID_ARGUMENT, "NULL argument");
        require(s->has_normals, LVRGB_ERR_STATE, "no normals: call lvrgb_calculate_normals or lvrgb_set_normals");
        require(g->resolution > 0, LVRGB_ERR_INVALID_ARGUMENT, "resolution must be > 0");
        require(g->decomposition == 0 || g->decomposition == 1, LVRGB_ERR_UNSUPPORTED,
                "decomposition must be 0 (MC) or 1 (PMC)");
        require(s->T.n > 0, LVRGB_ERR_INVALID_ARGUMENT, "empty point cloud");
        DeviceScope dev(s->device);
        cudaStream_t st = as_stream(stream);
        GridConfig c;
        c.resolution = g->resolution;
        c.is_voxelsize = g->is_voxelsize;
        c.extrude = g->extrude;
        c.kd = s->cfg.kd;
        c.decomposition = g->decomposition;
        if (!s->d_sdf_stats) s->d_sdf_stats = s->ws.get<unsigned long long>("api.sdfstats", 8);
        LVRGB_CUDA(cudaMemsetAsync(s->d_sdf_stats, 0, 8 * sizeof(unsigned long long), st));
        c.sdf_stats = s->d_sdf_stats;
        GridTimings tm;
        s->has_grid = false;
        s->ev_used[3] = false;  // a new mesh has had no planar pass yet
        grid_reconstruct(s->T, s->normals, s->bb, c, s->ws, s->grid, s->d_err, st, &tm);
        for (int i = 0; i < 4; i++) s->grid_ms[i] = tm.ms[i];
        check_kernel_error(s, st);
        s->has_grid = true;
        if (info) {
            info->cells_all = s->grid.ncells_all;
            info->grid_vertices = s->grid.nqp;
            info->cells_valid = s->grid.ncells_valid;
            info->vertices = s->grid.nverts;
            info->faces = s->grid.nfaces;
            info->voxelsize = s->grid.vs;
            for (int i = 0; i < 4; i++) info->stage_ms[i] = tm.ms[i];
        }
    });
}

lvrgb_status lvrgb_reconstruct_cells(lvrgb_surface s, float voxel_size, int32_t decomposition, const float* centers,
                                     const float* tsdf_values, int64_t ncells, const int64_t* chunk_offsets,
                                     int32_t nchunks, const float* inner_boxes, lvrgb_mesh_info* info,
                                     int32_t on_device, void* stream) {
    return guarded([&] {
        NvtxRange nvtx_range("lvrgb.reconstruct_cells");
        require(s != nullptr, LVRGB_ERR_INVALID_ARGUMENT, "surface is NULL");
        require(voxel_size > 0 && std::isfinite(voxel_size), LVRGB_ERR_INVALID_ARGUMENT, "voxel size must be > 0");
        require(decomposition == 0 || decomposition == 1, LVRGB_ERR_UNSUPPORTED,
                "decomposition must be 0 (MC) or 1 (PMC)");
        require(ncells >= 0 && ncells < (int64_t(1) << 28), LVRGB_ERR_INVALID_ARGUMENT, "cell count out of range");
        require(ncells == 0 || (centers && tsdf_values), LVRGB_ERR_INVALID_ARGUMENT, "NULL array");
        std::vector<int64_t> off;
        if (chunk_offsets) {
            require(nchunks >= 1, LVRGB_ERR_INVALID_ARGUMENT, "nchunks must be >= 1");
            require(chunk_offsets[0] == 0 && chunk_offsets[nchunks] == ncells, LVRGB_ERR_INVALID_ARGUMENT,
                    "chunk_offsets must run from 0 to ncells");
            for (int c = 0; c < nchunks; c++)
                require(chunk_offsets[c + 1] >= chunk_offsets[c], LVRGB_ERR_INVALID_ARGUMENT,
                        "chunk_offsets must not decrease");
            off.assign(chunk_offsets, chunk_offsets + nchunks + 1);
        } else {
            require(inner_boxes == nullptr, LVRGB_ERR_INVALID_ARGUMENT, "inner_boxes need chunk_offsets");
            nchunks = 1;
            off = {0, ncells};
        }
        DeviceScope dev(s->device);
        cudaStream_t st = as_stream(stream);
        const int n = int(ncells);
        const float* dc = stage_in(s->ws, "cells.c", centers, size_t(n) * 3, on_device, st);
        const float* dt = stage_in(s->ws, "cells.t", tsdf_values, size_t(n) * 8, on_device, st);
        int64_t* doff = s->ws.get<int64_t>("cells.off", off.size());
        LVRGB_CUDA(cudaMemcpyAsync(doff, off.data(), off.size() * sizeof(int64_t), cudaMemcpyHostToDevice, st));
        float* dbox = nullptr;
        if (inner_boxes) {
            dbox = s->ws.get<float>("cells.box", size_t(nchunks) * 6);
            LVRGB_CUDA(cudaMemcpyAsync(dbox, inner_boxes, size_t(nchunks) * 6 * sizeof(float), cudaMemcpyHostToDevice,
                                       st));
        }
        s->has_grid = false;
        s->ev_used[3] = false;  // a new mesh has had no planar pass yet
        grid_from_cells(dc, dt, n, doff, nchunks, dbox, voxel_size, decomposition, s->ws, s->grid, s->d_err, st);
        LVRGB_CUDA(cudaStreamSynchronize(st));  // the host offsets and boxes are read by then
        check_kernel_error(s, st);
        s->has_grid = true;
        if (info) {
            *info = lvrgb_mesh_info{};
            info->cells_all = s->grid.ncells_all;
            info->grid_vertices = s->grid.nqp;
            info->cells_valid = s->grid.ncells_valid;
            info->vertices = s->grid.nverts;
            info->faces = s->grid.nfaces;
            info->voxelsize = s->grid.vs;
        }
    });
}

lvrgb_status lvrgb_optimize_planar_faces(lvrgb_surface s, int32_t kc, int64_t* moved, void* stream) {
    return guarded([&] {
        NvtxRange nvtx_range("lvrgb.optimize_planar_faces");
        require(s != nullptr, LVRGB_ERR_INVALID_ARGUMENT, "surface is NULL");
        require(s->has_grid, LVRGB_ERR_STATE, "no mesh: call lvrgb_reconstruct");
        require(kc >= 1 && kc <= kSmemHeapMax, LVRGB_ERR_INVALID_ARGUMENT, "kc must be in 1..96");
        DeviceScope dev(s->device);
        cudaStream_t st = as_stream(stream);
        record(s, 6, st);
        const long long m = optimize_planar_faces(s->T, s->d_box, s->grid, kc, s->ws, s->d_err, st);
        record(s, 7, st);
        s->ev_used[3] = true;
        check_kernel_error(s, st);
        if (moved) *moved = m;
    });
}

lvrgb_status lvrgb_mesh_vertex_normals(lvrgb_surface s, float* vertex_normals, int32_t on_device, void* stream) {
    return guarded([&] {
        NvtxRange nvtx_range("lvrgb.mesh_vertex_normals");
        require(s != nullptr, LVRGB_ERR_INVALID_ARGUMENT, "surface is NULL");
        require(s->has_grid, LVRGB_ERR_STATE, "no mesh: call lvrgb_reconstruct");
        const size_t nv = size_t(s->grid.nverts);
        require(nv == 0 || vertex_normals != nullptr, LVRGB_ERR_INVALID_ARGUMENT, "NULL array");
        if (nv == 0) return;
        DeviceScope dev(s->device);
        cudaStream_t st = as_stream(stream);
        float* d = stage_out(s->ws, "api.vnormals", vertex_normals, nv * 3, on_device);
        mesh_vertex_normals(s->T, s->normals, s->d_box, s->grid.verts, int(nv), s->grid.faces, int(s->grid.nfaces),
                            d, s->ws, s->d_err, st);
        finish_out(vertex_normals, d, nv * 3, on_device, st);
        check_kernel_error(s, st);
    });
}

lvrgb_status lvrgb_mesh_vertex_colors(lvrgb_surface s, const uint8_t* point_colors, int32_t width,
                                      uint8_t* vertex_colors, int32_t on_device, void* stream) {
    return guarded([&] {
        require(s != nullptr, LVRGB_ERR_INVALID_ARGUMENT, "surface is NULL");
        require(s->has_grid, LVRGB_ERR_STATE, "no mesh: call lvrgb_reconstruct");
        require(width >= 1 && width <= 16, LVRGB_ERR_INVALID_ARGUMENT, "colour width must be 1..16 bytes");
        const size_t nv = size_t(s->grid.nverts);
        require(nv == 0 || (point_colors && vertex_colors), LVRGB_ERR_INVALID_ARGUMENT, "NULL array");
        if (nv == 0) return;
        DeviceScope dev(s->device);
        cudaStream_t st = as_stream(stream);
        const uint8_t* dc = stage_in(s->ws, "vc.in", point_colors, size_t(s->T.n) * width, on_device, st);
        uint8_t* d = stage_out(s->ws, "api.vcolors", vertex_colors, nv * width, on_device);
        mesh_vertex_colors(s->T, s->d_box, s->grid.verts, int(nv), dc, width, d, s->ws, s->d_err, st);
        finish_out(vertex_colors, d, nv * width, on_device, st);
        check_kernel_error(s, st);
    });
}

lvrgb_status lvrgb_vertex_normals(lvrgb_surface s, const float* vertices, int64_t nv, const uint32_t* faces,
                                  int64_t nf, float* vertex_normals, int64_t* nearest_count, int32_t on_device,
                                  void* stream) {
    return guarded([&] {
        NvtxRange nvtx_range("lvrgb.vertex_normals");
        require(s != nullptr, LVRGB_ERR_INVALID_ARGUMENT, "surface is NULL");
        require(s->has_normals, LVRGB_ERR_STATE, "no normals: call lvrgb_calculate_normals or lvrgb_set_normals");
        require(nv >= 0 && nv < (int64_t(1) << 31), LVRGB_ERR_INVALID_ARGUMENT, "vertex count out of range");
        require(nf >= 0 && 3 * nf < (int64_t(1) << 31), LVRGB_ERR_INVALID_ARGUMENT, "face count out of range");
        require(nv == 0 || (vertices && vertex_normals), LVRGB_ERR_INVALID_ARGUMENT, "NULL array");
        require(nf == 0 || faces, LVRGB_ERR_INVALID_ARGUMENT, "NULL array");
        require(nf == 0 || nv > 0, LVRGB_ERR_INVALID_ARGUMENT, "faces without vertices");
        long long mz = 0;
        if (nv > 0) {
            DeviceScope dev(s->device);
            cudaStream_t st = as_stream(stream);
            const float* dv = stage_in(s->ws, "vn.in.v", vertices, size_t(nv) * 3, on_device, st);
            const uint32_t* df = stage_in(s->ws, "vn.in.f", faces, size_t(nf) * 3, on_device, st);
            require(max_index(df, size_t(nf) * 3, s->ws, st) < uint64_t(nv), LVRGB_ERR_INVALID_ARGUMENT,
                    "face index out of range");
            float* d = stage_out(s->ws, "api.vnormals", vertex_normals, size_t(nv) * 3, on_device);
            mz = mesh_vertex_normals(s->T, s->normals, s->d_box, dv, int(nv), df, int(nf), d, s->ws, s->d_err, st);
            finish_out(vertex_normals, d, size_t(nv) * 3, on_device, st);
            check_kernel_error(s, st);
        }
        if (nearest_count) *nearest_count = mz;
    });
}

lvrgb_status lvrgb_get_mesh(lvrgb_surface s, float* vertices, uint32_t* faces, int32_t* vertex_edges,
                            int32_t on_device, void* stream) {
    return guarded([&] {
        require(s != nullptr, LVRGB_ERR_INVALID_ARGUMENT, "surface is NULL");
        require(s->has_grid, LVRGB_ERR_STATE, "no mesh: call lvrgb_reconstruct");
        DeviceScope dev(s->device);
        cudaStream_t st = as_stream(stream);
        const GridResult& R = s->grid;
        const size_t nv = size_t(R.nverts), nf = size_t(R.nfaces);
        if (vertices) {
            if (on_device) {
                if (nv) LVRGB_CUDA(cudaMemcpyAsync(vertices, R.verts, nv * 3 * sizeof(float), cudaMemcpyDeviceToDevice, st));
            } else {
                finish_out(vertices, R.verts, nv * 3, 0, st);
            }
        }
        if (faces) {
            if (on_device) {
                if (nf) LVRGB_CUDA(cudaMemcpyAsync(faces, R.faces, nf * 3 * sizeof(uint32_t), cudaMemcpyDeviceToDevice, st));
            } else {
                finish_out(faces, R.faces, nf * 3, 0, st);
            }
        }
        if (vertex_edges) {
            int32_t* d = stage_out(s->ws, "api.vedges", vertex_edges, nv * 4, on_device);
            if (nv) {
                decode_edges_kernel<<<ceil_div(nv, 256), 256, 0, st>>>(R.vert_keys, int(nv), R.base[0], R.base[1],
                                                                             R.base[2], d);
                LVRGB_LAUNCH_CHECK();
            }
            finish_out(vertex_edges, d, nv * 4, on_device, st);
        }
        if (!on_device) LVRGB_CUDA(cudaStreamSynchronize(st));
    });
}

lvrgb_status lvrgb_get_grid(lvrgb_surface s, int32_t* lattice, float* position, float* distance, uint8_t* invalid,
                            int32_t on_device, void* stream) {
    return guarded([&] {
        require(s != nullptr, LVRGB_ERR_INVALID_ARGUMENT, "surface is NULL");
        require(s->has_grid, LVRGB_ERR_STATE, "no grid: call lvrgb_reconstruct");
        DeviceScope dev(s->device);
        cudaStream_t st = as_stream(stream);
        const GridResult& R = s->grid;
        const size_t nq = size_t(R.nqp);
        if (lattice) {
            int32_t* d = stage_out(s->ws, "api.lat", lattice, nq * 3, on_device);
            if (nq) {
                decode_lattice_kernel<<<ceil_div(nq, 256), 256, 0, st>>>(R.qp_keys, nullptr, int(nq), R.base[0],
                                                                               R.base[1], R.base[2], d);
                LVRGB_LAUNCH_CHECK();
            }
            finish_out(lattice, d, nq * 3, on_device, st);
        }
        if (position) {
            float* d = stage_out(s->ws, "api.pos", position, nq * 3, on_device);
            if (nq) {
                pos3_kernel<<<ceil_div(nq, 256), 256, 0, st>>>(R.qp_pos, int(nq), d);
                LVRGB_LAUNCH_CHECK();
            }
            finish_out(position, d, nq * 3, on_device, st);
        }
        if (distance) {
            if (on_device) {
                if (nq) LVRGB_CUDA(cudaMemcpyAsync(distance, R.qp_dist, nq * sizeof(float), cudaMemcpyDeviceToDevice, st));
            } else {
                finish_out(distance, R.qp_dist, nq, 0, st);
            }
        }
        if (invalid) {
            if (on_device) {
                if (nq) LVRGB_CUDA(cudaMemcpyAsync(invalid, R.qp_invalid, nq, cudaMemcpyDeviceToDevice, st));
            } else {
                finish_out(invalid, R.qp_invalid, nq, 0, st);
            }
        }
        if (!on_device) LVRGB_CUDA(cudaStreamSynchronize(st));
    });
}

namespace {
// Builds the half-edge arrays of faces (device) and copies them out.
void halfedges_out(lvrgb_surface s, const uint32_t* faces, int nf, int nv, lvrgb_halfedge_info* info,
                   uint32_t* he_vertex, uint32_t* he_next, uint32_t* he_prev, uint32_t* he_face, uint32_t* vertex_he,
                   uint32_t* face_he, int32_t on_device, cudaStream_t st) {
    HalfedgeMesh H;
    build_halfedges(faces, nf, nv, s->ws, H, st);
    if (info) {
        info->vertices = H.nverts;
        info->faces = H.nfaces;
        info->edges = H.nedges;
        info->boundary_halfedges = H.boundary;
        info->complex_edges = H.complex_edges;
        info->complex_vertices = H.complex_vertices;
    }
    require(H.complex_edges == 0, LVRGB_ERR_TOPOLOGY, "the mesh has complex edges");
    const size_t nh = size_t(2 * H.nedges);
    auto out = [&](uint32_t* dst, const uint32_t* src, size_t n, const char* name) {
        if (!dst || n == 0) return;
        uint32_t* d = stage_out(s->ws, name, dst, n, on_device);
        LVRGB_CUDA(cudaMemcpyAsync(d, src, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, st));
        finish_out(dst, d, n, on_device, st);
    };
    out(he_vertex, H.he_vertex, nh, "he.out.v");
    out(he_next, H.he_next, nh, "he.out.n");
    out(he_prev, H.he_prev, nh, "he.out.p");
    out(he_face, H.he_face, nh, "he.out.f");
    out(vertex_he, H.vertex_he, size_t(H.nverts), "he.out.vh");
    out(face_he, H.face_he, size_t(H.nfaces), "he.out.fh");
    if (!on_device) LVRGB_CUDA(cudaStreamSynchronize(st));
}
}  // namespace

lvrgb_status lvrgb_mesh_halfedges(lvrgb_surface s, lvrgb_halfedge_info* info, uint32_t* he_vertex, uint32_t* he_next,
                                  uint32_t* he_prev, uint32_t* he_face, uint32_t* vertex_he, uint32_t* face_he,
                                  int32_t on_device, void* stream) {
    return guarded([&] {
        NvtxRange nvtx_range("lvrgb.mesh_halfedges");
        require(s != nullptr, LVRGB_ERR_INVALID_ARGUMENT, "surface is NULL");
        require(s->has_grid, LVRGB_ERR_STATE, "no mesh: call lvrgb_reconstruct");
        DeviceScope dev(s->device);
        halfedges_out(s, s->grid.faces, int(s->grid.nfaces), int(s->grid.nverts), info, he_vertex, he_next, he_prev,
                      he_face, vertex_he, face_he, on_device, as_stream(stream));
    });
}

lvrgb_status lvrgb_halfedges(lvrgb_surface s, const uint32_t* faces, int64_t nf, int64_t nv, lvrgb_halfedge_info* info,
                             uint32_t* he_vertex, uint32_t* he_next, uint32_t* he_prev, uint32_t* he_face,
                             uint32_t* vertex_he, uint32_t* face_he, int32_t on_device, void* stream) {
    return guarded([&] {
        NvtxRange nvtx_range("lvrgb.halfedges");
        require(s != nullptr, LVRGB_ERR_INVALID_ARGUMENT, "surface is NULL");
        require(nf >= 0 && 3 * nf < (int64_t(1) << 31), LVRGB_ERR_INVALID_ARGUMENT, "face count out of range");
        require(nv >= 0 && nv < (int64_t(1) << 31), LVRGB_ERR_INVALID_ARGUMENT, "vertex count out of range");
        require(nf == 0 || faces != nullptr, LVRGB_ERR_INVALID_ARGUMENT, "NULL array");
        DeviceScope dev(s->device);
        cudaStream_t st = as_stream(stream);
        const uint32_t* df = stage_in(s->ws, "he.in.f", faces, size_t(nf) * 3, on_device, st);
        if (nf > 0)
            require(max_index(df, size_t(nf) * 3, s->ws, st) < uint64_t(nv), LVRGB_ERR_INVALID_ARGUMENT,
                    "face index out of range");
        halfedges_out(s, df, int(nf), int(nv), info, he_vertex, he_next, he_prev, he_face, vertex_he, face_he,
                      on_device, st);
    });
}

lvrgb_status lvrgb_get_cell_tsdf(lvrgb_surface s, float* centers, float* tsdf_values, int32_t on_device,
                                 void* stream) {
    return guarded([&] {
        require(s != nullptr, LVRGB_ERR_INVALID_ARGUMENT, "surface is NULL");
        require(s->has_grid, LVRGB_ERR_STATE, "no grid: call lvrgb_reconstruct");
        const size_t n = size_t(s->grid.ncells_valid);
        if (n == 0 || (!centers && !tsdf_values)) return;
        DeviceScope dev(s->device);
        cudaStream_t st = as_stream(stream);
        float* dc = centers ? stage_out(s->ws, "api.cc", centers, n * 3, on_device) : nullptr;
        float* dt = tsdf_values ? stage_out(s->ws, "api.tsdf", tsdf_values, n * 8, on_device) : nullptr;
        cell_tsdf(s->grid, dc, dt, st);
        if (centers) finish_out(centers, dc, n * 3, on_device, st);
        if (tsdf_values) finish_out(tsdf_values, dt, n * 8, on_device, st);
        if (!on_device) LVRGB_CUDA(cudaStreamSynchronize(st));
    });
}

lvrgb_status lvrgb_get_cells(lvrgb_surface s, int32_t* cells_all, int32_t* cells_valid, int32_t on_device,
                             void* stream) {
    return guarded([&] {
        require(s != nullptr, LVRGB_ERR_INVALID_ARGUMENT, "surface is NULL");
        require(s->has_grid, LVRGB_ERR_STATE, "no grid: call lvrgb_reconstruct");
        DeviceScope dev(s->device);
        cudaStream_t st = as_stream(stream);
        const GridResult& R = s->grid;
        if (cells_all) {
            const size_t n = size_t(R.ncells_all);
            int32_t* d = stage_out(s->ws, "api.ca", cells_all, n * 3, on_device);
            if (n) {
                decode_lattice_kernel<<<ceil_div(n, 256), 256, 0, st>>>(R.cell_keys, nullptr, int(n), R.base[0],
                                                                             R.base[1], R.base[2], d);
                LVRGB_LAUNCH_CHECK();
            }
            finish_out(cells_all, d, n * 3, on_device, st);
        }
        if (cells_valid) {
            const size_t n = size_t(R.ncells_valid);
            int32_t* d = stage_out(s->ws, "api.cv", cells_valid, n * 3, on_device);
            if (n) {
                decode_lattice_kernel<<<ceil_div(n, 256), 256, 0, st>>>(R.cell_keys, R.valid_cells, int(n),
                                                                             R.base[0], R.base[1], R.base[2], d);
                LVRGB_LAUNCH_CHECK();
            }
            finish_out(cells_valid, d, n * 3, on_device, st);
        }
        if (!on_device) LVRGB_CUDA(cudaStreamSynchronize(st));
    });
}

lvrgb_status lvrgb_surface_set_points(lvrgb_surface s, const float* xyz, int64_t n, int32_t on_device,
                                      void* stream) {
    return guarded([&] {
        require(s != nullptr, LVRGB_ERR_INVALID_ARGUMENT, "surface is NULL");
        DeviceScope dev(s->device);
        build_points(s, xyz, n, on_device, as_stream(stream));
    });
}

lvrgb_status lvrgb_surface_timings(lvrgb_surface s, float out[8]) {
    return guarded([&] {
        require(s != nullptr && out != nullptr, LVRGB_ERR_INVALID_ARGUMENT, "NULL argument");
        DeviceScope dev(s->device);
        for (int i = 0; i < 8; i++) out[i] = 0.0f;
        for (int k = 0; k < 3; k++) {
            if (!s->ev_used[k]) continue;
            LVRGB_CUDA(cudaEventSynchronize(s->ev[2 * k + 1]));
            LVRGB_CUDA(cudaEventElapsedTime(&out[k], s->ev[2 * k], s->ev[2 * k + 1]));
        }
        for (int i = 0; i < 4; i++) out[3 + i] = s->grid_ms[i];
        if (s->ev_used[3]) {
            LVRGB_CUDA(cudaEventSynchronize(s->ev[7]));
            LVRGB_CUDA(cudaEventElapsedTime(&out[7], s->ev[6], s->ev[7]));
        }
    });
}

lvrgb_status lvrgb_kernel_launches(uint64_t* out) {
    if (!out) return fail(LVRGB_ERR_INVALID_ARGUMENT, "out is NULL");
    *out = g_launches.load();
    return LVRGB_OK;
}

lvrgb_status lvrgb_debug_fail_allocation(int64_t n) {
    alloc_fault_countdown().store(n > 0 ? n : 0);
    return LVRGB_OK;
}

lvrgb_status lvrgb_debug_round_collapse(int32_t enable) {
    g_round_collapse.store(enable ? 1 : 0);
    return LVRGB_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Scan projects: normals of many scans in one pass (lvrgb_batch_*).
// ---------------------------------------------------------------------------
struct lvrgb_batch_s {
    lvrgb_surface_config cfg;
    int device = 0;
    Workspace ws;
    std::vector<int64_t> offsets;
    std::vector<float> flips;
    float* d_xyz = nullptr;
    BatchRun R;
    int* d_err = nullptr;
    uint32_t* d_stats = nullptr;
    cudaStream_t bs = nullptr;  // the batch's own stream (graphs need a non-default stream)
    cudaEvent_t ev[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    // per search round of the last timed eager run (lvrgb_batch_round_times)
    cudaEvent_t round_ev[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    bool rounds_timed = false;
    // search rounds collapsed after this one (0: none), chosen from the
    // fitted-per-round counts of the previous eager run
    int collapse_after = 0;
    // launch shape of the one-warp-per-query searches (lvrgb_batch_autotune)
    int wide_tile = 0, wide_slack = 2;
    cudaGraphExec_t exec = nullptr;
    bool ran = false;
    float ms[4] = {0, 0, 0, 0};
    ~lvrgb_batch_s() {
        if (exec) cudaGraphExecDestroy(exec);
        for (auto& e : ev)
            if (e) cudaEventDestroy(e);
        for (auto& e : round_ev)
            if (e) cudaEventDestroy(e);
        if (bs) cudaStreamDestroy(bs);
    }
};

namespace {

NormalsConfig batch_config(const lvrgb_batch_s* b) {
    NormalsConfig c;
    c.kn = b->cfg.kn;
    c.nem = b->cfg.nem;
    c.adaptive = b->cfg.adaptive;
    c.gap_threshold = b->cfg.gap_threshold > 0 ? b->cfg.gap_threshold : 1e-3f;
    c.wide_tile = b->wide_tile;
    c.wide_slack = b->wide_slack;
    return c;
}

void batch_run_eager(lvrgb_batch b, bool timed) {
    if (b->R.prepared_bucket != b->cfg.bucket)
        batch_prepare(b->offsets, b->flips, batch_config(b), b->cfg.ki, b->cfg.bucket, b->ws, b->R, b->bs);
    if (timed)
        for (auto& e : b->round_ev)
            if (!e) LVRGB_CUDA(cudaEventCreate(&e));
    batch_pipeline(b->d_xyz, batch_config(b), b->cfg.ki, b->cfg.seed_radius, b->ws, b->R, b->d_err, b->d_stats, b->bs,
                   timed ? b->ev : nullptr, timed ? b->round_ev : nullptr, b->collapse_after);
    if (timed) b->rounds_timed = true;
    b->ran = true;
}

// Runs the pipeline on the batch stream, ordered after `caller` and before
// whatever the caller enqueues next.
template <typename F>
void on_batch_stream(lvrgb_batch b, cudaStream_t caller, F&& f) {
    LVRGB_CUDA(cudaEventRecord(b->ev[4], caller));
    LVRGB_CUDA(cudaStreamWaitEvent(b->bs, b->ev[4], 0));
    f();
    LVRGB_CUDA(cudaEventRecord(b->ev[5], b->bs));
    LVRGB_CUDA(cudaStreamWaitEvent(caller, b->ev[5], 0));
}

void batch_check(lvrgb_batch b) {
    int herr = 0;
    LVRGB_CUDA(cudaStreamSynchronize(b->bs));
    LVRGB_CUDA(cudaMemcpy(&herr, b->d_err, sizeof(int), cudaMemcpyDeviceToHost));
    if (herr) {
        LVRGB_CUDA(cudaMemset(b->d_err, 0, sizeof(int)));
        throw ApiError{LVRGB_ERR_KERNEL, "kNN traversal reported an internal limit"};
    }
}

}  // namespace

extern "C" {

lvrgb_status lvrgb_batch_create(const lvrgb_surface_config* cfg, const float* xyz, const int64_t* scan_offsets,
                                int32_t nscans, const float* flip_points, int32_t on_device, void* stream,
                                lvrgb_batch* out) {
    if (!out) return fail(LVRGB_ERR_INVALID_ARGUMENT, "out is NULL");
    *out = nullptr;
    lvrgb_batch b = nullptr;
    lvrgb_status st = guarded([&] {
        require(cfg && scan_offsets && flip_points, LVRGB_ERR_INVALID_ARGUMENT, "NULL argument");
        require(nscans >= 1 && nscans <= 65535, LVRGB_ERR_INVALID_ARGUMENT, "nscans must be in 1..65535");
        require(cfg->kn > 0 && cfg->ki >= 0, LVRGB_ERR_INVALID_ARGUMENT, "kn must be > 0, ki >= 0");
        check_nem(cfg->nem);
        require(cfg->nem != 1, LVRGB_ERR_UNSUPPORTED, "nem 1 (RANSAC) runs on single surfaces, not on scan projects");
        check_lbvh_k(cfg->kn, cfg->nem);
        require(cfg->ki <= first_search_k(cfg->kn, cfg->nem), LVRGB_ERR_UNSUPPORTED,
                "scan projects interpolate from the estimation's neighbour lists: ki must be <= 2 * kn "
                "(<= kn for nem 4)");
        require(cfg->bucket >= 0 && cfg->bucket <= 32, LVRGB_ERR_INVALID_ARGUMENT, "bucket must be in 0..32");
        require(scan_offsets[0] == 0, LVRGB_ERR_INVALID_ARGUMENT, "scan_offsets[0] must be 0");
        for (int k = 0; k < nscans; k++)
            require(scan_offsets[k + 1] > scan_offsets[k], LVRGB_ERR_INVALID_ARGUMENT,
                    "scan offsets must be strictly increasing (no empty scan)");
        const int64_t n = scan_offsets[nscans];
        require(n < (int64_t(1) << 31) - 32 * int64_t(nscans), LVRGB_ERR_INVALID_ARGUMENT, "too many points");
        require(xyz != nullptr, LVRGB_ERR_INVALID_ARGUMENT, "xyz is NULL");
        DeviceScope dev(cfg->device);
        cudaStream_t st = as_stream(stream);
        b = new lvrgb_batch_s();
        b->cfg = *cfg;
        if (b->cfg.bucket == 0) b->cfg.bucket = 32;
        if (b->cfg.seed_radius == 0) b->cfg.seed_radius = 1;
        b->device = cfg->device;
        b->offsets.assign(scan_offsets, scan_offsets + nscans + 1);
        b->flips.assign(flip_points, flip_points + 3 * size_t(nscans));
        LVRGB_CUDA(cudaStreamCreateWithFlags(&b->bs, cudaStreamNonBlocking));
        for (auto& e : b->ev) LVRGB_CUDA(cudaEventCreate(&e));
        b->d_err = b->ws.get<int>("batch.err", 4);
        b->d_stats = b->ws.get<uint32_t>("batch.stats", kNormalStats);
        LVRGB_CUDA(cudaMemsetAsync(b->d_err, 0, 4 * sizeof(int), st));
        b->d_xyz = b->ws.get<float>("batch.xyz", size_t(n) * 3);
        LVRGB_CUDA(cudaMemcpyAsync(b->d_xyz, xyz, size_t(n) * 3 * sizeof(float),
                                   on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, st));
        require_finite_points(b->ws, b->d_xyz, n, st);
    });
    if (st != LVRGB_OK) {
        delete b;
        return st;
    }
    *out = b;
    return LVRGB_OK;
}

lvrgb_status lvrgb_batch_destroy(lvrgb_batch b) {
    if (!b) return LVRGB_OK;
    return guarded([&] {
        DeviceScope dev(b->device);
        delete b;
    });
}

// After an eager run: collapse the search rounds from which almost nothing
// fits (same results, fewer searches).  The choice is made from the counts of
// that run and used by the following runs and the captured graph.
void choose_collapse(lvrgb_batch b) {
    uint32_t fitted[kNormalStats];
    LVRGB_CUDA(cudaMemcpy(fitted, b->d_stats, sizeof(fitted), cudaMemcpyDeviceToHost));
    int64_t n = 0;
    for (int r = 0; r < 5; r++) n += fitted[r];
    b->collapse_after = collapse_after_round(b->cfg.kn, b->cfg.nem, b->cfg.adaptive, fitted, n);
}

lvrgb_status lvrgb_batch_calculate_normals(lvrgb_batch b, int32_t use_graph, void* stream) {
    return guarded([&] {
        NvtxRange nvtx_range("lvrgb.batch_calculate_normals");
        require(b != nullptr, LVRGB_ERR_INVALID_ARGUMENT, "batch is NULL");
        DeviceScope dev(b->device);
        cudaStream_t caller = as_stream(stream);
        if (!use_graph) {
            on_batch_stream(b, caller, [&] { batch_run_eager(b, true); });
            batch_check(b);
            choose_collapse(b);
            for (int i = 0; i < 3; i++) LVRGB_CUDA(cudaEventElapsedTime(&b->ms[i], b->ev[i], b->ev[i + 1]));
            LVRGB_CUDA(cudaEventElapsedTime(&b->ms[3], b->ev[0], b->ev[3]));
            return;
        }
        if (!b->exec) {
            // An eager pass sizes every buffer and sets kernel attributes, then
            // the same launch sequence is captured once.
            on_batch_stream(b, caller, [&] { batch_run_eager(b, false); });
            batch_check(b);
            choose_collapse(b);
            // and once more with that choice, so the capture finds every buffer sized
            on_batch_stream(b, caller, [&] { batch_run_eager(b, false); });
            batch_check(b);
            cudaGraph_t g = nullptr;
            LVRGB_CUDA(cudaStreamBeginCapture(b->bs, cudaStreamCaptureModeRelaxed));
            try {
                batch_run_eager(b, false);
            } catch (...) {
                cudaStreamEndCapture(b->bs, &g);
                if (g) cudaGraphDestroy(g);
                throw;
            }
            LVRGB_CUDA(cudaStreamEndCapture(b->bs, &g));
            const cudaError_t e = cudaGraphInstantiate(&b->exec, g, 0);
            cudaGraphDestroy(g);
            LVRGB_CUDA(e);
        }
        on_batch_stream(b, caller, [&] {
            LVRGB_CUDA(cudaEventRecord(b->ev[0], b->bs));
            LVRGB_CUDA(cudaGraphLaunch(b->exec, b->bs));
            LVRGB_CUDA(cudaEventRecord(b->ev[3], b->bs));
        });
        batch_check(b);
        b->ms[0] = b->ms[1] = b->ms[2] = 0.0f;
        LVRGB_CUDA(cudaEventElapsedTime(&b->ms[3], b->ev[0], b->ev[3]));
    });
}

lvrgb_status lvrgb_batch_get_normals(lvrgb_batch b, float* normals, int32_t on_device, void* stream) {
    return guarded([&] {
        require(b != nullptr && normals != nullptr, LVRGB_ERR_INVALID_ARGUMENT, "NULL argument");
        require(b->ran, LVRGB_ERR_STATE, "no normals: call lvrgb_batch_calculate_normals");
        DeviceScope dev(b->device);
        cudaStream_t st = as_stream(stream);
        const size_t n = size_t(b->offsets.back());
        float* d = stage_out(b->ws, "batch.out3", normals, n * 3, on_device);
        on_batch_stream(b, st, [&] { batch_scatter_normals(b->R, d, b->bs); });
        finish_out(normals, d, n * 3, on_device, st);
        if (!on_device) LVRGB_CUDA(cudaStreamSynchronize(st));
    });
}

lvrgb_status lvrgb_batch_grid_distances(lvrgb_batch b, const float* q, const int64_t* q_offsets, float voxel_size,
                                        float* distance, uint8_t* invalid, int32_t on_device, void* stream) {
    return guarded([&] {
        NvtxRange nvtx_range("lvrgb.batch_grid_distances");
        require(b != nullptr && q_offsets != nullptr, LVRGB_ERR_INVALID_ARGUMENT, "NULL argument");
        require(b->ran, LVRGB_ERR_STATE, "no normals: call lvrgb_batch_calculate_normals");
        require(voxel_size > 0, LVRGB_ERR_INVALID_ARGUMENT, "voxel_size must be > 0");
        const int S = int(b->offsets.size()) - 1;
        require(q_offsets[0] == 0, LVRGB_ERR_INVALID_ARGUMENT, "q_offsets[0] must be 0");
        for (int k = 0; k < S; k++)
            require(q_offsets[k + 1] >= q_offsets[k], LVRGB_ERR_INVALID_ARGUMENT, "q_offsets must not decrease");
        const int64_t nq = q_offsets[S];
        require(nq < (int64_t(1) << 31), LVRGB_ERR_INVALID_ARGUMENT, "query count out of range");
        require(nq == 0 || (q && distance && invalid), LVRGB_ERR_INVALID_ARGUMENT, "NULL array");
        if (nq == 0) return;
        DeviceScope dev(b->device);
        cudaStream_t st = as_stream(stream);
        int64_t* d_off = b->ws.get<int64_t>("chunk.qoff", size_t(S) + 1);
        LVRGB_CUDA(cudaMemcpyAsync(d_off, q_offsets, sizeof(int64_t) * (size_t(S) + 1), cudaMemcpyHostToDevice, st));
        const float* dq = stage_in(b->ws, "chunk.q", q, size_t(nq) * 3, on_device, st);
        float* dd = stage_out(b->ws, "chunk.d", distance, size_t(nq), on_device);
        uint8_t* di = stage_out(b->ws, "chunk.inv", invalid, size_t(nq), on_device);
        on_batch_stream(b, st, [&] {
            chunk_grid_distances(b->R.tree, b->R.normals, b->cfg.kd, dq, d_off, int(nq), voxel_size, dd, di, b->ws,
                                 b->d_err, b->bs);
        });
        finish_out(distance, dd, size_t(nq), on_device, st);
        finish_out(invalid, di, size_t(nq), on_device, st);
        LVRGB_CUDA(cudaStreamSynchronize(st));
        batch_check(b);
    });
}

lvrgb_status lvrgb_batch_autotune(lvrgb_batch b, int32_t* bucket, int32_t* seed_radius, void* stream) {
    return guarded([&] {
        require(b != nullptr, LVRGB_ERR_INVALID_ARGUMENT, "batch is NULL");
        DeviceScope dev(b->device);
        cudaStream_t caller = as_stream(stream);
        // Staged search, each candidate running the whole pipeline twice (the
        // second run timed): LBVH bucket size and seed radius, then the
        // one-warp-per-query kernel's queries per warp tile, then its key
        // buffer size (in units of k).
        auto timed_run = [&]() {
            float t = 0;
            for (int rep = 0; rep < 2; rep++) {
                on_batch_stream(b, caller, [&] { batch_run_eager(b, true); });
                batch_check(b);
                LVRGB_CUDA(cudaEventElapsedTime(&t, b->ev[0], b->ev[3]));
            }
            return t;
        };
        const int cands[4][2] = {{32, 1}, {32, 2}, {16, 1}, {16, 2}};
        float best = 1e30f;
        int bb = b->cfg.bucket, br = b->cfg.seed_radius;
        for (const auto& c : cands) {
            b->cfg.bucket = c[0];
            b->cfg.seed_radius = c[1];
            const float t = timed_run();
            if (t < best) {
                best = t;
                bb = c[0];
                br = c[1];
            }
        }
        b->cfg.bucket = bb;
        b->cfg.seed_radius = br;
        choose_collapse(b);
        best = 1e30f;
        int bt = 0;
        for (int tile : {0, 4, 16, 32}) {
            b->wide_tile = tile;
            const float t = timed_run();
            if (t < best) {
                best = t;
                bt = tile;
            }
        }
        b->wide_tile = bt;
        best = 1e30f;
        int bs = 2;
        for (int slack : {2, 3, 4}) {
            b->wide_slack = slack;
            const float t = timed_run();
            if (t < best) {
                best = t;
                bs = slack;
            }
        }
        b->wide_slack = bs;
        if (b->exec) {
            cudaGraphExecDestroy(b->exec);
            b->exec = nullptr;
        }
        on_batch_stream(b, caller, [&] { batch_run_eager(b, false); });
        batch_check(b);
        if (bucket) *bucket = bb;
        if (seed_radius) *seed_radius = br;
    });
}

lvrgb_status lvrgb_batch_tuning(lvrgb_batch b, int32_t out[4]) {
    return guarded([&] {
        require(b != nullptr && out != nullptr, LVRGB_ERR_INVALID_ARGUMENT, "NULL argument");
        out[0] = b->cfg.bucket;
        out[1] = b->cfg.seed_radius;
        out[2] = b->wide_tile;
        out[3] = b->wide_slack;
    });
}

lvrgb_status lvrgb_batch_round_times(lvrgb_batch b, float ms[5]) {
    return guarded([&] {
        require(b != nullptr && ms != nullptr, LVRGB_ERR_INVALID_ARGUMENT, "NULL argument");
        DeviceScope dev(b->device);
        for (int i = 0; i < 5; i++) ms[i] = 0.0f;
        if (!b->rounds_timed) return;
        LVRGB_CUDA(cudaEventSynchronize(b->round_ev[5]));
        for (int i = 0; i < 5; i++) LVRGB_CUDA(cudaEventElapsedTime(&ms[i], b->round_ev[i], b->round_ev[i + 1]));
    });
}

lvrgb_status lvrgb_batch_stats(lvrgb_batch b, uint32_t counters[16], float ms[4]) {
    return guarded([&] {
        require(b != nullptr, LVRGB_ERR_INVALID_ARGUMENT, "batch is NULL");
        DeviceScope dev(b->device);
        if (counters) LVRGB_CUDA(cudaMemcpy(counters, b->d_stats, kNormalStats * sizeof(uint32_t), cudaMemcpyDeviceToHost));
        if (ms)
            for (int i = 0; i < 4; i++) ms[i] = b->ms[i];
    });
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Allocation-free kNN for small point sets (lvrgb_knn_small_noalloc).
//
// Some callers must not allocate device memory during a call: code running
// inside a real-time loop or a driver callback where cudaMalloc/cudaFree would
// synchronize the device and stall other work, hosts that hand a library a
// fixed device-memory budget up front, and plugins whose host process owns
// every allocation.  For them this entry point takes its scratch (sorted
// points, tree, sort buffers, packed queries) from one file-scope device
// array of kNoAllocBytes that every GPU loading this library reserves until
// the process exits.  Its device address is looked up once per device with
// cudaGetSymbolAddress (the host-side name of a __device__ array is not a
// device address and must never be passed to a kernel).
// ---------------------------------------------------------------------------
namespace {

constexpr size_t kNoAllocBytes = size_t(8) << 20;
constexpr int64_t kNoAllocMaxPoints = 65536;
constexpr int64_t kNoAllocMaxQueries = 65536;
constexpr int kNoAllocMaxK = kSmemHeapMax;
constexpr int kNoAllocBucket = 32;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

constexpr int kMaxDevices = 128;
std::mutex g_noalloc_mu;
unsigned char* g_noalloc_ptr[kMaxDevices] = {nullptr};

// Device address of g_noalloc_scratch on the current device (set-up on the
// first call per device).
unsigned char* noalloc_scratch() {
    int dev = 0;
    LVRGB_CUDA(cudaGetDevice(&dev));
    require(dev >= 0 && dev < kMaxDevices, LVRGB_ERR_INVALID_ARGUMENT, "device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        LVRGB_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        g_noalloc_ptr[dev] = static_cast<unsigned char*>(p);
    }
    return g_noalloc_ptr[dev];
}

struct Carver {
    unsigned char* base;
    size_t off = 0;
    template <typename T>
    T* take(size_t count) {
        T* p = reinterpret_cast<T*>(base + off);
        off += (count * sizeof(T) + 255) & ~size_t(255);
        if (off > kNoAllocBytes) throw ApiError{LVRGB_ERR_OUT_OF_MEMORY, "allocation-free scratch exhausted"};
        return p;
    }
};


}  // namespace

extern "C" {

lvrgb_status lvrgb_knn_small_noalloc(const float* points, int64_t n, const float* queries, int64_t nq, int32_t k,
                                     uint32_t* idx, float* dist, void* stream) {
    return guarded([&] {
        require(n >= 1 && n <= kNoAllocMaxPoints, LVRGB_ERR_INVALID_ARGUMENT,
                "lvrgb_knn_small_noalloc: point count must be in 1..65536");
        require(nq >= 0 && nq <= kNoAllocMaxQueries, LVRGB_ERR_INVALID_ARGUMENT,
                "lvrgb_knn_small_noalloc: query count must be in 0..65536");
        require(k >= 1 && k <= kNoAllocMaxK, LVRGB_ERR_INVALID_ARGUMENT,
                "lvrgb_knn_small_noalloc: k must be in 1..96");
        require(points && (nq == 0 || (queries && idx && dist)), LVRGB_ERR_INVALID_ARGUMENT,
                "lvrgb_knn_small_noalloc: NULL array");
        cudaStream_t st = as_stream(stream);
        Carver C{noalloc_scratch()};
        const int np = int(n), nb = (np + kNoAllocBucket - 1) / kNoAllocBucket;
        LbvhBuffers B;
        B.pts = C.take<float4>(size_t(np));
        B.inv = C.take<uint32_t>(size_t(np));
        B.nodes = C.take<TreeNode>(size_t(nb > 1 ? nb - 1 : 1));
        B.bkeys = C.take<uint64_t>(size_t(nb));
        B.bparent = C.take<int>(size_t(nb));
        B.counters = C.take<int>(size_t(nb > 1 ? nb - 1 : 1));
        B.codes = C.take<uint64_t>(size_t(np));
        B.codes2 = C.take<uint64_t>(size_t(np));
        B.idx = C.take<uint32_t>(size_t(np));
        B.idx2 = C.take<uint32_t>(size_t(np));
        B.sort_tmp = C.take<unsigned char>(radix_sort_temp_bytes<uint64_t>(size_t(np)));
        B.box_tmp = C.take<unsigned char>(bbox_temp_bytes(size_t(np)));
        B.box = C.take<float>(8);
        B.err = C.take<int>(4);
        float4* qs = C.take<float4>(size_t(nq > 0 ? nq : 1));
        int* first_bad = C.take<int>(1);
        // The array keeps the previous call's contents: clear what must start
        // at zero (the error word) and reset the non-finite marker to "none"
        // (bytes 0x7f: 0x7f7f7f7f is above every point index allowed here).
        LVRGB_CUDA(cudaMemsetAsync(B.err, 0, 4 * sizeof(int), st));
        LVRGB_CUDA(cudaMemsetAsync(first_bad, 0x7f, sizeof(int), st));
        // A NaN or infinite coordinate breaks the tree's ordering, as in
        // lvrgb_surface_create: find the first such point.  The build below only
        // does arithmetic on the coordinates, so it runs before the check is read.
        first_nonfinite_kernel<<<ceil_div(np, 256), 256, 0, st>>>(points, np, first_bad);
        LVRGB_LAUNCH_CHECK();
        Lbvh T;
        lbvh_build_into(points, np, kNoAllocBucket, B, T, st);
        // Morton frame of the tree for the search seeds (one 24-byte read of
        // the box), read in the same synchronization as the non-finite marker.
        float h[6];
        int bad = 0;
        LVRGB_CUDA(cudaMemcpyAsync(h, B.box, sizeof(h), cudaMemcpyDeviceToHost, st));
        LVRGB_CUDA(cudaMemcpyAsync(&bad, first_bad, sizeof(int), cudaMemcpyDeviceToHost, st));
        LVRGB_CUDA(cudaStreamSynchronize(st));
        if (bad != 0x7f7f7f7f)
            throw ApiError{LVRGB_ERR_INVALID_ARGUMENT,
                           "lvrgb_knn_small_noalloc: point " + std::to_string(bad) + " has a non-finite coordinate"};
        const float ext = std::max(std::max(h[3] - h[0], h[4] - h[1]), h[5] - h[2]);
        for (int a = 0; a < 3; a++) T.mn[a] = h[a];
        T.scale = morton_scale(ext);
        T.seed_radius = 1;
        if (nq == 0) return;
        pack_queries_kernel<<<ceil_div(nq, 256), 256, 0, st>>>(queries, int(nq), qs);
        LVRGB_LAUNCH_CHECK();
        knn_rows_smem(T, qs, int(nq), k, idx, dist, nullptr, B.err, st);
        int herr = 0;
        LVRGB_CUDA(cudaMemcpyAsync(&herr, B.err, sizeof(int), cudaMemcpyDeviceToHost, st));
        LVRGB_CUDA(cudaStreamSynchronize(st));
        require(herr == 0, LVRGB_ERR_KERNEL, "kNN traversal reported an internal limit");
    });
}

const char* lvrgb_last_error(void) { return g_last_error.c_str(); }

const char* lvrgb_version(void) { return "lvr2_gb300 0.1 (sm_103a)"; }

}  // extern "C"
