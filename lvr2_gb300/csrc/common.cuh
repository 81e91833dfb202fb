// common.cuh -- shared device helpers for the lvr2 GB300 reconstruction path.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <cfloat>
#include <cstdio>

namespace lvrgb {

// Host-side status plumbing: every CUDA call in the library goes through
// LVRGB_CUDA so that the C ABI can turn a failure into a status code.
struct CudaError {
    cudaError_t err;
    const char* file;
    int line;
};

#define LVRGB_CUDA(call)                                                  \
    do {                                                                  \
        cudaError_t _e = (call);                                          \
        if (_e != cudaSuccess) throw ::lvrgb::CudaError{_e, __FILE__, __LINE__}; \
    } while (0)

// Counts the kernels this library launches (lvrgb_kernel_launches) and turns
// a launch failure into a CudaError.  Written after every launch.
void count_launch();
#define LVRGB_LAUNCH_CHECK()               \
    do {                                   \
        ::lvrgb::count_launch();           \
        LVRGB_CUDA(cudaGetLastError());    \
    } while (0)

constexpr int kWarp = 32;
constexpr unsigned kFull = 0xffffffffu;

// Sentinel heap key: squared distance +inf, index 0xffffffff.  Any real
// candidate key compares below it.
constexpr unsigned long long kKeyEmpty = 0x7f800000ffffffffull;

__device__ __forceinline__ unsigned long long make_key(float d2, uint32_t idx) {
    return (static_cast<unsigned long long>(__float_as_uint(d2)) << 32) | idx;
}
__device__ __forceinline__ float key_d2(unsigned long long k) {
    return __uint_as_float(static_cast<uint32_t>(k >> 32));
}
__device__ __forceinline__ uint32_t key_idx(unsigned long long k) {
    return static_cast<uint32_t>(k & 0xffffffffu);
}

// Squared distance with a fixed operation order and no contraction:
// fl(fl(fl(dx*dx) + fl(dy*dy)) + fl(dz*dz)), dx = fl(qx - px).  The CPU
// oracle evaluates the same expression, so neighbour sets match bit for bit.
__device__ __forceinline__ float dist2(float qx, float qy, float qz, float px, float py, float pz) {
    float dx = __fsub_rn(qx, px);
    float dy = __fsub_rn(qy, py);
    float dz = __fsub_rn(qz, pz);
    return __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
}

// Squared distance from q to an axis-aligned box, evaluated with the same
// monotone operations as dist2: it never exceeds dist2 of a point inside the
// box, so pruning with it is exact.
__device__ __forceinline__ float box_dist2(float qx, float qy, float qz, float lx, float ly, float lz,
                                           float hx, float hy, float hz) {
    float dx = fmaxf(fmaxf(__fsub_rn(lx, qx), __fsub_rn(qx, hx)), 0.0f);
    float dy = fmaxf(fmaxf(__fsub_rn(ly, qy), __fsub_rn(qy, hy)), 0.0f);
    float dz = fmaxf(fmaxf(__fsub_rn(lz, qz), __fsub_rn(qz, hz)), 0.0f);
    return __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
}

// 3-D Morton spread/compact of up to 21 bits per axis (lattice keys use 20,
// the point LBVH 21).
__host__ __device__ __forceinline__ uint64_t spread20(uint64_t v) {
    v &= 0x1fffffull;
    v = (v | (v << 32)) & 0x1f00000000ffffull;
    v = (v | (v << 16)) & 0x1f0000ff0000ffull;
    v = (v | (v << 8)) & 0x100f00f00f00f00full;
    v = (v | (v << 4)) & 0x10c30c30c30c30c3ull;
    v = (v | (v << 2)) & 0x1249249249249249ull;
    return v;
}
__host__ __device__ __forceinline__ uint32_t compact20(uint64_t v) {
    v &= 0x1249249249249249ull;
    v = (v ^ (v >> 2)) & 0x10c30c30c30c30c3ull;
    v = (v ^ (v >> 4)) & 0x100f00f00f00f00full;
    v = (v ^ (v >> 8)) & 0x1f0000ff0000ffull;
    v = (v ^ (v >> 16)) & 0x1f00000000ffffull;
    v = (v ^ (v >> 32)) & 0x1fffffull;
    return static_cast<uint32_t>(v);
}
// 60-bit lattice key from three 20-bit non-negative coordinates.
__host__ __device__ __forceinline__ uint64_t lattice_key(uint32_t x, uint32_t y, uint32_t z) {
    return spread20(x) | (spread20(y) << 1) | (spread20(z) << 2);
}
__host__ __device__ __forceinline__ void lattice_decode(uint64_t k, uint32_t& x, uint32_t& y, uint32_t& z) {
    x = compact20(k);
    y = compact20(k >> 1);
    z = compact20(k >> 2);
}

__host__ __device__ inline int ceil_div(long long a, long long b) { return static_cast<int>((a + b - 1) / b); }

}  // namespace lvrgb
