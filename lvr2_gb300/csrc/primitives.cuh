// primitives.cuh -- device-wide scan, radix sort and reductions used by the
// LBVH build and the sparse-grid build.  All of them are deterministic: the
// same input gives the same output bits on every run.
#pragma once
#include "common.cuh"

namespace lvrgb {

// ---- exclusive prefix sum of uint32 ------------------------------------
size_t scan_temp_bytes(size_t n);
// out[i] = sum_{j<i} in[j]; if d_total != nullptr it receives the sum of all.
// in and out may alias.
void exclusive_scan_u32(const uint32_t* in, uint32_t* out, size_t n, void* temp,
                        uint32_t* d_total, cudaStream_t s);

// ---- LSD radix sort of (key, value) pairs on key bits [lo_bit, hi_bit) -----
// Stable.  Ping-pongs between (keys, vals) and (keys_alt, vals_alt); returns
// true when the sorted result ends in the *_alt buffers.  vals may be null.
template <typename K>
size_t radix_sort_temp_bytes(size_t n);
template <typename K>
bool radix_sort_pairs(K* keys, uint32_t* vals, K* keys_alt, uint32_t* vals_alt, size_t n, int lo_bit,
                      int hi_bit, void* temp, cudaStream_t s);

// ---- min/max of float4 xyz (w ignored) ------------------------------------
size_t bbox_temp_bytes(size_t n);
// out[0..2] = min xyz, out[3..5] = max xyz (device pointer, 6 floats).
void bbox_float3(const float* xyz, size_t n, int stride_floats, float* out, void* temp, cudaStream_t s);

// ---- selection helpers ----------------------------------------------------
// Head flags of a sorted uint64 array (flags[i] = keys[i] != keys[i-1]).
void head_flags_u64(const uint64_t* keys, size_t n, uint32_t* flags, cudaStream_t s);
// out[pos[i]] = in[i] where flags[i] != 0, pos = exclusive scan of flags.
void scatter_flagged_u64(const uint64_t* in, const uint32_t* flags, const uint32_t* pos, size_t n,
                         uint64_t* out, cudaStream_t s);
void scatter_flagged_u32(const uint32_t* in, const uint32_t* flags, const uint32_t* pos, size_t n,
                         uint32_t* out, cudaStream_t s);
void iota_u32(uint32_t* out, size_t n, cudaStream_t s);

}  // namespace lvrgb
