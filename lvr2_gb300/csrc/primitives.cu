// primitives.cu -- scan, LSD radix sort (warp match/ballot ranking), bbox
// reduction and selection helpers.
#include "primitives.cuh"

namespace lvrgb {

namespace {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;  // 2048

__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t t = __shfl_up_sync(kFull, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

// Block-wide exclusive scan of one value per thread (256 threads).
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t& total) {
    __shared__ uint32_t s_warp[kScanThreads / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t incl = warp_incl_scan(v);
    if (lane == 31) s_warp[w] = incl;
    __syncthreads();
    if (w == 0) {
        uint32_t x = lane < kScanThreads / 32 ? s_warp[lane] : 0;
        uint32_t xi = warp_incl_scan(x);
        if (lane < kScanThreads / 32) s_warp[lane] = xi - x;
        total = __shfl_sync(kFull, xi, kScanThreads / 32 - 1);
    }
    __syncthreads();
    uint32_t r = s_warp[w] + incl - v;
    __syncthreads();
    return r;
}

__global__ void scan_reduce_kernel(const uint32_t* __restrict__ in, size_t n, uint32_t* __restrict__ sums) {
    size_t base = size_t(blockIdx.x) * kScanTile;
    uint32_t acc = 0;
#pragma unroll
    for (int r = 0; r < kScanItems; r++) {
        size_t i = base + size_t(r) * kScanThreads + threadIdx.x;
        if (i < n) acc += in[i];
    }
    // block reduce
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(kFull, acc, o);
    __shared__ uint32_t s[kScanThreads / 32];
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t = 0;
        for (int w = 0; w < kScanThreads / 32; w++) t += s[w];
        sums[blockIdx.x] = t;
    }
}

__global__ void scan_apply_kernel(const uint32_t* in, uint32_t* out, size_t n,
                                  const uint32_t* __restrict__ offsets, uint32_t* d_total) {
    size_t base = size_t(blockIdx.x) * kScanTile + size_t(threadIdx.x) * kScanItems;
    uint32_t v[kScanItems];
    uint32_t local = 0;
#pragma unroll
    for (int j = 0; j < kScanItems; j++) {
        v[j] = (base + j < n) ? in[base + j] : 0u;
        local += v[j];
    }
    uint32_t total;
    uint32_t ex = block_excl_scan(local, total);
    uint32_t off = (offsets ? offsets[blockIdx.x] : 0u) + ex;
#pragma unroll
    for (int j = 0; j < kScanItems; j++) {
        if (base + j < n) out[base + j] = off;
        off += v[j];
    }
    if (d_total && blockIdx.x == gridDim.x - 1 && threadIdx.x == kScanThreads - 1) *d_total = off;
}

}  // namespace

size_t scan_temp_bytes(size_t n) {
    size_t bytes = 0;
    while (n > size_t(kScanTile)) {
        size_t nb = (n + kScanTile - 1) / kScanTile;
        bytes += ((nb * sizeof(uint32_t) + 255) / 256) * 256;
        n = nb;
    }
    return bytes + 256;
}

void exclusive_scan_u32(const uint32_t* in, uint32_t* out, size_t n, void* temp, uint32_t* d_total,
                        cudaStream_t s) {
    if (n == 0) {
        if (d_total) LVRGB_CUDA(cudaMemsetAsync(d_total, 0, sizeof(uint32_t), s));
        return;
    }
    size_t nb = (n + kScanTile - 1) / kScanTile;
    if (nb == 1) {
        scan_apply_kernel<<<1, kScanThreads, 0, s>>>(in, out, n, nullptr, d_total);
        LVRGB_LAUNCH_CHECK();
        return;
    }
    uint32_t* sums = static_cast<uint32_t*>(temp);
    void* rest = static_cast<char*>(temp) + ((nb * sizeof(uint32_t) + 255) / 256) * 256;
    scan_reduce_kernel<<<unsigned(nb), kScanThreads, 0, s>>>(in, n, sums);
    LVRGB_LAUNCH_CHECK();
    exclusive_scan_u32(sums, sums, nb, rest, nullptr, s);
    scan_apply_kernel<<<unsigned(nb), kScanThreads, 0, s>>>(in, out, n, sums, d_total);
    LVRGB_LAUNCH_CHECK();
}

// ---------------------------------------------------------------------------
// Radix sort.  One pass = histogram kernel, exclusive scan of the
// digit-major count matrix, and a stable scatter.  Within a tile the rank of
// an item among equal digits comes from __match_any_sync per 32-item warp
// round plus running per-warp counters, so no item order is lost.
// ---------------------------------------------------------------------------
namespace {

constexpr int kSortThreads = 256;
constexpr int kSortWarps = kSortThreads / 32;
constexpr int kSortItems = 16;
constexpr int kSortTile = kSortThreads * kSortItems;  // 4096
constexpr int kRadixBits = 8;
constexpr int kRadix = 1 << kRadixBits;

template <typename K>
__global__ void __launch_bounds__(kSortThreads) radix_hist_kernel(const K* __restrict__ keys, size_t n,
                                                                  int shift, uint32_t mask,
                                                                  uint32_t* __restrict__ counts,
                                                                  int ntiles) {
    // one sub-histogram per warp: shared atomics without cross-warp contention
    __shared__ uint32_t h[kSortWarps][kRadix];
#pragma unroll
    for (int j = 0; j < kSortWarps; j++) h[j][threadIdx.x] = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const size_t base = size_t(blockIdx.x) * kSortTile + size_t(w) * (kSortTile / kSortWarps);
#pragma unroll 4
    for (int r = 0; r < kSortItems; r++) {
        const size_t i = base + size_t(r) * 32 + lane;
        if (i < n) atomicAdd(&h[w][uint32_t(keys[i] >> shift) & mask], 1u);
    }
    __syncthreads();
    uint32_t c = 0;
#pragma unroll
    for (int j = 0; j < kSortWarps; j++) c += h[j][threadIdx.x];
    counts[size_t(threadIdx.x) * ntiles + blockIdx.x] = c;
}

// Dynamic shared memory of radix_scatter_kernel<K>.
template <typename K>
constexpr size_t scatter_smem_bytes() {
    return size_t(kSortWarps + 2) * kRadix * sizeof(uint32_t) + size_t(kSortTile) * (sizeof(K) + sizeof(uint32_t));
}

// Stable scatter of one tile: items are ranked within the tile by digit
// (warp rounds of __match_any_sync keep their order), placed in shared memory
// in digit order, and then written out so that each digit's run goes to
// consecutive global addresses (coalesced stores).
template <typename K, bool kVals>
__global__ void __launch_bounds__(kSortThreads) radix_scatter_kernel(
    const K* __restrict__ kin, const uint32_t* __restrict__ vin, K* __restrict__ kout,
    uint32_t* __restrict__ vout, size_t n, int shift, uint32_t mask, const uint32_t* __restrict__ offsets,
    int ntiles) {
    extern __shared__ __align__(16) unsigned char sm[];
    uint32_t(*s_cnt)[kRadix] = reinterpret_cast<uint32_t(*)[kRadix]>(sm);
    uint32_t* s_goff = reinterpret_cast<uint32_t*>(sm) + kSortWarps * kRadix;
    uint32_t* s_toff = s_goff + kRadix;
    K* s_key = reinterpret_cast<K*>(sm + size_t(kSortWarps + 2) * kRadix * sizeof(uint32_t));
    uint32_t* s_val = reinterpret_cast<uint32_t*>(s_key + kSortTile);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int j = 0; j < kSortWarps; j++) s_cnt[j][threadIdx.x] = 0;
    s_goff[threadIdx.x] = offsets[size_t(threadIdx.x) * ntiles + blockIdx.x];
    __syncthreads();

    const unsigned lt = (1u << lane) - 1u;
    const size_t tile0 = size_t(blockIdx.x) * kSortTile;
    const size_t base = tile0 + size_t(w) * (kSortTile / kSortWarps);
    K key[kSortItems];
    uint32_t val[kSortItems];
    uint32_t rank[kSortItems];
#pragma unroll
    for (int r = 0; r < kSortItems; r++) {
        size_t i = base + size_t(r) * 32 + lane;
        bool ok = i < n;
        key[r] = ok ? kin[i] : K(0);
        if (kVals) val[r] = ok ? vin[i] : 0u;
        uint32_t d = ok ? uint32_t(key[r] >> shift) & mask : 0xffffffffu;
        unsigned peers = __match_any_sync(kFull, d);
        uint32_t b = ok ? s_cnt[w][d] : 0u;
        __syncwarp();
        if (ok && lane == __ffs(peers) - 1) s_cnt[w][d] = b + __popc(peers);
        __syncwarp();
        rank[r] = b + __popc(peers & lt);
    }
    __syncthreads();
    // per digit: offsets of the warps' runs within the digit, then the
    // digit's offset within the tile (block-wide exclusive scan of totals)
    uint32_t total = 0;
#pragma unroll
    for (int j = 0; j < kSortWarps; j++) {
        const uint32_t c = s_cnt[j][threadIdx.x];
        s_cnt[j][threadIdx.x] = total;
        total += c;
    }
    {
        uint32_t incl = total;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(kFull, incl, o);
            if (lane >= o) incl += t;
        }
        __shared__ uint32_t s_warp[kSortWarps];
        if (lane == 31) s_warp[w] = incl;
        __syncthreads();
        uint32_t before = 0;
#pragma unroll
        for (int j = 0; j < kSortWarps; j++) before += j < w ? s_warp[j] : 0u;
        s_toff[threadIdx.x] = before + incl - total;
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < kSortItems; r++) {
        size_t i = base + size_t(r) * 32 + lane;
        if (i < n) {
            const uint32_t d = uint32_t(key[r] >> shift) & mask;
            const uint32_t local = s_toff[d] + s_cnt[w][d] + rank[r];
            s_key[local] = key[r];
            if (kVals) s_val[local] = val[r];
        }
    }
    __syncthreads();
    const int m = int(n - tile0 < size_t(kSortTile) ? n - tile0 : size_t(kSortTile));
    for (int i = threadIdx.x; i < m; i += kSortThreads) {
        const K k = s_key[i];
        const uint32_t d = uint32_t(k >> shift) & mask;
        const size_t dst = size_t(s_goff[d]) + size_t(i) - s_toff[d];
        kout[dst] = k;
        if (kVals) vout[dst] = s_val[i];
    }
}

}  // namespace

template <typename K>
size_t radix_sort_temp_bytes(size_t n) {
    size_t ntiles = (n + kSortTile - 1) / kSortTile;
    size_t cnt = ntiles * kRadix;
    return ((cnt * sizeof(uint32_t) + 255) / 256) * 256 + scan_temp_bytes(cnt);
}

template <typename K>
bool radix_sort_pairs(K* keys, uint32_t* vals, K* keys_alt, uint32_t* vals_alt, size_t n, int lo_bit,
                      int hi_bit, void* temp, cudaStream_t s) {
    if (n <= 1 || hi_bit <= lo_bit) return false;
    int ntiles = int((n + kSortTile - 1) / kSortTile);
    size_t cnt = size_t(ntiles) * kRadix;
    uint32_t* counts = static_cast<uint32_t*>(temp);
    void* scan_tmp = static_cast<char*>(temp) + ((cnt * sizeof(uint32_t) + 255) / 256) * 256;
    K* kin = keys;
    K* kout = keys_alt;
    uint32_t* vin = vals;
    uint32_t* vout = vals_alt;
    bool alt = false;
    {
        // more than 48 KB of dynamic shared memory needs an opt-in, once per
        // kernel and device (outside any stream capture: the first sort on a
        // device runs eagerly)
        static bool configured[256] = {};
        int dev = 0;
        LVRGB_CUDA(cudaGetDevice(&dev));
        if (dev >= 0 && dev < 256 && !configured[dev]) {
            constexpr int smem = int(scatter_smem_bytes<K>());
            LVRGB_CUDA(cudaFuncSetAttribute(radix_scatter_kernel<K, true>,
                                            cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
            LVRGB_CUDA(cudaFuncSetAttribute(radix_scatter_kernel<K, false>,
                                            cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
            configured[dev] = true;
        }
    }
    for (int shift = lo_bit; shift < hi_bit; shift += kRadixBits) {
        int bits = hi_bit - shift < kRadixBits ? hi_bit - shift : kRadixBits;
        uint32_t mask = (1u << bits) - 1u;
        radix_hist_kernel<K><<<ntiles, kSortThreads, 0, s>>>(kin, n, shift, mask, counts, ntiles);
        LVRGB_LAUNCH_CHECK();
        exclusive_scan_u32(counts, counts, cnt, scan_tmp, nullptr, s);
        constexpr size_t smem = scatter_smem_bytes<K>();
        if (vals)
            radix_scatter_kernel<K, true><<<ntiles, kSortThreads, smem, s>>>(kin, vin, kout, vout, n, shift,
                                                                             mask, counts, ntiles);
        else
            radix_scatter_kernel<K, false><<<ntiles, kSortThreads, smem, s>>>(kin, nullptr, kout, nullptr, n,
                                                                              shift, mask, counts, ntiles);
        LVRGB_LAUNCH_CHECK();
        K* tk = kin; kin = kout; kout = tk;
        uint32_t* tv = vin; vin = vout; vout = tv;
        alt = !alt;
    }
    return alt;
}

template size_t radix_sort_temp_bytes<uint32_t>(size_t);
template size_t radix_sort_temp_bytes<uint64_t>(size_t);
template bool radix_sort_pairs<uint32_t>(uint32_t*, uint32_t*, uint32_t*, uint32_t*, size_t, int, int,
                                         void*, cudaStream_t);
template bool radix_sort_pairs<uint64_t>(uint64_t*, uint32_t*, uint64_t*, uint32_t*, size_t, int, int,
                                         void*, cudaStream_t);

// ---------------------------------------------------------------------------
// Bounding box: per-block partial min/max, then one block combines them.
// ---------------------------------------------------------------------------
namespace {
constexpr int kBoxThreads = 256;
constexpr int kBoxBlocks = 1024;

__global__ void bbox_partial_kernel(const float* __restrict__ xyz, size_t n, int stride, float* part) {
    float mn[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, mx[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x) {
#pragma unroll
        for (int c = 0; c < 3; c++) {
            float v = xyz[i * stride + c];
            mn[c] = fminf(mn[c], v);
            mx[c] = fmaxf(mx[c], v);
        }
    }
#pragma unroll
    for (int c = 0; c < 3; c++) {
        for (int o = 16; o > 0; o >>= 1) {
            mn[c] = fminf(mn[c], __shfl_down_sync(kFull, mn[c], o));
            mx[c] = fmaxf(mx[c], __shfl_down_sync(kFull, mx[c], o));
        }
    }
    __shared__ float s[kBoxThreads / 32][6];
    if ((threadIdx.x & 31) == 0)
        for (int c = 0; c < 3; c++) { s[threadIdx.x >> 5][c] = mn[c]; s[threadIdx.x >> 5][3 + c] = mx[c]; }
    __syncthreads();
    if (threadIdx.x < 6) {
        float v = s[0][threadIdx.x];
        for (int w = 1; w < kBoxThreads / 32; w++)
            v = threadIdx.x < 3 ? fminf(v, s[w][threadIdx.x]) : fmaxf(v, s[w][threadIdx.x]);
        part[blockIdx.x * 6 + threadIdx.x] = v;
    }
}

__global__ void bbox_final_kernel(const float* part, int nparts, float* out) {
    int c = threadIdx.x;
    if (c >= 6) return;
    float v = part[c];
    for (int b = 1; b < nparts; b++) v = c < 3 ? fminf(v, part[b * 6 + c]) : fmaxf(v, part[b * 6 + c]);
    out[c] = v;
}
}  // namespace

size_t bbox_temp_bytes(size_t) { return kBoxBlocks * 6 * sizeof(float); }

void bbox_float3(const float* xyz, size_t n, int stride, float* out, void* temp, cudaStream_t s) {
    int nb = int((n + kBoxThreads - 1) / kBoxThreads);
    if (nb > kBoxBlocks) nb = kBoxBlocks;
    if (nb < 1) nb = 1;
    bbox_partial_kernel<<<nb, kBoxThreads, 0, s>>>(xyz, n, stride, static_cast<float*>(temp));
    LVRGB_LAUNCH_CHECK();
    bbox_final_kernel<<<1, 32, 0, s>>>(static_cast<float*>(temp), nb, out);
    LVRGB_LAUNCH_CHECK();
}

// ---------------------------------------------------------------------------
namespace {
__global__ void head_flags_kernel(const uint64_t* __restrict__ k, size_t n, uint32_t* __restrict__ f) {
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n) f[i] = (i == 0 || k[i] != k[i - 1]) ? 1u : 0u;
}
template <typename T>
__global__ void scatter_flagged_kernel(const T* __restrict__ in, const uint32_t* __restrict__ f,
                                       const uint32_t* __restrict__ pos, size_t n, T* __restrict__ out) {
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n && f[i]) out[pos[i]] = in[i];
}
__global__ void iota_kernel(uint32_t* out, size_t n) {
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n) out[i] = uint32_t(i);
}
}  // namespace

void head_flags_u64(const uint64_t* keys, size_t n, uint32_t* flags, cudaStream_t s) {
    if (!n) return;
    head_flags_kernel<<<ceil_div(n, 256), 256, 0, s>>>(keys, n, flags);
    LVRGB_LAUNCH_CHECK();
}
void scatter_flagged_u64(const uint64_t* in, const uint32_t* f, const uint32_t* pos, size_t n, uint64_t* out,
                         cudaStream_t s) {
    if (!n) return;
    scatter_flagged_kernel<uint64_t><<<ceil_div(n, 256), 256, 0, s>>>(in, f, pos, n, out);
    LVRGB_LAUNCH_CHECK();
}
void scatter_flagged_u32(const uint32_t* in, const uint32_t* f, const uint32_t* pos, size_t n, uint32_t* out,
                         cudaStream_t s) {
    if (!n) return;
    scatter_flagged_kernel<uint32_t><<<ceil_div(n, 256), 256, 0, s>>>(in, f, pos, n, out);
    LVRGB_LAUNCH_CHECK();
}
void iota_u32(uint32_t* out, size_t n, cudaStream_t s) {
    if (!n) return;
    iota_kernel<<<ceil_div(n, 256), 256, 0, s>>>(out, n);
    LVRGB_LAUNCH_CHECK();
}

}  // namespace lvrgb
