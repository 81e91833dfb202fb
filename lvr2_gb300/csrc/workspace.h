// workspace.h -- grow-only named device buffers owned by a handle.
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <string>
#include <unordered_map>

#include "common.cuh"

namespace lvrgb {

// Host-side allocation fault injection (lvrgb_debug_fail_allocation): when
// the countdown reaches zero, that device allocation of a workspace fails as
// cudaErrorMemoryAllocation without calling the driver.  0 = off.
inline std::atomic<long long>& alloc_fault_countdown() {
    static std::atomic<long long> c{0};
    return c;
}
inline bool alloc_fault_due() {
    long long c = alloc_fault_countdown().load();
    while (c > 0) {
        if (alloc_fault_countdown().compare_exchange_weak(c, c - 1)) return c == 1;
    }
    return false;
}

class Workspace {
  public:
    Workspace() = default;
    Workspace(const Workspace&) = delete;
    Workspace& operator=(const Workspace&) = delete;
    ~Workspace() {
        release();
        if (pinned_) cudaFreeHost(pinned_);
    }

    // Small pinned host area for device-to-host reads of counts.
    uint64_t* pinned() {
        if (!pinned_) LVRGB_CUDA(cudaMallocHost(&pinned_, 64 * sizeof(uint64_t)));
        return pinned_;
    }

    // Returns a device buffer of at least count elements of T.  A buffer only
    // grows; growing it discards its contents.
    template <typename T>
    T* get(const std::string& name, size_t count) {
        size_t bytes = count * sizeof(T);
        if (bytes == 0) bytes = 16;
        auto& e = bufs_[name];
        if (e.bytes < bytes) {
            if (e.ptr) LVRGB_CUDA(cudaFree(e.ptr));
            e.ptr = nullptr;
            e.bytes = 0;
            size_t want = bytes + bytes / 8;  // headroom for slightly larger calls
            want = (want + 255) & ~size_t(255);
            if (alloc_fault_due()) throw CudaError{cudaErrorMemoryAllocation, __FILE__, __LINE__};
            LVRGB_CUDA(cudaMalloc(&e.ptr, want));
            e.bytes = want;
        }
        return static_cast<T*>(e.ptr);
    }
    size_t bytes_held() const {
        size_t t = 0;
        for (auto& kv : bufs_) t += kv.second.bytes;
        return t;
    }
    void release() {
        for (auto& kv : bufs_)
            if (kv.second.ptr) cudaFree(kv.second.ptr);
        bufs_.clear();
    }

  private:
    struct Entry {
        void* ptr = nullptr;
        size_t bytes = 0;
    };
    std::unordered_map<std::string, Entry> bufs_;
    uint64_t* pinned_ = nullptr;
};

}  // namespace lvrgb
