// Small host-side helpers for device memory and launches.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <utility>

#include "common.cuh"

namespace gb300 {

// Owning device allocation (cudaMalloc), grown on demand, never shrunk.
template <class T>
class DeviceBuffer {
public:
    DeviceBuffer() = default;
    DeviceBuffer(const DeviceBuffer&) = delete;
    DeviceBuffer& operator=(const DeviceBuffer&) = delete;
    ~DeviceBuffer() { release(); }

    T* get() const { return ptr_; }
    size_t size() const { return count_; }

    // Ensures room for `count` elements; returns true when the allocation changed.
    bool reserve(size_t count) {
        if (count <= count_ && ptr_ != nullptr) return false;
        release();
        const size_t bytes = (count == 0 ? 1 : count) * sizeof(T);
        GB_CUDA_CHECK(cudaMalloc(reinterpret_cast<void**>(&ptr_), bytes));
        count_ = count;
        return true;
    }
    void release() {
        if (ptr_) cudaFree(ptr_);
        ptr_ = nullptr;
        count_ = 0;
    }
    void upload(const T* host, size_t count, cudaStream_t s) {
        reserve(count);
        if (count) GB_CUDA_CHECK(cudaMemcpyAsync(ptr_, host, count * sizeof(T), cudaMemcpyHostToDevice, s));
    }

private:
    T* ptr_ = nullptr;
    size_t count_ = 0;
};

struct DeviceInfo {
    int device = 0;
    int sms = 0;
    int smem_optin = 0;  // largest dynamic + static shared memory of one CTA (bytes)
    int smem_per_sm = 0;  // shared memory of one SM (bytes)
};

inline DeviceInfo current_device() {
    DeviceInfo d;
    GB_CUDA_CHECK(cudaGetDevice(&d.device));
    GB_CUDA_CHECK(cudaDeviceGetAttribute(&d.sms, cudaDevAttrMultiProcessorCount, d.device));
    GB_CUDA_CHECK(cudaDeviceGetAttribute(&d.smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, d.device));
    GB_CUDA_CHECK(cudaDeviceGetAttribute(&d.smem_per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, d.device));
    return d;
}

// Grid of `blocks_per_sm` (or the occupancy limit, whichever is smaller) blocks per SM.
template <class K>
int persistent_grid(K kernel, int threads, int sms, int want_per_sm = 64) {
    int per_sm = 0;
    GB_CUDA_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, 0));
    if (per_sm < 1) per_sm = 1;
    if (per_sm > want_per_sm) per_sm = want_per_sm;
    return per_sm * sms;
}

}  // namespace gb300
