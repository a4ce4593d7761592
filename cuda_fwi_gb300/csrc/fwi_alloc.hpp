// Device memory of the library's engines, through an allocator the caller can
// replace (fwi_psv_set_device_allocator): an application's pool allocator, or
// a test's allocator that fails on purpose.  No counterpart in the reference,
// which calls cudaMalloc directly and exits when it fails
// (forward_kernel_PSV_GPU.cu:19-27).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>

#include "../../include/fwi_psv.h"

namespace fwi {

struct DeviceAllocator {
    fwi_psv_alloc_fn alloc = nullptr;  // null: cudaMalloc / cudaFree
    fwi_psv_free_fn release = nullptr;
    void* ctx = nullptr;
};

inline std::mutex g_alloc_mu;
inline DeviceAllocator g_alloc;

inline void set_device_allocator(const DeviceAllocator& a) {
    std::lock_guard<std::mutex> lk(g_alloc_mu);
    g_alloc = a;
}

// n bytes of device memory on the current device.  *used receives the
// allocator that made them (a buffer is freed through it even after the
// process-wide allocator changed).  Returns cudaSuccess, or
// cudaErrorMemoryAllocation when the allocator returned null, or
// cudaErrorMisalignedAddress when it returned a pointer not aligned to 256
// bytes (the tensor maps and the vector loads need 16; cudaMalloc gives 256).
inline cudaError_t device_alloc(void** p, size_t n, DeviceAllocator* used) {
    DeviceAllocator a;
    {
        std::lock_guard<std::mutex> lk(g_alloc_mu);
        a = g_alloc;
    }
    *used = a;
    if (!a.alloc) return cudaMalloc(p, n);
    *p = a.alloc(n, a.ctx);
    if (!*p) return cudaErrorMemoryAllocation;
    if (reinterpret_cast<uintptr_t>(*p) & 255u) {
        a.release(*p, a.ctx);
        *p = nullptr;
        return cudaErrorMisalignedAddress;
    }
    return cudaSuccess;
}

// Freed as cudaFree would: after the device has finished the work queued on
// the memory (cudaFree synchronises; a pool's release does not, and the pool
// may hand the memory to other work at once).
inline void device_free(void* p, const DeviceAllocator& a) {
    if (!p) return;
    if (a.alloc) {
        cudaDeviceSynchronize();
        a.release(p, a.ctx);
    } else {
        cudaFree(p);
    }
}

}  // namespace fwi
