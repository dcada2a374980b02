// kb_runtime.h -- host-side helpers shared by the runtime translation units:
// an owning device buffer and the small state-setting launchers.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>

#include <atomic>
#include <string>
#include <utility>

#include "../../include/krabgpu.h"
#include "kb_common.h"

namespace kb {

// Device allocations and frees made by the library (every one goes through
// DevBuf), for kb_debug_allocation_counts.
extern std::atomic<unsigned long long> g_dev_allocs, g_dev_frees;
// Allocation-failure injection (kb_debug_fail_allocations): while positive,
// each device allocation fails as if the device were out of memory, without
// calling cudaMalloc, and takes one off the count.
extern std::atomic<long long> g_fail_allocs;

template <typename T>
struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { release(); }
    cudaError_t alloc(size_t count) {
        release();
        if (count == 0) return cudaSuccess;
        if (g_fail_allocs.load(std::memory_order_relaxed) > 0 &&
            g_fail_allocs.fetch_sub(1, std::memory_order_relaxed) > 0)
            return cudaErrorMemoryAllocation;
        g_dev_allocs.fetch_add(1, std::memory_order_relaxed);
        cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&p), count * sizeof(T));
        if (e != cudaSuccess) {
            p = nullptr;
            cudaGetLastError();
            return e;
        }
        n = count;
        return cudaSuccess;
    }
    void release() {
        if (p) {
            g_dev_frees.fetch_add(1, std::memory_order_relaxed);
            cudaFree(p);
        }
        p = nullptr;
        n = 0;
    }
    void swap(DevBuf& o) {
        std::swap(p, o.p);
        std::swap(n, o.n);
    }
};

// Record a failure message for kb_last_error() and return the code.
kb_status fail(kb_status code, const std::string& msg);
kb_status cuda_fail(cudaError_t e, const char* what);
// The status of the exception being handled, for the catch block of an entry
// point: host allocation failures are KB_ERR_OOM, anything else KB_ERR_STATE,
// and no exception crosses the C ABI.
kb_status exception_status() noexcept;

// Stream-ordered writes of small device state (values travel as kernel
// arguments, so no host staging buffer has to outlive the call).
cudaError_t launch_set_rep(Rep* dst, const Rep& v, cudaStream_t s);
cudaError_t launch_set_u64(unsigned long long* dst, unsigned long long v, cudaStream_t s);
cudaError_t launch_add_u64(unsigned long long* dst, unsigned long long v, cudaStream_t s);

}  // namespace kb
