// kb_noalloc.cu -- kb_field_neighbor_digest_noalloc: the per-query neighbour
// count + digest of kb_field_neighbor_digest with its staging buffers (query
// points in, counts and digests out) in one fixed device array of this
// translation unit instead of buffers allocated per call.
//
// Who needs it: a host that cannot allocate device memory at the moment it
// asks for digests.  Two kinds of caller are meant.  (1) A host that has
// committed the rest of the device's memory to its own pools: a per-call
// cudaMalloc of the staging buffers would fail mid-run.  (2) A host that
// queries between steps while other streams on the device are busy:
// cudaFree synchronises the whole device, so freeing the per-call buffers
// stalls that other work.  This entry point makes no cudaMalloc, cudaFree or
// other allocating call (torch's allocator included); it stages through the
// array below and copies the results to the caller's host buffers.
//
// Limits and sharing:
//   * at most KB_NOALLOC_MAX_QUERIES query points per call (larger requests
//     are refused with KB_ERR_ARG; split them);
//   * the array exists once per device and every call on that device uses
//     it; it keeps the last call's contents.  Each call writes every slot it
//     reads back (the query kernel stores a count and a digest for each of
//     its nq points), so nothing has to start at zero;
//   * calls whose GPU work overlaps race on the array: two host threads
//     calling it for fields on the same device, or any caller that issues
//     other work into the array.  A single call is ordered on its field's
//     stream and returns after its results are on the host;
//   * the first call on a device runs the set-up for that device (it takes
//     the array's device address with cudaGetSymbolAddress, which may load
//     this module onto the device).  Make that first call before any stream
//     capture on the device.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../include/krabgpu.h"
#include "kb_common.h"
#include "kb_launch.h"
#include "kb_runtime.h"

namespace kb {

// Defined in kb_api.cpp: the field's device, and its read buffer as query
// arguments (materialising the read buffer first; the device must be current).
int field_device(const kb_field* f);
kb_status field_query_view(kb_field* f, int32_t kind, float dist, QueryArgs* a, cudaStream_t* s);

namespace {

// Per query point: float2 in, u32 count out, u32 digest out (16 bytes).
constexpr size_t NA_MAX = KB_NOALLOC_MAX_QUERIES;
constexpr size_t NA_OFF_Q = 0;
constexpr size_t NA_OFF_COUNTS = NA_OFF_Q + NA_MAX * sizeof(float2);
constexpr size_t NA_OFF_DIGEST = NA_OFF_COUNTS + NA_MAX * sizeof(uint32_t);
constexpr size_t NA_BYTES = NA_OFF_DIGEST + NA_MAX * sizeof(uint32_t);
static_assert(NA_BYTES == 16u * NA_MAX, "staging layout");

static __device__ __align__(256) unsigned char g_noalloc_scratch[NA_BYTES];

constexpr int NA_MAX_DEVICES = 64;
std::mutex g_setup_mu;
unsigned char* g_scratch_ptr[NA_MAX_DEVICES] = {};

// Once per device, with that device current: the array's device address.
kb_status scratch_for_device(int dev, unsigned char** out) {
    if (dev < 0 || dev >= NA_MAX_DEVICES) return fail(KB_ERR_ARG, "device index out of range");
    std::lock_guard<std::mutex> lk(g_setup_mu);
    if (!g_scratch_ptr[dev]) {
        void* ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return cuda_fail(e, "cudaGetSymbolAddress(no-alloc staging array)");
        }
        if (!ptr) return fail(KB_ERR_CUDA, "cudaGetSymbolAddress returned a null address");
        g_scratch_ptr[dev] = static_cast<unsigned char*>(ptr);
    }
    *out = g_scratch_ptr[dev];
    return KB_OK;
}

struct DevicePin {
    int prev = -1;
    cudaError_t err = cudaSuccess;
    explicit DevicePin(int dev) {
        err = cudaGetDevice(&prev);
        if (err == cudaSuccess && prev != dev) err = cudaSetDevice(dev);
    }
    ~DevicePin() {
        int now = -1;
        if (cudaGetDevice(&now) == cudaSuccess && prev >= 0 && now != prev) cudaSetDevice(prev);
    }
};

#define NA_CUDA(call)                                        \
    do {                                                     \
        cudaError_t e_ = (call);                             \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call);  \
    } while (0)

}  // namespace
}  // namespace kb

using namespace kb;

extern "C" kb_status kb_field_neighbor_digest_noalloc(kb_field* f, int32_t kind, float dist,
                                                      size_t nq, const float* qxy,
                                                      uint32_t* counts, uint32_t* digest) try {
    if (!f || (nq && (!qxy || !counts || !digest))) return fail(KB_ERR_ARG, "null argument");
    if (kind != KB_QUERY_RELAX && kind != KB_QUERY_EXACT) return fail(KB_ERR_ARG, "bad query kind");
    if (nq > NA_MAX)
        return fail(KB_ERR_ARG, "kb_field_neighbor_digest_noalloc: " + std::to_string(nq) +
                                    " query points exceed its fixed staging array of " +
                                    std::to_string(NA_MAX) + "; split the request");
    DevicePin pin(field_device(f));
    if (pin.err != cudaSuccess) return cuda_fail(pin.err, "selecting the field's device");
    unsigned char* scratch = nullptr;
    if (kb_status st = scratch_for_device(field_device(f), &scratch)) return st;
    QueryArgs a{};
    cudaStream_t s = nullptr;
    if (kb_status st = field_query_view(f, kind, dist, &a, &s)) return st;
    if (nq == 0) return KB_OK;
    float2* dq = reinterpret_cast<float2*>(scratch + NA_OFF_Q);
    uint32_t* dcounts = reinterpret_cast<uint32_t*>(scratch + NA_OFF_COUNTS);
    uint32_t* ddig = reinterpret_cast<uint32_t*>(scratch + NA_OFF_DIGEST);
    const uint32_t n = (uint32_t)nq;
    NA_CUDA(cudaMemcpyAsync(dq, qxy, sizeof(float2) * n, cudaMemcpyHostToDevice, s));
    a.nq = n;
    a.q = dq;
    a.counts = dcounts;
    a.digest = ddig;
    a.offsets = nullptr;
    a.out_ids = nullptr;
    a.out_st = nullptr;
    a.cap = 0;
    NA_CUDA(launch_query(a, s));
    NA_CUDA(cudaMemcpyAsync(counts, dcounts, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost, s));
    NA_CUDA(cudaMemcpyAsync(digest, ddig, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost, s));
    NA_CUDA(cudaStreamSynchronize(s));
    return KB_OK;
} catch (...) {
    return exception_status();
}
