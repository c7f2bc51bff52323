// noalloc.cu — Morton ordering for callers that cannot allocate device memory.
//
// Some callers of this library must not call cudaMalloc: code whose device memory is owned by
// another framework's allocator that has already reserved most of the GPU (a fresh cudaMalloc
// fails or fragments that pool), code that must not take the device-wide synchronisation that
// cudaMalloc/cudaFree can imply while other streams are running, and fixed-budget loops that
// must never allocate after start-up. They already own their inputs and outputs.
// gbh_morton_order_noalloc serves them: it runs the collect, Morton-key and stable radix-sort
// kernels of the tree build with every temporary taken from one file-scope device array
// (g_scratch) instead of an allocation.
//
// g_scratch holds kScratchBytes (4.5 MiB) on every GPU that loads the library, until the
// process exits, whether or not the entry point is called. It is enough for up to
// kNoAllocMaxBodies (262,144) bodies; larger calls are rejected.
//
// The host cannot use the name g_scratch as a device address (in host code it names a
// host-side stand-in), so the device address is looked up once per device, with that device
// current, by cudaGetSymbolAddress, and passed to the kernels. The looked-up address belongs to
// the device's context of that moment: a cudaDeviceReset destroys it, and the entry point must
// not be called on that device again in the same process.
//
// Each call waits for its stream before it returns (it reads the number of sorted bodies back to
// the host).
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <mutex>

#include "gbh_internal.cuh"

namespace {

constexpr int64_t kNoAllocMaxBodies = 262144;
constexpr size_t kScratchBytes = size_t(4608) << 10;  // 4.5 MiB
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

std::mutex g_setup_mu;
void *g_scratch_addr[kMaxDevices] = {};

int report(char *err, int errlen, int code, const char *msg) {
    if (err && errlen > 0) {
        std::strncpy(err, msg, size_t(errlen) - 1);
        err[errlen - 1] = 0;
    }
    return code;
}

int report_cuda(char *err, int errlen, const char *what, cudaError_t e) {
    char buf[256];
    std::snprintf(buf, sizeof buf, "%s: %s", what, cudaGetErrorString(e));
    return report(err, errlen, e == cudaErrorMemoryAllocation ? GBH_ERR_NOMEM : GBH_ERR_CUDA, buf);
}

}  // namespace

extern "C" int gbh_morton_order_noalloc(int32_t device, void *stream, int64_t n, const double *px, const double *py,
                                        const double *pz, const uint8_t *kind, const uint8_t *alive, uint64_t *keys,
                                        int32_t *order, int64_t *nstars, char *err, int errlen) {
    report(err, errlen, GBH_OK, "");
    if (n < 0) return report(err, errlen, GBH_ERR_ARG, "n < 0");
    if (n > kNoAllocMaxBodies) {
        char buf[160];
        std::snprintf(buf, sizeof buf, "n = %lld exceeds the %lld bodies the static scratch array holds",
                      static_cast<long long>(n), static_cast<long long>(kNoAllocMaxBodies));
        return report(err, errlen, GBH_ERR_ARG, buf);
    }
    if (!nstars) return report(err, errlen, GBH_ERR_ARG, "nstars is NULL");
    *nstars = 0;
    if (n > 0 && (!px || !py || !pz || !keys || !order))
        return report(err, errlen, GBH_ERR_ARG, "array argument is NULL");
    if (device < 0 || device >= kMaxDevices) return report(err, errlen, GBH_ERR_ARG, "device out of range");
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return report_cuda(err, errlen, "cudaSetDevice", e);
    void *scratch = nullptr;
    {
        // Set-up, once per device with that device current: the device address of g_scratch.
        std::lock_guard<std::mutex> lock(g_setup_mu);
        if (!g_scratch_addr[device]) {
            if (gbh::morton_sort_scratch_bytes(kNoAllocMaxBodies) > kScratchBytes)  // a build inconsistency
                return report(err, errlen, GBH_ERR_STATE,
                              "internal error: the static scratch array is smaller than its stated capacity");
            void *ptr = nullptr;
            e = cudaGetSymbolAddress(&ptr, g_scratch);
            if (e != cudaSuccess) return report_cuda(err, errlen, "cudaGetSymbolAddress", e);
            g_scratch_addr[device] = ptr;
        }
        scratch = g_scratch_addr[device];
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    int64_t launches = 0;
    gbh::Launch L{s, &launches, 0};
    gbh::DevInfo *info = nullptr;
    // morton_sort clears the DevInfo at the start of the array; every other temporary it uses is
    // written before it is read, so the previous call's leftovers need no clearing.
    e = gbh::morton_sort(L, n, px, py, pz, kind, alive, keys, order, scratch, kScratchBytes, &info);
    if (e != cudaSuccess) return report_cuda(err, errlen, "Morton ordering", e);
    gbh::DevInfo h;
    e = cudaMemcpyAsync(&h, info, sizeof h, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return report_cuda(err, errlen, "Morton ordering", e);
    if (h.err && h.err_where == gbh::kErrNonFinite)
        return report(err, errlen, GBH_ERR_ARG, "an alive star has a non-finite position (outputs are undefined)");
    if (h.err) return report(err, errlen, GBH_ERR_LIMIT, "device-side consistency check failed in the radix sort");
    *nstars = n > 0 ? h.nstars : 0;
    return GBH_OK;
}
