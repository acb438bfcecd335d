// Allocation-free genetic values: brr_xbeta_noalloc.
//
// Some callers of this library cannot allocate device memory at the moment
// they need genetic values: a host runtime that has reserved the whole GPU
// with its own pool and forbids further cudaMalloc, a serving loop that
// must never block on the allocator, or code that runs between the
// phases of a chain where an allocation would synchronise the device.  For
// them this entry point computes out = sum_q b[q] * x[:, idx[q]] without any
// allocation: the (index, beta) term list is staged in a fixed, file-scope
// device array, and the caller owns the output buffer.
//
// The array holds at most BRR_NOALLOC_MAX_TERMS terms (12 bytes each,
// 768 KiB); every GPU that loads the library keeps it until the process exits.
// Host code never uses the array's name as an address: at set-up, once per
// device context and with that device current, cudaGetSymbolAddress gives the
// device address that is passed to the kernel.  The address is cached per
// CUDA context, keyed by the context's process-unique id (cuCtxGetId: the
// primary context of a device, or any other context the caller made
// current), so a context created again after cudaDeviceReset looks the
// address up again even when the driver reuses the old context's handle.  The first call on a device (or in a new
// context) performs that set-up, so it should come before any stream capture.
// All calls share the one array; the kernel reads only the n entries the same
// call wrote, so nothing has to start at zero, and calls that overlap on the
// GPU (two streams, two host threads, two contexts on one device) race on it.
// Every call is synchronous: it returns once the output is written.
//
// The output buffer is checked before the launch, without allocating: it must
// be device (or managed) memory of the context's device, with at least N
// doubles from d_out to the end of its allocation.
#include <cuda.h>
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "brr_device.cuh"
#include "brr_internal.h"

namespace brr {

struct NoallocTerms {
    uint32_t idx[BRR_NOALLOC_MAX_TERMS];
    double beta[BRR_NOALLOC_MAX_TERMS];
};

static __device__ __align__(256) NoallocTerms g_noalloc_terms;

// Variant of the residual-refresh GEMV that reads its term list from the
// static array and writes sum_q beta_q * x[i, idx_q] for four individuals per
// thread, walking the terms in the caller's order (deterministic).
__global__ void __launch_bounds__(kThreads) k_xbeta_static(int kind, int64_t N, const uint8_t *__restrict__ codes,
                                                           int64_t col_stride, const double *__restrict__ table,
                                                           const NoallocTerms *__restrict__ terms, int64_t n,
                                                           double *__restrict__ out)
{
    const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t i0 = 4 * b;
    if (i0 >= N)
        return;
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    for (int64_t q = 0; q < n; ++q) {
        const uint32_t j = terms->idx[q];
        const double bj = terms->beta[q];
        const unsigned v = codes[(int64_t)j * col_stride + b];
        double x[4];
        if (kind == BRR_KIND_DENSE) {
            const double l0 = table[4 * j], l1 = table[4 * j + 1], l2 = table[4 * j + 2], l3 = table[4 * j + 3];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const unsigned c = (v >> (2 * k)) & 3u;
                x[k] = (c & 2u) ? ((c & 1u) ? l3 : l2) : ((c & 1u) ? l1 : l0);
            }
        } else {
            const double mean = table[4 * j], sd = table[4 * j + 1];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const unsigned c = (v >> (2 * k)) & 3u;
                const double g = c == 0u ? 2.0 : (c == 2u ? 1.0 : 0.0);
                x[k] = c == 1u ? 0.0 : (g - mean) / sd;
            }
        }
#pragma unroll
        for (int k = 0; k < 4; ++k)
            acc[k] = fma(bj, x[k], acc[k]);
    }
#pragma unroll
    for (int k = 0; k < 4; ++k)
        if (i0 + k < N)
            out[i0 + k] = acc[k];
}

namespace {

constexpr int kMaxContexts = 64;
std::mutex g_setup_mutex;

// Device address of the static term array, per CUDA context: the module (and
// with it the array) is loaded once per context, so a context made anew gets
// a fresh lookup.  Contexts are told apart by their id, which the driver never
// reuses within a process (a destroyed context's handle may be reused).
struct TermsAddr {
    unsigned long long ctx_id;
    NoallocTerms *addr;
};
TermsAddr g_terms_addr[kMaxContexts] = {};
int g_n_terms_addr = 0;

typedef CUresult (*CtxGetCurrentFn)(CUcontext *);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long *);
typedef CUresult (*MemGetAddressRangeFn)(CUdeviceptr *, size_t *, CUdeviceptr);
CtxGetCurrentFn g_ctx_get_current = nullptr;
CtxGetIdFn g_ctx_get_id = nullptr;
MemGetAddressRangeFn g_mem_get_address_range = nullptr;

// Driver entry points of the three queries, through the runtime (the library
// does not link libcuda directly).  Called with g_setup_mutex held.
cudaError_t driver_entry_points(std::string &why)
{
    if (g_ctx_get_current && g_ctx_get_id && g_mem_get_address_range)
        return cudaSuccess;
    const char *names[3] = {"cuCtxGetCurrent", "cuCtxGetId", "cuMemGetAddressRange"};
    void *f[3] = {nullptr, nullptr, nullptr};
    for (int k = 0; k < 3; ++k) {
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        const cudaError_t e = cudaGetDriverEntryPointByVersion(names[k], &f[k], 12000, cudaEnableDefault, &q);
        if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !f[k]) {
            why = std::string("the driver entry point ") + names[k] + " is unavailable";
            return e != cudaSuccess ? e : cudaErrorNotSupported;
        }
    }
    g_ctx_get_current = reinterpret_cast<CtxGetCurrentFn>(f[0]);
    g_ctx_get_id = reinterpret_cast<CtxGetIdFn>(f[1]);
    g_mem_get_address_range = reinterpret_cast<MemGetAddressRangeFn>(f[2]);
    return cudaSuccess;
}

// Device address of the static term array in the current context.
cudaError_t terms_address(NoallocTerms **out, std::string &why)
{
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    cudaError_t e = driver_entry_points(why);
    if (e != cudaSuccess)
        return e;
    CUcontext cur = nullptr;
    unsigned long long id = 0;
    if (g_ctx_get_current(&cur) != CUDA_SUCCESS || !cur || g_ctx_get_id(cur, &id) != CUDA_SUCCESS) {
        why = "no current CUDA context";
        return cudaErrorInvalidDevice;
    }
    for (int k = 0; k < g_n_terms_addr; ++k)
        if (g_terms_addr[k].ctx_id == id) {
            *out = g_terms_addr[k].addr;
            return cudaSuccess;
        }
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_terms);
    if (e != cudaSuccess) {
        why = std::string("cudaGetSymbolAddress of the static term array failed: ") + cudaGetErrorString(e);
        return e;
    }
    // the table is small: past kMaxContexts contexts the oldest entry makes room
    if (g_n_terms_addr == kMaxContexts) {
        for (int k = 1; k < kMaxContexts; ++k)
            g_terms_addr[k - 1] = g_terms_addr[k];
        --g_n_terms_addr;
    }
    g_terms_addr[g_n_terms_addr++] = {id, static_cast<NoallocTerms *>(p)};
    *out = static_cast<NoallocTerms *>(p);
    return cudaSuccess;
}

}  // namespace

// Whether p is device (or managed) memory of device `dev` with at least `bytes`
// bytes from p to the end of its allocation; `name` names the argument in the
// message.  Allocates nothing and launches nothing, so a caller can refuse a
// buffer that a kernel would read or write out of bounds.
bool device_range_check(int dev, const void *p, size_t bytes, const char *name, std::string &why)
{
    cudaPointerAttributes a{};
    cudaError_t e = cudaPointerGetAttributes(&a, p);
    if (e != cudaSuccess) {
        cudaGetLastError();
        why = std::string(name) + " is not a CUDA pointer: " + cudaGetErrorString(e);
        return false;
    }
    if (a.type != cudaMemoryTypeDevice && a.type != cudaMemoryTypeManaged) {
        why = std::string(name) + " must be device or managed memory (got host or unregistered memory)";
        return false;
    }
    if (a.device != dev) {
        why = std::string(name) + " belongs to device " + std::to_string(a.device) + ", the call runs on device " +
              std::to_string(dev);
        return false;
    }
    {
        std::lock_guard<std::mutex> lock(g_setup_mutex);
        if (driver_entry_points(why) != cudaSuccess)
            return false;
    }
    CUdeviceptr base = 0;
    size_t size = 0;
    if (g_mem_get_address_range(&base, &size, (CUdeviceptr)p) != CUDA_SUCCESS) {
        why = std::string("the allocation holding ") + name + " could not be found";
        return false;
    }
    const size_t left = (size_t)(base + size - (CUdeviceptr)p);
    if (left < bytes) {
        why = std::string(name) + " has " + std::to_string(left) + " bytes to the end of its allocation; " +
              std::to_string(bytes) + " are needed";
        return false;
    }
    return true;
}

// The output of brr_xbeta_noalloc: N doubles, 8-byte aligned, in device (or
// managed) memory of device `dev`.
bool noalloc_check_output(int dev, const void *d_out, size_t bytes, std::string &why)
{
    if ((uintptr_t)d_out % alignof(double) != 0) {
        why = "d_out must be aligned to 8 bytes";
        return false;
    }
    return device_range_check(dev, d_out, bytes, "d_out", why);
}

cudaError_t noalloc_xbeta(cudaStream_t st, int kind, int64_t N, const uint8_t *codes, int64_t col_stride,
                          const double *table, const uint32_t *idx, const double *b, int64_t n, double *d_out,
                          std::string &why)
{
    NoallocTerms *terms = nullptr;
    cudaError_t e = terms_address(&terms, why);
    if (e != cudaSuccess)
        return e;
    if (n > 0) {
        e = cudaMemcpyAsync(terms->idx, idx, sizeof(uint32_t) * n, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(terms->beta, b, sizeof(double) * n, cudaMemcpyHostToDevice, st);
        if (e != cudaSuccess) {
            why = std::string("staging the term list failed: ") + cudaGetErrorString(e);
            return e;
        }
    }
    const int64_t nb = (N + 3) / 4;
    k_xbeta_static<<<(unsigned)((nb + kThreads - 1) / kThreads), kThreads, 0, st>>>(kind, N, codes, col_stride, table,
                                                                                     terms, n, d_out);
    e = cudaGetLastError();
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(st);
    if (e != cudaSuccess)
        why = std::string("the genetic-value kernel failed: ") + cudaGetErrorString(e);
    return e;
}

}  // namespace brr
