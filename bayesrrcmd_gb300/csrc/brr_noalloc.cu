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
// device and with that device current, cudaGetSymbolAddress gives the device
// address that is passed to the kernel.  The first call on a device performs
// that set-up, so it should come before any stream capture.  All calls share
// the one array; the kernel reads only the n entries the same call wrote, so
// nothing has to start at zero, and calls that overlap on the GPU (two
// streams, two host threads, two contexts on one device) race on it.
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

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
NoallocTerms *g_terms_addr[kMaxDevices] = {};

// Device address of the static term array on the current device, looked up
// once per device.
cudaError_t terms_address(int dev, NoallocTerms **out)
{
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_terms_addr[dev]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_terms);
        if (e != cudaSuccess)
            return e;
        g_terms_addr[dev] = static_cast<NoallocTerms *>(p);
    }
    *out = g_terms_addr[dev];
    return cudaSuccess;
}

}  // namespace

cudaError_t noalloc_xbeta(int dev, cudaStream_t st, int kind, int64_t N, const uint8_t *codes, int64_t col_stride,
                          const double *table, const uint32_t *idx, const double *b, int64_t n, double *d_out,
                          std::string &why)
{
    if (dev < 0 || dev >= kMaxDevices) {
        why = "device ordinal beyond the set-up table";
        return cudaErrorInvalidDevice;
    }
    NoallocTerms *terms = nullptr;
    cudaError_t e = terms_address(dev, &terms);
    if (e != cudaSuccess) {
        why = std::string("cudaGetSymbolAddress of the static term array failed: ") + cudaGetErrorString(e);
        return e;
    }
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
