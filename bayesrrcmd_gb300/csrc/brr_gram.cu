// Marker Gram matrix G[j,k] = x_j . x_k of the standardised dense columns,
// stored as a packed lower triangle (entry (j, k), j > k, at j(j-1)/2 + k) in
// FP64.  The blocked FP32C sweep uses it to resolve several markers per grid
// round exactly: after marker p changes the residual by dBeta_p * x_p, the
// dot product of a later marker t moves by dBeta_p * G[p, t].
//
// With g the genotype (0 when missing), m the non-missing indicator, sigma and
// c the per-marker scale and column mean of the dense builder:
//   x_j . x_k = s_j s_k (P_jk - c_k Q_jk - c_j Q_kj + c_j c_k R_jk)
//   P = g_j . g_k,  Q_jk = g_j . m_k,  R = m_j . m_k
// (missing genotypes take the value (mean - colmean) * sigma, which is zero up
// to the rounding of the two means and is left out).  P, Q, R are integer
// sums below 2^24, computed exactly by BF16 GEMMs with FP32 accumulation
// (cuBLAS, a plain library GEMM) on tiles of markers; the FP64 combination runs
// in k_gram_combine.
#include <cublas_v2.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <string>

#include "brr_device.cuh"
#include "brr_internal.h"

namespace brr {

// Rows [m0, m0+mt) of the genotype matrix as BF16 (row length npad, padding
// zero), and optionally the non-missing indicator.
__global__ void k_decode_bf16(const uint8_t *__restrict__ codes, int64_t col_stride, int64_t N, int64_t npad,
                              int64_t m0, int64_t mt, __nv_bfloat16 *__restrict__ gp, __nv_bfloat16 *__restrict__ nm)
{
    const int64_t total = mt * (npad / 4);
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = e / (npad / 4);
        const int64_t b = e - r * (npad / 4);
        const unsigned v = (4 * b < N) ? codes[(m0 + r) * col_stride + b] : 0x55u;
        __nv_bfloat16 g4[4], m4[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const unsigned c = (v >> (2 * k)) & 3u;
            const bool valid = 4 * b + k < N;
            const float g = (!valid || c == 1u) ? 0.f : (c == 0u ? 2.f : (c == 2u ? 1.f : 0.f));
            g4[k] = __float2bfloat16(g);
            m4[k] = __float2bfloat16((valid && c != 1u) ? 1.f : 0.f);
        }
        const int64_t o = r * npad + 4 * b;
#pragma unroll
        for (int k = 0; k < 4; ++k)
            gp[o + k] = g4[k];
        if (nm) {
#pragma unroll
            for (int k = 0; k < 4; ++k)
                nm[o + k] = m4[k];
        }
    }
}

// Tile (rows j in [j0, j0+tj), columns k in [k0, k0+tk)) of the products, each
// stored column-major with the k index fastest: X[(j - j0) * tk + (k - k0)].
__global__ void k_gram_combine(int64_t j0, int64_t tj, int64_t k0, int64_t tk, const float *__restrict__ P,
                               const float *__restrict__ Q1, const float *__restrict__ Q2, const float *__restrict__ R,
                               const double *__restrict__ scale, const int64_t *__restrict__ counts, int64_t N,
                               double *__restrict__ G)
{
    const int64_t total = tj * tk;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t a = e / tk, b = e - a * tk;
        const int64_t j = j0 + a, k = k0 + b;
        if (k >= j)
            continue;
        const double sj = scale[2 * j], cj = scale[2 * j + 1];
        const double sk = scale[2 * k], ck = scale[2 * k + 1];
        double q1, q2, r;
        if (Q1) {
            q1 = (double)Q1[e];
            q2 = (double)Q2[e];
            r = (double)R[e];
        } else {
            q1 = (double)(counts[4 * j + 1] + 2 * counts[4 * j + 2]);
            q2 = (double)(counts[4 * k + 1] + 2 * counts[4 * k + 2]);
            r = (double)N;
        }
        const double inner = (((double)P[e] - ck * q1) - cj * q2) + (cj * ck) * r;
        G[j * (j - 1) / 2 + k] = (sj * sk) * inner;
    }
}

cudaError_t gram_bytes_needed(int64_t N, int64_t M, bool missing, size_t *gram, size_t *work)
{
    const int64_t npad = ((N + 7) / 8) * 8;
    const int64_t T = std::min<int64_t>(M, 8192);
    *gram = (size_t)(M * (M - 1) / 2) * sizeof(double);
    *work = (size_t)M * npad * 2 * (missing ? 2 : 1) + (size_t)T * T * 4 * (missing ? 4 : 1);
    return cudaSuccess;
}

int build_gram(const uint8_t *codes, int64_t col_stride, int64_t N, int64_t M, const double *scale,
               const int64_t *counts, bool missing, double *G, cudaStream_t st, std::string &why, float *device_ms)
{
    const int64_t npad = ((N + 7) / 8) * 8;
    const int64_t T = std::min<int64_t>(M, 8192);
    __nv_bfloat16 *gp = nullptr, *nm = nullptr;
    float *tiles = nullptr;
    cublasHandle_t h = nullptr;
    int rc = 0;
    auto cu = [&](cudaError_t e, const char *what) {
        if (e != cudaSuccess && rc == 0) {
            why = std::string(what) + ": " + cudaGetErrorString(e);
            rc = -1;
        }
    };
    cu(cudaMalloc(&gp, sizeof(__nv_bfloat16) * (size_t)M * npad), "allocation of the BF16 genotypes");
    if (missing)
        cu(cudaMalloc(&nm, sizeof(__nv_bfloat16) * (size_t)M * npad), "allocation of the indicators");
    cu(cudaMalloc(&tiles, sizeof(float) * (size_t)T * T * (missing ? 4 : 1)), "allocation of the product tiles");
    if (rc == 0 && cublasCreate(&h) != CUBLAS_STATUS_SUCCESS) {
        why = "cublasCreate failed";
        rc = -1;
    }
    if (rc == 0)
        cublasSetStream(h, st);
    cudaEvent_t ev[2] = {nullptr, nullptr};
    if (rc == 0) {
        cu(cudaEventCreate(&ev[0]), "event");
        cu(cudaEventCreate(&ev[1]), "event");
    }
    if (rc == 0)
        cu(cudaEventRecord(ev[0], st), "event");
    if (rc == 0) {
        k_decode_bf16<<<152 * 8, 256, 0, st>>>(codes, col_stride, N, npad, 0, M, gp, nm);
        cu(cudaGetLastError(), "decode");
    }
    const float one = 1.f, zero = 0.f;
    float *P = tiles, *Q1 = missing ? tiles + (size_t)T * T : nullptr, *Q2 = missing ? tiles + 2 * (size_t)T * T : nullptr,
          *R = missing ? tiles + 3 * (size_t)T * T : nullptr;
    // out (tk x tj, column-major, k fastest) = A(rows k) * B(rows j)^T over the N axis
    auto gemm = [&](const __nv_bfloat16 *A, const __nv_bfloat16 *B, int64_t k0, int64_t tk, int64_t j0, int64_t tj,
                    float *out) {
        if (rc)
            return;
        const cublasStatus_t s =
            cublasGemmEx(h, CUBLAS_OP_T, CUBLAS_OP_N, (int)tk, (int)tj, (int)npad, &one, A + k0 * npad, CUDA_R_16BF,
                         (int)npad, B + j0 * npad, CUDA_R_16BF, (int)npad, &zero, out, CUDA_R_32F, (int)tk,
                         CUBLAS_COMPUTE_32F, CUBLAS_GEMM_DEFAULT);
        if (s != CUBLAS_STATUS_SUCCESS) {
            why = "cublasGemmEx failed (" + std::to_string((int)s) + ")";
            rc = -1;
        }
    };
    for (int64_t j0 = 0; j0 < M && rc == 0; j0 += T) {
        const int64_t tj = std::min<int64_t>(T, M - j0);
        for (int64_t k0 = 0; k0 <= j0 && rc == 0; k0 += T) {
            const int64_t tk = std::min<int64_t>(T, M - k0);
            gemm(gp, gp, k0, tk, j0, tj, P);            // P[j,k]  = g_j . g_k
            if (missing) {
                gemm(nm, gp, k0, tk, j0, tj, Q1);       // Q1[j,k] = g_j . m_k
                gemm(gp, nm, k0, tk, j0, tj, Q2);       // Q2[j,k] = m_j . g_k
                gemm(nm, nm, k0, tk, j0, tj, R);        // R[j,k]  = m_j . m_k
            }
            if (rc == 0) {
                k_gram_combine<<<152 * 8, 256, 0, st>>>(j0, tj, k0, tk, P, Q1, Q2, R, scale, counts, N, G);
                cu(cudaGetLastError(), "combine");
            }
        }
    }
    if (rc == 0)
        cu(cudaEventRecord(ev[1], st), "event");
    cu(cudaStreamSynchronize(st), "Gram build");
    if (rc == 0 && device_ms)
        cu(cudaEventElapsedTime(device_ms, ev[0], ev[1]), "event");
    for (cudaEvent_t e : ev)
        if (e)
            cudaEventDestroy(e);
    if (h)
        cublasDestroy(h);
    cudaFree(gp);
    cudaFree(nm);
    cudaFree(tiles);
    return rc;
}

}  // namespace brr
