// Marker Gram matrix G[j,k] = x_j . x_k of the standardised dense columns,
// stored as a packed lower triangle (entry (j, k), j > k, at j(j-1)/2 + k) as
// double-float pairs.  The blocked FP32C sweep uses it to resolve several markers per grid
// round exactly: after marker p changes the residual by dBeta_p * x_p, the
// dot product of a later marker t moves by dBeta_p * G[p, t].
//
// With g the genotype (0 when missing), m the non-missing indicator, sigma and
// c the per-marker scale and column mean of the dense builder:
//   x_j . x_k = s_j s_k (P_jk - c_k Q_jk - c_j Q_kj + c_j c_k R_jk)
//   P = g_j . g_k,  Q_jk = g_j . m_k,  R = m_j . m_k
// (missing genotypes take the value (mean - colmean) * sigma, which is zero up
// to the rounding of the two means and is left out).  P, Q, R are integer
// sums below 2^24.  They come from FP4 (E2M1, block scales all 1) or FP8
// (E4M3) GEMMs with FP32 accumulation on tiles of 8,192 markers (cuBLASLt, a
// plain library GEMM); 0, 1 and 2 are exact in both, every product and partial
// sum is an integer below 2^24, so the FP32 results are exact.  The build takes
// the first of FP4, FP8 and BF16 for which the library has an algorithm for
// every tile shape.  k_gram_combine forms the entries from exact 64-bit
// integer numerators (see there), one CTA row per marker j of the tile.
#include <cublasLt.h>
#include <cublas_v2.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <string>

#include "brr_device.cuh"
#include "brr_internal.h"

namespace brr {


// Per-marker constants of the combination: a_k = s_k / n_k as a double-float
// pair, and the marker's genotype sum q_k and count of present genotypes n_k.
__global__ void k_gram_consts(int64_t M, int64_t N, const double *__restrict__ scale,
                              const int64_t *__restrict__ counts, float2 *__restrict__ af,
                              longlong2 *__restrict__ qn)
{
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= M)
        return;
    const long long n = (long long)(N - counts[4 * k + 3]);
    const long long q = (long long)(counts[4 * k + 1] + 2 * counts[4 * k + 2]);
    float h, l;
    df_from_double(scale[2 * k] / (double)n, h, l);
    af[k] = make_float2(h, l);
    qn[k] = make_longlong2(q, n);
}

// Rows j in [j0, j0+tj) (one per blockIdx.y) and columns k in [k0, k0+tk),
// k < j, of the tile.  The products are stored column-major with the k index
// fastest: X[(j - j0) * ldp + (k - k0)].  With the column means c = q / n,
//   G = s_j s_k (P - c_k Q1 - c_j Q2 + c_j c_k R)
//     = a_j a_k (n_j n_k P - n_j q_k Q1 - q_j n_k Q2 + q_j q_k R),
// the second factor an exact 64-bit integer (|terms| < 4 N^3; without missing
// genotypes Q1 = q_j, Q2 = q_k, R = N), so the centred sum has no cancellation
// error; it is split into a double-float pair and multiplied by a_j a_k.
__global__ void k_gram_combine(int64_t j0, int64_t k0, int64_t tk, int64_t ldp, int64_t N,
                               const float *__restrict__ P, const float *__restrict__ Q1,
                               const float *__restrict__ Q2, const float *__restrict__ R,
                               const float2 *__restrict__ af, const longlong2 *__restrict__ qn,
                               float2 *__restrict__ G)
{
    const int64_t a = blockIdx.y;
    const int64_t j = j0 + a;
    const int64_t kend = j - k0 < tk ? j - k0 : tk;
    if (kend <= 0)
        return;
    const float2 aj = af[j];
    const longlong2 qnj = qn[j];
    const float *Prow = P + a * ldp;
    float2 *Grow = G + j * (j - 1) / 2 + k0;
    for (int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; b < kend; b += (int64_t)gridDim.x * blockDim.x) {
        const float2 ak = af[k0 + b];
        const longlong2 qnk = qn[k0 + b];
        const long long p = (long long)Prow[b];
        long long q1 = qnj.x, q2 = qnk.x, r = N;
        if (Q1) {
            const int64_t e = a * ldp + b;
            q1 = (long long)Q1[e];
            q2 = (long long)Q2[e];
            r = (long long)R[e];
        }
        const long long num = qnj.y * qnk.y * p - qnj.y * qnk.x * q1 - qnj.x * qnk.y * q2 + qnj.x * qnk.x * r;
        const float nh = __ll2float_rn(num);
        const float nl = __ll2float_rn(num - __float2ll_rn(nh));
        float sh, sl, gh, gl;
        df_mul(aj.x, aj.y, ak.x, ak.y, sh, sl);
        df_mul(sh, sl, nh, nl, gh, gl);
        Grow[b] = make_float2(gh, gl);
    }
}

// Rows [0, M) of the genotype matrix as FP8 E4M3 bytes (row length npad, a
// multiple of 16, padding zero) and optionally the non-missing indicator; one
// thread per 16 individuals (four code bytes in, 16 bytes out).
__global__ void k_decode_fp8(const uint8_t *__restrict__ codes, int64_t col_stride, int64_t N, int64_t npad,
                             int64_t M, uint8_t *__restrict__ gp, uint8_t *__restrict__ nm)
{
    const int64_t groups = npad / 16;
    const int64_t total = M * groups;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = e / groups;
        const int64_t q = e - r * groups;
        const uint32_t v = *reinterpret_cast<const uint32_t *>(codes + r * col_stride + 4 * q);
        uint32_t g[4], m[4];
#pragma unroll
        for (int w = 0; w < 4; ++w) {
            uint32_t gw = 0, mw = 0;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const unsigned c = (v >> (8 * w + 2 * k)) & 3u;
                const bool valid = 16 * q + 4 * w + k < N;
                // code 0: genotype 2 (E4M3 0x40), code 2: genotype 1 (0x38), code 3: 0, code 1: missing
                const uint32_t gb = !valid ? 0u : (c == 0u ? 0x40u : (c == 2u ? 0x38u : 0u));
                const uint32_t mb = (valid && c != 1u) ? 0x38u : 0u;
                gw |= gb << (8 * k);
                mw |= mb << (8 * k);
            }
            g[w] = gw;
            m[w] = mw;
        }
        reinterpret_cast<uint4 *>(gp + r * npad)[q] = make_uint4(g[0], g[1], g[2], g[3]);
        if (nm)
            reinterpret_cast<uint4 *>(nm + r * npad)[q] = make_uint4(m[0], m[1], m[2], m[3]);
    }
}

// Rows [0, M) of the genotype matrix as FP4 E2M1 (two individuals per byte,
// the first in the low half; row length npad, a multiple of 128, padding zero)
// and optionally the non-missing indicator; one thread per 16 individuals.
__global__ void k_decode_fp4(const uint8_t *__restrict__ codes, int64_t col_stride, int64_t N, int64_t npad,
                             int64_t M, uint8_t *__restrict__ gp, uint8_t *__restrict__ nm)
{
    const int64_t groups = npad / 16;
    const int64_t total = M * groups;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = e / groups;
        const int64_t q = e - r * groups;
        // the code bytes of individuals past the column's stored bytes are not read
        const int64_t b0 = 4 * q;
        uint32_t v = 0x55555555u;
        if (b0 + 4 <= col_stride)
            v = *reinterpret_cast<const uint32_t *>(codes + r * col_stride + b0);
        uint32_t g[2] = {0u, 0u}, m[2] = {0u, 0u};
#pragma unroll
        for (int k = 0; k < 16; ++k) {
            const unsigned c = (v >> (2 * k)) & 3u;
            const bool valid = 16 * q + k < N;
            // code 0: genotype 2 (E2M1 0x4), code 2: genotype 1 (0x2), code 3: 0, code 1: missing
            const uint32_t gb = !valid ? 0u : (c == 0u ? 0x4u : (c == 2u ? 0x2u : 0u));
            const uint32_t mb = (valid && c != 1u) ? 0x2u : 0u;
            g[k >> 3] |= gb << (4 * (k & 7));
            m[k >> 3] |= mb << (4 * (k & 7));
        }
        reinterpret_cast<uint2 *>(gp + r * (npad / 2))[q] = make_uint2(g[0], g[1]);
        if (nm)
            reinterpret_cast<uint2 *>(nm + r * (npad / 2))[q] = make_uint2(m[0], m[1]);
    }
}

// Rows [0, M) of the genotype matrix as BF16 (row length npad, padding zero),
// and optionally the non-missing indicator.
__global__ void k_decode_bf16(const uint8_t *__restrict__ codes, int64_t col_stride, int64_t N, int64_t npad,
                              int64_t M, __nv_bfloat16 *__restrict__ gp, __nv_bfloat16 *__restrict__ nm)
{
    const int64_t total = M * (npad / 4);
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = e / (npad / 4);
        const int64_t b = e - r * (npad / 4);
        const unsigned v = (4 * b < N) ? codes[r * col_stride + b] : 0x55u;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const unsigned c = (v >> (2 * k)) & 3u;
            const bool valid = 4 * b + k < N;
            const float g = (!valid || c == 1u) ? 0.f : (c == 0u ? 2.f : (c == 2u ? 1.f : 0.f));
            gp[r * npad + 4 * b + k] = __float2bfloat16(g);
            if (nm)
                nm[r * npad + 4 * b + k] = __float2bfloat16((valid && c != 1u) ? 1.f : 0.f);
        }
    }
}

namespace {

constexpr int64_t kTile = 8192;
constexpr size_t kLtWorkspace = (size_t)64 << 20;

inline int64_t round16(int64_t x) { return (x + 15) / 16 * 16; }
inline int64_t round128(int64_t x) { return (x + 127) / 128 * 128; }
int g_route_bits = 0;   // element bits of the last Gram build's GEMM operands

// FP4 or FP8 GEMMs through cuBLASLt: out (tk x tj, column-major, k fastest,
// leading dimension ld) = A(rows k0..) * B(rows j0..)^T over the npad-long
// rows.  FP4 operands carry a UE4M3 scale per 16 elements along a row, all 1.0
// here (`scales`, sized for the largest operand of the build).
struct LtGemm {
    cublasLtHandle_t h = nullptr;
    cublasLtMatmulDesc_t op = nullptr;
    cublasLtMatmulPreference_t pref = nullptr;
    void *ws = nullptr;
    int64_t npad = 0;
    cudaDataType_t type = CUDA_R_8F_E4M3;
    // the algorithm chosen for each tile shape of the build (at most four)
    struct Choice {
        int64_t tk, tj;
        cublasLtMatmulAlgo_t algo;
    };
    Choice chosen[4];
    int n_chosen = 0;

    bool init(int64_t np, cudaDataType_t t, const void *scales)
    {
        npad = np;
        type = t;
        const cublasOperation_t ta = CUBLAS_OP_T, tb = CUBLAS_OP_N;
        size_t wsb = kLtWorkspace;
        bool ok = cublasLtCreate(&h) == CUBLAS_STATUS_SUCCESS &&
                  cublasLtMatmulDescCreate(&op, CUBLAS_COMPUTE_32F, CUDA_R_32F) == CUBLAS_STATUS_SUCCESS &&
                  cublasLtMatmulDescSetAttribute(op, CUBLASLT_MATMUL_DESC_TRANSA, &ta, sizeof(ta)) ==
                      CUBLAS_STATUS_SUCCESS &&
                  cublasLtMatmulDescSetAttribute(op, CUBLASLT_MATMUL_DESC_TRANSB, &tb, sizeof(tb)) ==
                      CUBLAS_STATUS_SUCCESS &&
                  cublasLtMatmulPreferenceCreate(&pref) == CUBLAS_STATUS_SUCCESS &&
                  cublasLtMatmulPreferenceSetAttribute(pref, CUBLASLT_MATMUL_PREF_MAX_WORKSPACE_BYTES, &wsb,
                                                       sizeof(wsb)) == CUBLAS_STATUS_SUCCESS &&
                  cudaMalloc(&ws, kLtWorkspace) == cudaSuccess;
        if (ok && t == CUDA_R_4F_E2M1) {
            const int32_t mode = CUBLASLT_MATMUL_MATRIX_SCALE_VEC16_UE4M3;
            ok = cublasLtMatmulDescSetAttribute(op, CUBLASLT_MATMUL_DESC_A_SCALE_MODE, &mode, sizeof(mode)) ==
                     CUBLAS_STATUS_SUCCESS &&
                 cublasLtMatmulDescSetAttribute(op, CUBLASLT_MATMUL_DESC_B_SCALE_MODE, &mode, sizeof(mode)) ==
                     CUBLAS_STATUS_SUCCESS &&
                 cublasLtMatmulDescSetAttribute(op, CUBLASLT_MATMUL_DESC_A_SCALE_POINTER, &scales, sizeof(scales)) ==
                     CUBLAS_STATUS_SUCCESS &&
                 cublasLtMatmulDescSetAttribute(op, CUBLASLT_MATMUL_DESC_B_SCALE_POINTER, &scales, sizeof(scales)) ==
                     CUBLAS_STATUS_SUCCESS;
        }
        return ok;
    }
    // 0: done; 1: no algorithm for the shape (nothing launched); -1: error.
    // With A, B null: only the query for an algorithm.
    int run(const uint8_t *A, const uint8_t *B, int64_t tk, int64_t tj, int64_t ld, float *out, cudaStream_t st)
    {
        cublasLtMatrixLayout_t la = nullptr, lb = nullptr, lc = nullptr;
        int rc = -1;
        if (cublasLtMatrixLayoutCreate(&la, type, npad, tk, npad) == CUBLAS_STATUS_SUCCESS &&
            cublasLtMatrixLayoutCreate(&lb, type, npad, tj, npad) == CUBLAS_STATUS_SUCCESS &&
            cublasLtMatrixLayoutCreate(&lc, CUDA_R_32F, tk, tj, ld) == CUBLAS_STATUS_SUCCESS) {
            const cublasLtMatmulAlgo_t *algo = nullptr;
            for (int c = 0; c < n_chosen; ++c)
                if (chosen[c].tk == tk && chosen[c].tj == tj)
                    algo = &chosen[c].algo;
            cublasLtMatmulHeuristicResult_t hr{};
            int n = 0;
            if (!algo) {
                if (cublasLtMatmulAlgoGetHeuristic(h, op, la, lb, lc, lc, pref, 1, &hr, &n) == CUBLAS_STATUS_SUCCESS &&
                    n >= 1) {
                    algo = &hr.algo;
                    if (n_chosen < 4)
                        chosen[n_chosen++] = Choice{tk, tj, hr.algo};
                }
            }
            if (!algo) {
                rc = 1;
            } else if (!A || !B) {
                rc = 0;
            } else {
                const float one = 1.f, zero = 0.f;
                rc = cublasLtMatmul(h, op, &one, A, la, B, lb, &zero, out, lc, out, lc, algo, ws, kLtWorkspace,
                                    st) == CUBLAS_STATUS_SUCCESS
                         ? 0
                         : -1;
            }
        }
        if (la)
            cublasLtMatrixLayoutDestroy(la);
        if (lb)
            cublasLtMatrixLayoutDestroy(lb);
        if (lc)
            cublasLtMatrixLayoutDestroy(lc);
        return rc;
    }
    ~LtGemm()
    {
        if (pref)
            cublasLtMatmulPreferenceDestroy(pref);
        if (op)
            cublasLtMatmulDescDestroy(op);
        if (h)
            cublasLtDestroy(h);
        cudaFree(ws);
    }
};

}  // namespace

cudaError_t gram_bytes_needed(int64_t N, int64_t M, bool missing, size_t *gram, size_t *work)
{
    const int64_t npad = round16(N);
    const int64_t T = round128(std::min<int64_t>(M, kTile));
    *gram = (size_t)(M * (M - 1) / 2) * sizeof(float2);
    // the BF16 route's rows (2 bytes per genotype) bound the FP8 route's (1 byte)
    *work = (size_t)round16(M) * npad * 2 * (missing ? 2 : 1) + (size_t)T * T * 4 * (missing ? 4 : 1) * 2 +
            (size_t)M * 24 + kLtWorkspace;
    return cudaSuccess;
}

int build_gram(const uint8_t *codes, int64_t col_stride, int64_t N, int64_t M, const double *scale,
               const int64_t *counts, bool missing, float2 *G, cudaStream_t st, std::string &why, float *device_ms)
{
    // FP4 rows are multiples of 128 elements, FP8 and BF16 rows of 16; tile
    // sides are multiples of 128 (FP4) or 16 (padding rows and columns are
    // zero and their products are not read)
    const int64_t T = std::min<int64_t>(M, kTile);
    const int64_t Tp = round128(T);
    void *gp = nullptr, *nm = nullptr, *scales = nullptr;
    float *tiles = nullptr;
    float2 *af = nullptr;
    longlong2 *qn = nullptr;
    int rc = 0;
    auto cu = [&](cudaError_t e, const char *what) {
        if (e != cudaSuccess && rc == 0) {
            why = std::string(what) + ": " + cudaGetErrorString(e);
            rc = -1;
        }
    };
    cudaEvent_t ev[2] = {nullptr, nullptr};
    cu(cudaEventCreate(&ev[0]), "event");
    cu(cudaEventCreate(&ev[1]), "event");
    // two sets of product tiles: the combination of one tile runs on a second
    // stream while the tensor cores form the next
    const size_t set_floats = (size_t)Tp * Tp * (missing ? 4 : 1);
    cu(cudaMalloc(&tiles, sizeof(float) * set_floats * 2), "allocation of the product tiles");
    cudaStream_t sc = nullptr;
    cudaEvent_t ev_gemm[2] = {nullptr, nullptr}, ev_comb[2] = {nullptr, nullptr};
    cu(cudaStreamCreateWithFlags(&sc, cudaStreamNonBlocking), "stream");
    for (int b = 0; b < 2; ++b) {
        cu(cudaEventCreateWithFlags(&ev_gemm[b], cudaEventDisableTiming), "event");
        cu(cudaEventCreateWithFlags(&ev_comb[b], cudaEventDisableTiming), "event");
    }
    cu(cudaMalloc(&af, sizeof(float2) * (size_t)M), "allocation of the per-marker constants");
    cu(cudaMalloc(&qn, sizeof(longlong2) * (size_t)M), "allocation of the per-marker counts");
    float *P = tiles;   // the first set, for the choice of the route
    if (rc == 0)
        cu(cudaEventRecord(ev[0], st), "event");

    // the first route with an algorithm for every tile shape of the build: full
    // tiles and the last one
    const int64_t last = M - (M - 1) / T * T;
    int bits = 0;          // 4, 8 (cuBLASLt) or 16 (BF16 cublasGemmEx)
    int64_t npad = 0, Mp = 0;
    LtGemm lt;
    for (int cand : {4, 8}) {
        if (rc)
            break;
        const int64_t np = cand == 4 ? round128(N) : round16(N);
        const int64_t side = cand == 4 ? 128 : 16;
        if (cand == 4) {
            // UE4M3 scale 1.0 (0x38) for every 16 elements of the largest operand
            const size_t sbytes = (size_t)Tp * (size_t)(((np / 16) + 3) / 4 * 4);
            cu(cudaMalloc(&scales, sbytes), "allocation of the FP4 block scales");
            if (rc == 0)
                cu(cudaMemsetAsync(scales, 0x38, sbytes, st), "scales");
        }
        LtGemm trial;
        bool ok = rc == 0 && trial.init(np, cand == 4 ? CUDA_R_4F_E2M1 : CUDA_R_8F_E4M3, scales);
        for (int a = 0; a < 2 && ok; ++a)
            for (int b = 0; b < 2 && ok; ++b) {
                const int64_t sa = a ? (last + side - 1) / side * side : Tp;
                const int64_t sb = b ? (last + side - 1) / side * side : Tp;
                ok = trial.run(nullptr, nullptr, sa, sb, Tp, P, st) == 0;
            }
        if (ok) {
            bits = cand;
            npad = np;
            Mp = (M + side - 1) / side * side + (Tp - T);
            lt.init(np, cand == 4 ? CUDA_R_4F_E2M1 : CUDA_R_8F_E4M3, scales);
            break;
        }
        if (cand == 4) {
            cudaFree(scales);
            scales = nullptr;
        }
    }
    if (bits == 0) {
        bits = 16;
        npad = round16(N);
        Mp = round16(M);
    }
    // genotype and indicator rows: half a byte, a byte or two bytes per individual
    const size_t row_bytes = bits == 4 ? (size_t)npad / 2 : (size_t)npad * (bits / 8);
    cu(cudaMalloc(&gp, (size_t)Mp * row_bytes), "allocation of the decoded genotypes");
    if (missing)
        cu(cudaMalloc(&nm, (size_t)Mp * row_bytes), "allocation of the decoded indicators");
    if (rc == 0) {
        cu(cudaMemsetAsync(gp, 0, (size_t)Mp * row_bytes, st), "clear");
        if (nm)
            cu(cudaMemsetAsync(nm, 0, (size_t)Mp * row_bytes, st), "clear");
    }
    cublasHandle_t hb = nullptr;
    if (rc == 0 && bits == 16) {
        if (cublasCreate(&hb) != CUBLAS_STATUS_SUCCESS) {
            why = "cublasCreate failed";
            rc = -1;
        } else {
            cublasSetStream(hb, st);
        }
    }
    if (rc == 0) {
        if (bits == 4)
            k_decode_fp4<<<152 * 8, 256, 0, st>>>(codes, col_stride, N, npad, M, (uint8_t *)gp, (uint8_t *)nm);
        else if (bits == 8)
            k_decode_fp8<<<152 * 8, 256, 0, st>>>(codes, col_stride, N, npad, M, (uint8_t *)gp, (uint8_t *)nm);
        else
            k_decode_bf16<<<152 * 8, 256, 0, st>>>(codes, col_stride, N, npad, M, (__nv_bfloat16 *)gp,
                                                  (__nv_bfloat16 *)nm);
        cu(cudaGetLastError(), "decode");
        k_gram_consts<<<(unsigned)((M + 255) / 256), 256, 0, st>>>(M, N, scale, counts, af, qn);
        cu(cudaGetLastError(), "constants");
    }
    const float one = 1.f, zero = 0.f;
    auto gemm = [&](const void *A, const void *B, int64_t k0, int64_t tk, int64_t j0, int64_t tj, float *out) {
        if (rc)
            return;
        if (bits != 16) {
            if (lt.run((const uint8_t *)A + k0 * row_bytes, (const uint8_t *)B + j0 * row_bytes, tk, tj, Tp, out,
                       st) != 0) {
                why = "cuBLASLt low-precision GEMM failed";
                rc = -1;
            }
            return;
        }
        const cublasStatus_t s = cublasGemmEx(hb, CUBLAS_OP_T, CUBLAS_OP_N, (int)tk, (int)tj, (int)npad, &one,
                                              (const __nv_bfloat16 *)A + k0 * npad, CUDA_R_16BF, (int)npad,
                                              (const __nv_bfloat16 *)B + j0 * npad, CUDA_R_16BF, (int)npad, &zero,
                                              out, CUDA_R_32F, (int)Tp, CUBLAS_COMPUTE_32F, CUBLAS_GEMM_DEFAULT);
        if (s != CUBLAS_STATUS_SUCCESS) {
            why = "cublasGemmEx failed (" + std::to_string((int)s) + ")";
            rc = -1;
        }
    };
    const int64_t side = bits == 4 ? 128 : 16;
    int64_t tile = 0;
    for (int64_t j0 = 0; j0 < M && rc == 0; j0 += T) {
        const int64_t tj = std::min<int64_t>(T, M - j0);
        for (int64_t k0 = 0; k0 <= j0 && rc == 0; k0 += T, ++tile) {
            const int64_t tk = std::min<int64_t>(T, M - k0);
            const int b = (int)(tile & 1);
            float *Pb = tiles + (size_t)b * set_floats;
            float *Q1b = missing ? Pb + (size_t)Tp * Tp : nullptr, *Q2b = missing ? Pb + 2 * (size_t)Tp * Tp : nullptr,
                  *Rb = missing ? Pb + 3 * (size_t)Tp * Tp : nullptr;
            // the set is free once the combination of two tiles back is done
            if (tile >= 2)
                cu(cudaStreamWaitEvent(st, ev_comb[b], 0), "wait");
            // low-precision tile sides rounded up (those rows exist and are zero)
            const int64_t gk = bits != 16 ? (tk + side - 1) / side * side : tk;
            const int64_t gj = bits != 16 ? (tj + side - 1) / side * side : tj;
            gemm(gp, gp, k0, gk, j0, gj, Pb);            // P[j,k]  = g_j . g_k
            if (missing) {
                gemm(nm, gp, k0, gk, j0, gj, Q1b);       // Q1[j,k] = g_j . m_k
                gemm(gp, nm, k0, gk, j0, gj, Q2b);       // Q2[j,k] = m_j . g_k
                gemm(nm, nm, k0, gk, j0, gj, Rb);        // R[j,k]  = m_j . m_k
            }
            if (rc == 0) {
                cu(cudaEventRecord(ev_gemm[b], st), "event");
                cu(cudaStreamWaitEvent(sc, ev_gemm[b], 0), "wait");
                const dim3 grid((unsigned)((tk + 1023) / 1024), (unsigned)tj);
                k_gram_combine<<<grid, 256, 0, sc>>>(j0, k0, tk, Tp, N, Pb, Q1b, Q2b, Rb, af, qn, G);
                cu(cudaGetLastError(), "combine");
                cu(cudaEventRecord(ev_comb[b], sc), "event");
            }
        }
    }
    // the build ends when the last combinations have
    for (int b = 0; b < 2 && rc == 0; ++b)
        if (tile > b)
            cu(cudaStreamWaitEvent(st, ev_comb[b], 0), "wait");
    if (rc == 0)
        cu(cudaEventRecord(ev[1], st), "event");
    cu(cudaStreamSynchronize(st), "Gram build");
    if (sc)
        cu(cudaStreamSynchronize(sc), "Gram build");
    if (rc == 0 && device_ms)
        cu(cudaEventElapsedTime(device_ms, ev[0], ev[1]), "event");
    for (cudaEvent_t e : ev)
        if (e)
            cudaEventDestroy(e);
    for (int b = 0; b < 2; ++b) {
        if (ev_gemm[b])
            cudaEventDestroy(ev_gemm[b]);
        if (ev_comb[b])
            cudaEventDestroy(ev_comb[b]);
    }
    if (sc)
        cudaStreamDestroy(sc);
    if (hb)
        cublasDestroy(hb);
    cudaFree(gp);
    cudaFree(nm);
    cudaFree(scales);
    cudaFree(tiles);
    cudaFree(af);
    cudaFree(qn);
    g_route_bits = rc == 0 ? bits : 0;
    return rc;
}

int gram_route_bits() { return g_route_bits; }

}  // namespace brr
