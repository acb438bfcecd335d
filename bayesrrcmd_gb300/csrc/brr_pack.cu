// Device packer: PLINK BED payload -> device marker store.
//
// Replaces the per-genotype MarkerBuilder calls of the reference preprocess
// (src/preprocessgraph.cpp:24-60 drives DenseMarkerBuilder /
// RaggedSparseMarkerBuilder::processAllele once per genotype).  Here the 2-bit
// codes stay 2-bit in HBM (one column per marker, padded to 16-byte chunks of
// 64 individuals), per-marker genotype counts are reduced on the device and
// the standardisation table or ragged statistics are derived from the counts.
#include "brr_device.cuh"
#include "brr_internal.h"
#include "brr_stream.h"

namespace brr {

// Decode of one 2-bit field (src/preprocessgraph.cpp:43-56): allele1 = !bit0,
// allele2 = !bit1; (0,1) is missing (src/densemarkerbuilder.cpp:30).
//   code 0 -> g = 2, code 1 -> missing, code 2 -> g = 1, code 3 -> g = 0.

__global__ void __launch_bounds__(kThreads) k_pack_counts(const uint8_t *__restrict__ bed, int64_t N,
                                                          int64_t M, uint8_t *__restrict__ codes,
                                                          int64_t col_stride, int64_t *__restrict__ counts)
{
    const int64_t cb = (N + 3) >> 2;
    __shared__ int red[4][kThreads / 32];
    for (int64_t j = blockIdx.x; j < M; j += gridDim.x) {
        const uint8_t *src = bed + j * cb;
        uint8_t *dst = codes + j * col_stride;
        int c0 = 0, c1 = 0, c2 = 0, c3 = 0;
        for (int64_t b = threadIdx.x; b < col_stride; b += blockDim.x) {
            if (b < cb) {
                const unsigned v = src[b];
                dst[b] = (uint8_t)v;
                const int64_t i0 = b * 4;
                const int nvalid = (int)imin64(4, N - i0);
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    if (k < nvalid) {
                        const unsigned c = (v >> (2 * k)) & 3u;
                        c0 += c == 3u;   // g = 0
                        c1 += c == 2u;   // g = 1
                        c2 += c == 0u;   // g = 2
                        c3 += c == 1u;   // missing
                    }
                }
            } else {
                dst[b] = 0x55;  // padding: missing codes
            }
        }
        // block reduction of the four counters
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            c0 += __shfl_xor_sync(0xffffffffu, c0, o);
            c1 += __shfl_xor_sync(0xffffffffu, c1, o);
            c2 += __shfl_xor_sync(0xffffffffu, c2, o);
            c3 += __shfl_xor_sync(0xffffffffu, c3, o);
        }
        const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
        if (l == 0) {
            red[0][w] = c0;
            red[1][w] = c1;
            red[2][w] = c2;
            red[3][w] = c3;
        }
        __syncthreads();
        if (threadIdx.x < 4) {
            long long s = 0;
            for (int q = 0; q < (int)(blockDim.x >> 5); ++q)
                s += red[threadIdx.x][q];
            counts[4 * j + threadIdx.x] = s;
        }
        __syncthreads();
    }
}

// Dense standardisation table from the counts (src/densemarkerbuilder.cpp:43-60):
// missing -> mean of non-missing, centre by the column mean, scale to squared
// norm N-1.  The column holds four distinct values, so mean, column mean and
// squared norm follow from the counts; every operation is a separately rounded
// IEEE operation so the table is bit-identical to the CPU restatement.
__global__ void k_dense_tables(const int64_t *__restrict__ counts, int64_t N, int64_t M,
                               double *__restrict__ lut, double *__restrict__ scale, double *__restrict__ colsum,
                               int *bad)
{
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= M)
        return;
    const int64_t n0 = counts[4 * j], n1 = counts[4 * j + 1], n2 = counts[4 * j + 2], nm = counts[4 * j + 3];
    if (nm >= N) {
        atomicMin(bad, (int)j);
        return;
    }
    const double S = (double)(n1 + 2 * n2);
    const double mean = __ddiv_rn(S, __dsub_rn((double)N, (double)nm));
    const double colmean = __ddiv_rn(__dadd_rn(S, __dmul_rn((double)nm, mean)), (double)N);
    const double c0 = __dsub_rn(0.0, colmean), c1 = __dsub_rn(1.0, colmean);
    const double c2 = __dsub_rn(2.0, colmean), cm = __dsub_rn(mean, colmean);
    const double sqn = __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn((double)n0, __dmul_rn(c0, c0)),
                                                     __dmul_rn((double)n1, __dmul_rn(c1, c1))),
                                           __dmul_rn((double)n2, __dmul_rn(c2, c2))),
                                 __dmul_rn((double)nm, __dmul_rn(cm, cm)));
    if (!(sqn > 0.0)) {
        atomicMin(bad, (int)j);
        return;
    }
    const double sigma = __ddiv_rn(1.0, __dsqrt_rn(__ddiv_rn(sqn, __dsub_rn((double)N, 1.0))));
    lut[4 * j + 0] = __dmul_rn(c2, sigma);
    lut[4 * j + 1] = __dmul_rn(cm, sigma);
    lut[4 * j + 2] = __dmul_rn(c1, sigma);
    lut[4 * j + 3] = __dmul_rn(c0, sigma);
    scale[2 * j + 0] = sigma;
    scale[2 * j + 1] = colmean;
    // sum of the standardised column (zero up to rounding)
    colsum[j] = (double)n0 * lut[4 * j + 3] + (double)n1 * lut[4 * j + 2] + (double)n2 * lut[4 * j + 0] +
                (double)nm * lut[4 * j + 1];
}

// Ragged statistics (src/sparsemarker.cpp:8-19, src/raggedsparsemarkerbuilder.cpp:43-55):
// mean over N including missing, sd from the sum and sum of squares.
__global__ void k_ragged_stats(const int64_t *__restrict__ counts, int64_t N, int64_t M, int eigen,
                               double *__restrict__ stats, int *bad)
{
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= M)
        return;
    const int64_t n1 = counts[4 * j + 1], n2 = counts[4 * j + 2];
    double Zsum = (double)(n1 + 2 * n2);
    double sqrdZ = (double)(n1 + 4 * n2);
    const double Nd = (double)N;
    const double mean = __ddiv_rn(Zsum, Nd);
    if (eigen) {
        // src/eigensparsemarkerbuilder.cpp:46-56: the missing genotypes enter
        // sqrdZ and Zsum at the mean before the sd is formed
        const double nm = (double)counts[4 * j + 3];
        sqrdZ = __dadd_rn(sqrdZ, __dmul_rn(__dmul_rn(mean, mean), nm));
        Zsum = __dadd_rn(Zsum, __dmul_rn(mean, nm));
    }
    const double var = __ddiv_rn(__dadd_rn(__dsub_rn(sqrdZ, __dmul_rn(__dmul_rn(2.0, mean), Zsum)),
                                           __dmul_rn(__dmul_rn(Nd, mean), mean)),
                                 __dsub_rn(Nd, 1.0));
    const double sd = __dsqrt_rn(var);
    stats[4 * j + 0] = mean;
    stats[4 * j + 1] = sd;
    stats[4 * j + 2] = sqrdZ;
    stats[4 * j + 3] = Zsum;
    // src/raggedsparsemarker.cpp:68-77: a marker without ones and twos is invalid.
    if (n1 + n2 == 0 || !(sd > 0.0))
        atomicMin(bad, (int)j);
}

// Per (marker, slice) counts of ones / twos / missing for the slice-major
// ragged layout.  One CTA per marker, threads over slices.
__global__ void __launch_bounds__(kThreads) k_ragged_slice_counts(const uint8_t *__restrict__ codes,
                                                                  int64_t col_stride, int64_t M, int G,
                                                                  const int32_t *__restrict__ slice_lo,
                                                                  int32_t *__restrict__ cnt3)
{
    const int64_t MG = M * (int64_t)G;
    for (int64_t j = blockIdx.x; j < M; j += gridDim.x) {
        const uint8_t *col = codes + j * col_stride;
        for (int s = threadIdx.x; s < G; s += blockDim.x) {
            const int lo = slice_lo[s], hi = slice_lo[s + 1];
            int a = 0, b = 0, m = 0;
            for (int i = lo; i < hi; ++i) {
                const unsigned c = (col[i >> 2] >> (2 * (i & 3))) & 3u;
                a += c == 2u;
                b += c == 0u;
                m += c == 1u;
            }
            const int64_t e = j * G + s;
            cnt3[e] = a;
            cnt3[MG + 1 + e] = b;
            cnt3[2 * (MG + 1) + e] = m;
        }
    }
}

// Fill slice-local indices in ascending order (src/raggedsparsemarkerbuilder.cpp:25-41
// appends in decode order, i.e. ascending individual index).
__global__ void __launch_bounds__(kThreads) k_ragged_fill(const uint8_t *__restrict__ codes, int64_t col_stride,
                                                          int64_t M, int G, const int32_t *__restrict__ slice_lo,
                                                          const int32_t *__restrict__ off0,
                                                          const int32_t *__restrict__ off1,
                                                          const int32_t *__restrict__ off2,
                                                          uint16_t *__restrict__ idx0, uint16_t *__restrict__ idx1,
                                                          uint16_t *__restrict__ idx2)
{
    for (int64_t j = blockIdx.x; j < M; j += gridDim.x) {
        const uint8_t *col = codes + j * col_stride;
        for (int s = threadIdx.x; s < G; s += blockDim.x) {
            const int lo = slice_lo[s], hi = slice_lo[s + 1];
            const int64_t e = j * G + s;
            int32_t a = off0[e], b = off1[e], m = off2[e];
            for (int i = lo; i < hi; ++i) {
                const unsigned c = (col[i >> 2] >> (2 * (i & 3))) & 3u;
                const uint16_t li = (uint16_t)(i - lo);
                if (c == 2u)
                    idx0[a++] = li;
                else if (c == 0u)
                    idx1[b++] = li;
                else if (c == 1u)
                    idx2[m++] = li;
            }
        }
    }
}

// Exclusive scan of int32 in three passes (tile scan, scan of tile sums in one
// CTA, add).  Tiles of 1024 elements.
constexpr int kScanTile = 1024;

__global__ void __launch_bounds__(kThreads) k_scan_tiles(int32_t *data, int64_t n, int32_t *tile_sums)
{
    __shared__ int32_t sh[kScanTile];
    __shared__ int32_t wsum[kThreads / 32];
    const int64_t base = (int64_t)blockIdx.x * kScanTile;
    for (int k = threadIdx.x; k < kScanTile; k += blockDim.x)
        sh[k] = (base + k < n) ? data[base + k] : 0;
    __syncthreads();
    // each thread scans 4 consecutive elements
    const int t = threadIdx.x;
    int32_t v0 = sh[4 * t], v1 = sh[4 * t + 1], v2 = sh[4 * t + 2], v3 = sh[4 * t + 3];
    const int32_t tot = v0 + v1 + v2 + v3;
    int32_t x = tot;
    const int l = t & 31, w = t >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (l >= o)
            x += y;
    }
    if (l == 31)
        wsum[w] = x;
    __syncthreads();
    int32_t wpre = 0;
    for (int q = 0; q < w; ++q)
        wpre += wsum[q];
    const int32_t excl = wpre + x - tot;
    sh[4 * t] = excl;
    sh[4 * t + 1] = excl + v0;
    sh[4 * t + 2] = excl + v0 + v1;
    sh[4 * t + 3] = excl + v0 + v1 + v2;
    __syncthreads();
    for (int k = threadIdx.x; k < kScanTile; k += blockDim.x)
        if (base + k < n)
            data[base + k] = sh[k];
    if (threadIdx.x == blockDim.x - 1) {
        int32_t s = 0;
        for (int q = 0; q < (int)(blockDim.x >> 5); ++q)
            s += wsum[q];
        tile_sums[blockIdx.x] = s;
    }
}

__global__ void k_scan_sums(int32_t *tile_sums, int64_t ntiles)
{
    if (threadIdx.x != 0 || blockIdx.x != 0)
        return;
    int32_t run = 0;
    for (int64_t q = 0; q < ntiles; ++q) {
        const int32_t v = tile_sums[q];
        tile_sums[q] = run;
        run += v;
    }
}

__global__ void k_scan_add(int32_t *data, int64_t n, const int32_t *tile_sums)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
        data[i] += tile_sums[i / kScanTile];
}

cudaError_t launch_pack_counts(const uint8_t *bed, int64_t N, int64_t M, uint8_t *codes, int64_t col_stride,
                               int64_t *counts, cudaStream_t st)
{
    const int blocks = (int)imin64(M, 152 * 16);
    k_pack_counts<<<blocks, kThreads, 0, st>>>(bed, N, M, codes, col_stride, counts);
    return cudaGetLastError();
}

cudaError_t launch_dense_tables(const int64_t *counts, int64_t N, int64_t M, double *lut, double *scale,
                                double *colsum, int *bad, cudaStream_t st)
{
    k_dense_tables<<<(unsigned)((M + 255) / 256), 256, 0, st>>>(counts, N, M, lut, scale, colsum, bad);
    return cudaGetLastError();
}

cudaError_t launch_ragged_stats(const int64_t *counts, int64_t N, int64_t M, int eigen, double *stats, int *bad,
                                cudaStream_t st)
{
    k_ragged_stats<<<(unsigned)((M + 255) / 256), 256, 0, st>>>(counts, N, M, eigen, stats, bad);
    return cudaGetLastError();
}

cudaError_t launch_ragged_slice_counts(const uint8_t *codes, int64_t col_stride, int64_t M, int G,
                                       const int32_t *slice_lo, int32_t *cnt3, cudaStream_t st)
{
    const int blocks = (int)imin64(M, 152 * 16);
    k_ragged_slice_counts<<<blocks, kThreads, 0, st>>>(codes, col_stride, M, G, slice_lo, cnt3);
    return cudaGetLastError();
}

cudaError_t launch_exclusive_scan_i32(int32_t *data, int64_t n, int32_t *tmp, cudaStream_t st)
{
    const int64_t ntiles = (n + kScanTile - 1) / kScanTile;
    k_scan_tiles<<<(unsigned)ntiles, kThreads, 0, st>>>(data, n, tmp);
    k_scan_sums<<<1, 32, 0, st>>>(tmp, ntiles);
    k_scan_add<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(data, n, tmp);
    return cudaGetLastError();
}

cudaError_t launch_ragged_fill(const uint8_t *codes, int64_t col_stride, int64_t M, int G, const int32_t *slice_lo,
                               const int32_t *off0, const int32_t *off1, const int32_t *off2, uint16_t *idx0,
                               uint16_t *idx1, uint16_t *idx2, cudaStream_t st)
{
    const int blocks = (int)imin64(M, 152 * 16);
    k_ragged_fill<<<blocks, kThreads, 0, st>>>(codes, col_stride, M, G, slice_lo, off0, off1, off2, idx0, idx1,
                                               idx2);
    return cudaGetLastError();
}

}  // namespace brr

namespace brr {

// Seeded synthetic genotypes written directly as a BED payload: marker j has
// allele frequency p_j = p_lo + (p_hi - p_lo) * U, genotypes are two
// Bernoulli(p_j) draws, missing at rate `miss`.  Every byte is a function of
// (seed, j, byte index) through the same Philox stream as the sampler.
__global__ void k_synth_bed(uint8_t *__restrict__ out, int64_t N, int64_t M, uint32_t seed, double p_lo,
                            double p_hi, double miss, double beta_a, double beta_b)
{
    const int64_t cb = (N + 3) >> 2;
    for (int64_t j = blockIdx.x; j < M; j += gridDim.x) {
        float p;
        if (beta_a > 0.0) {
            // p ~ Beta(a, b) = X / (X + Y), X ~ Gamma(a), Y ~ Gamma(b), clipped to [p_lo, p_hi]
            __shared__ double s_p;
            if (threadIdx.x == 0) {
                double x = 1.0, y = 1.0;
                const StreamKey k{seed, 0x5EEDu};
                gamma_draw(k, (uint32_t)j, 12u, 0u, beta_a, &x);
                gamma_draw(k, (uint32_t)j, 12u, 1u, beta_b, &y);
                s_p = fmin(fmax(x / (x + y), p_lo), p_hi);
            }
            __syncthreads();
            p = (float)s_p;
            __syncthreads();
        } else {
            const U4 pb = philox4x32_10((uint32_t)j, 0u, 9u, 0u, seed, 0x5EEDu);
            p = (float)(p_lo + (p_hi - p_lo) * u53(pb.x, pb.y));
        }
        const uint32_t t1 = (uint32_t)fminf(4294967040.f, p * 4294967296.f);
        const uint32_t tm = (uint32_t)fminf(4294967040.f, (float)miss * 4294967296.f);
        for (int64_t b = threadIdx.x; b < cb; b += blockDim.x) {
            const U4 r = philox4x32_10((uint32_t)j, (uint32_t)b, 10u, 0u, seed, 0x5EEDu);
            const U4 q = philox4x32_10((uint32_t)j, (uint32_t)b, 11u, 0u, seed, 0x5EEDu);
            const uint32_t ra[4] = {r.x, r.y, r.z, r.w};
            const uint32_t qa[4] = {q.x, q.y, q.z, q.w};
            unsigned byte = 0;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                // two allele draws from the two halves of one 32-bit word (16 bits each)
                const unsigned a1 = (ra[k] & 0xFFFFu) < (t1 >> 16);
                const unsigned a2 = (ra[k] >> 16) < (t1 >> 16);
                const unsigned gv = a1 + a2;
                unsigned code = gv == 2 ? 0u : (gv == 1 ? 2u : 3u);
                if (qa[k] < tm)
                    code = 1u;
                if (b * 4 + k >= N)
                    code = 0u;
                byte |= code << (2 * k);
            }
            out[j * cb + b] = (uint8_t)byte;
        }
        // keep every marker polymorphic: individual 0 heterozygous, 1 homozygous
        if (threadIdx.x == 0 && N >= 2) {
            unsigned v = out[j * cb];
            v = (v & ~0x0Fu) | 2u | (3u << 2);
            out[j * cb] = (uint8_t)v;
        }
    }
}

cudaError_t launch_synth_bed(uint8_t *out, int64_t N, int64_t M, uint32_t seed, double p_lo, double p_hi,
                             double miss, cudaStream_t st, double beta_a, double beta_b)
{
    const int blocks = (int)imin64(M, 152 * 32);
    k_synth_bed<<<blocks, kThreads, 0, st>>>(out, N, M, seed, p_lo, p_hi, miss, beta_a, beta_b);
    return cudaGetLastError();
}

}  // namespace brr
