// Counter-based draw stream shared by the host driver and the device kernels.
//
// The reference draws its random numbers from one Boost mt19937 engine in a
// fixed call order (src/distributions_boost.cpp:16-65, call sites
// src/BayesRBase.cpp:60-63, :101-110, :198, :238-246, src/DenseBayesRRmz.cpp:39).
// A sequential engine cannot be replayed from many GPU threads, so every draw
// here is a pure function of (seed, chain, index, iteration, purpose, sub)
// through Philox4x32-10 (Salmon et al., "Parallel random numbers: as easy as
// 1, 2, 3", SC'11).  The same definitions are compiled for host and device so
// the CPU oracle and the GPU path consume identical uniforms.
#pragma once
#include <stdint.h>
#include <math.h>

#if defined(__CUDACC__)
#define BRR_HD __host__ __device__ __forceinline__
#else
#define BRR_HD inline
#endif

namespace brr {

enum Purpose : uint32_t {
    kPurposeInit = 1,    // initial sigmaG uniforms           (src/BayesRBase.cpp:60-63)
    kPurposeMu = 2,      // intercept normal                  (src/DenseBayesRRmz.cpp:39)
    kPurposeMarker = 3,  // per-marker (u, z)                 (src/BayesRBase.cpp:106-109)
    kPurposePerm = 4,    // sweep permutation                 (src/BayesRBase.cpp:198)
    kPurposeSigmaE = 5,  // residual-variance gamma           (src/BayesRBase.cpp:239)
    kPurposeSigmaG = 6,  // genetic-variance gamma per group  (src/BayesRBase.cpp:245)
    kPurposePi = 7,      // Dirichlet gammas                  (src/BayesRBase.cpp:246)
};

struct U4 { uint32_t x, y, z, w; };

BRR_HD U4 philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1)
{
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        const uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
        const uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
        c1 = (uint32_t)p1;
        c3 = (uint32_t)p0;
        c0 = n0;
        c2 = n2;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return U4{c0, c1, c2, c3};
}

struct StreamKey { uint32_t seed, chain; };

BRR_HD U4 stream_block(StreamKey k, uint32_t idx, uint32_t it, uint32_t purpose, uint32_t sub)
{
    return philox4x32_10(idx, it, purpose, sub, k.seed, k.chain);
}

// 53 random bits offset by one half: strictly inside (0, 1).
BRR_HD double u53(uint32_t a, uint32_t b)
{
    return ((double)(a >> 5) * 67108864.0 + (double)(b >> 6) + 0.5) * (1.0 / 9007199254740992.0);
}

// Box-Muller, cosine branch.
BRR_HD double box_muller(double v1, double v2)
{
    return sqrt(-2.0 * log(v1)) * cos(6.283185307179586 * v2);
}

// Marker j's (u, z) for iteration it.
BRR_HD void marker_draws(StreamKey k, uint32_t it, uint32_t j, double *u, double *z)
{
    const U4 b = stream_block(k, j, it, kPurposeMarker, 0);
    const U4 c = stream_block(k, j, it, kPurposeMarker, 1);
    *u = u53(b.x, b.y);
    *z = box_muller(u53(b.z, b.w), u53(c.x, c.y));
}

BRR_HD double uniform_init(StreamKey k, uint32_t g)
{
    const U4 b = stream_block(k, g, 0, kPurposeInit, 0);
    return u53(b.x, b.y);
}

BRR_HD double normal_mu(StreamKey k, uint32_t it)
{
    const U4 b = stream_block(k, 0, it, kPurposeMu, 0);
    return box_muller(u53(b.x, b.y), u53(b.z, b.w));
}

// Gamma(shape, 1): Marsaglia & Tsang (ACM TOMS 26(3), 2000); shape < 1 uses
// the G(shape+1) * U^(1/shape) boost.  Returns false if 1024 attempts fail.
BRR_HD bool gamma_draw(StreamKey k, uint32_t it, uint32_t purpose, uint32_t sub, double shape, double *out)
{
    if (!(shape > 0.0))
        return false;
    const double a = shape < 1.0 ? shape + 1.0 : shape;
    const double d = a - 1.0 / 3.0;
    const double c = 1.0 / sqrt(9.0 * d);
    for (uint32_t t = 0; t < 1024; ++t) {
        const U4 b = stream_block(k, t, it, purpose, sub);
        const U4 e = stream_block(k, t, it, purpose, sub | 0x80000000u);
        const double x = box_muller(u53(b.x, b.y), u53(b.z, b.w));
        double v = 1.0 + c * x;
        if (v <= 0.0)
            continue;
        v = v * v * v;
        const double u = u53(e.x, e.y);
        const double x2 = x * x;
        if (u < 1.0 - 0.0331 * (x2 * x2) || log(u) < 0.5 * x2 + d * (1.0 - v + log(v))) {
            double g = d * v;
            if (shape < 1.0)
                g = g * pow(u53(e.z, e.w), 1.0 / shape);
            *out = g;
            return true;
        }
    }
    return false;
}

// Inverse scaled chi-square (src/distributions_boost.cpp:45-47, :58-60).
BRR_HD bool inv_scaled_chisq(StreamKey k, uint32_t it, uint32_t purpose, uint32_t sub,
                             double dof, double scale, double *out)
{
    double g;
    if (!gamma_draw(k, it, purpose, sub, 0.5 * dof, &g))
        return false;
    const double sc = 1.0 / (0.5 * dof * scale);
    *out = 1.0 / (sc * g);
    return true;
}

// Fisher-Yates permutation of 0..M-1 for iteration it (host; defined in brr_api.cu).
void make_permutation(StreamKey key, uint32_t it, uint32_t M, uint32_t *perm);

}  // namespace brr
