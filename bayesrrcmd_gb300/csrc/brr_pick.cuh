// Reference component sampler (FP64 with an optional certified FP32 path),
// shared by the restart sweep and the blocked sweep.
#pragma once
#include <math.h>

#include "brr_device.cuh"

namespace brr {

// Component selection for one marker by one thread (src/BayesRBase.cpp:309-366).
// logL_k = c_k + h_k*num^2 with c_k = log(pi_k) - log(sigmaG/sigmaE*(N-1)*cVa_k + 1)/2
// and h_k = 1/(2*denom_k*sigmaE).  P(k) = exp(logL_k - max)/sum, zeroed where the
// reference's 700 guards fire (any |logL_q - logL_k| > 700 over q >= 1); the
// walk picks the first k whose cumulative probability reaches u.
// FP32 = true evaluates the exponentials in single precision from the FP64
// log-likelihood differences and keeps the decision only when u is further
// than 2e-5 from every cumulative bound it was compared with (the FP32 error
// is below 5e-6); otherwise the FP64 evaluation decides.
struct Pick {
    int comp;       // chosen component, -1 if none
    double beta;    // new beta (beta_old when none)
    double acum0;   // P(component 0) as stored in acum
};

template <bool FP32, int KM>
__device__ __forceinline__ Pick pick_marker(double num, double u, double z, double beta_old,
                                            const double *__restrict__ gc, int K)
{
    double L[KM];
    const double n2 = num * num;
#pragma unroll
    for (int k = 0; k < KM; ++k)
        L[k] = k < K ? (k == 0 ? gc[0] : fma(gc[4 * k + 2], n2, gc[4 * k])) : -INFINITY;
    double lmax = L[0], lmax1 = L[1], lmin1 = L[1];
#pragma unroll
    for (int k = 1; k < KM; ++k) {
        if (k < K) {
            lmax = fmax(lmax, L[k]);
            lmax1 = fmax(lmax1, L[k]);
            lmin1 = fmin(lmin1, L[k]);
        }
    }
    // the guards of components q >= 1 can only fire when the log-likelihoods of
    // components 1..K-1 span more than 700
    const bool wide = lmax1 - lmin1 > 700.0;
    const bool guard0 = (lmax1 - L[0] > 700.0) || (L[0] - lmin1 > 700.0);
    auto guarded = [&](int k) -> bool {
        return k == 0 ? guard0 : (wide && ((lmax1 - L[k] > 700.0) || (L[k] - lmin1 > 700.0)));
    };
    Pick res;
    res.comp = -1;
    res.beta = beta_old;
    res.acum0 = 0.0;
    bool decided = false;
    if (FP32) {
        float e[KM];
        float es = 0.f;
#pragma unroll
        for (int k = 0; k < KM; ++k) {
            e[k] = k < K ? __expf((float)(L[k] - lmax)) : 0.f;
            es += e[k];
        }
        const float ies = __frcp_rn(es);
        int chosen = -1;
        float acum = 0.f, prev = 0.f, a0 = 0.f;
        const float uf = (float)u;
#pragma unroll
        for (int k = 0; k < KM; ++k) {
            if (k < K && chosen < 0) {
                const float pk = guarded(k) ? 0.f : e[k] * ies;
                if (k == 0)
                    a0 = pk;
                prev = acum;
                acum += pk;
                if (uf <= acum)
                    chosen = k;
            }
        }
        const float tol = 2e-5f;
        const bool close = chosen >= 0 ? ((uf > acum - tol) || (chosen > 0 && uf < prev + tol)) : (uf < acum + tol);
        if (!close) {
            res.comp = chosen;
            res.acum0 = (double)a0;
            decided = true;
        }
    }
    if (!decided) {
        double e[KM];
        double es = 0.0;
#pragma unroll
        for (int k = 0; k < KM; ++k) {
            e[k] = k < K ? exp(L[k] - lmax) : 0.0;
            es += e[k];
        }
        const double ies = 1.0 / es;
        int chosen = -1;
        double acum = 0.0, a0 = 0.0;
#pragma unroll
        for (int k = 0; k < KM; ++k) {
            if (k < K && chosen < 0) {
                const double pk = guarded(k) ? 0.0 : e[k] * ies;
                if (k == 0)
                    a0 = pk;
                acum += pk;
                if (u <= acum)
                    chosen = k;
            }
        }
        res.comp = chosen;
        res.acum0 = a0;
    }
    if (res.comp == 0) {
        res.beta = 0.0;
    } else if (res.comp > 0) {
        const double sdk = gc[4 * res.comp + 3], invden = gc[4 * res.comp + 1];
        res.beta = __dadd_rn(__dmul_rn(z, sdk), __dmul_rn(num, invden));
    }
    return res;
}

// FP32 component selection with a rigorous error bound, falling back to the
// FP64 evaluation of pick_marker when the bound cannot certify the decision.
// With D_k = logL_k - logL_0 = dc_k + h_k*num^2 (dc_0 = h_0 = 0) evaluated by one
// FMA from rounded inputs, |error(D_k)| <= 3u(|dc_k| + |h_k num^2|) with
// u = 2^-24.  The 700 guards compare differences of D (the logL_0 offset
// cancels); a guard whose difference lies within the error band of 700
// falls back.  Probabilities then carry at most 2*max_err + 2^-21 relative
// error, so a u within tol = 4e-5 + 4*max_err of a cumulative bound falls back.
template <int KM>
__device__ __forceinline__ bool pick_f32(float xh, float xl, float uf, const float *__restrict__ gcf, int K,
                                         int &comp, float &a0out)
{
    // num = xh + xl (double-float); num^2 to FP32 within 3u
    const float n2 = __fmaf_rn(xh, xh, 2.f * xh * xl);
    float D[KM];
    float maxerr = 0.f;
#pragma unroll
    for (int k = 0; k < KM; ++k) {
        if (k == 0 || k >= K) {
            D[k] = k == 0 ? 0.f : -INFINITY;
        } else {
            const float dc = gcf[2 * k], h = gcf[2 * k + 1];
            D[k] = __fmaf_rn(h, n2, dc);
            maxerr = fmaxf(maxerr, 3.0e-7f * (fabsf(dc) + fabsf(h * n2)));
        }
    }
    float dmax = 0.f, dmax1 = D[1], dmin1 = D[1];
#pragma unroll
    for (int k = 1; k < KM; ++k) {
        if (k < K) {
            dmax = fmaxf(dmax, D[k]);
            dmax1 = fmaxf(dmax1, D[k]);
            dmin1 = fminf(dmin1, D[k]);
        }
    }
    const float band = 2.f * maxerr + 1e-3f;
    const float spread = dmax1 - dmin1;
    bool unsure = fabsf(spread - 700.f) < band || fabsf(dmax1 - 700.f) < band || fabsf(-dmin1 - 700.f) < band;
    const bool wide = spread > 700.f;
    const bool guard0 = (dmax1 > 700.f) || (-dmin1 > 700.f);
    float e[KM];
    float es = 0.f;
#pragma unroll
    for (int k = 0; k < KM; ++k) {
        e[k] = k < K ? __expf(D[k] - dmax) : 0.f;
        es += e[k];
    }
    const float ies = __frcp_rn(es);
    int chosen = -1;
    float acum = 0.f, prev = 0.f, a0 = 0.f;
#pragma unroll
    for (int k = 0; k < KM; ++k) {
        if (k < K && chosen < 0) {
            bool guard;
            if (k == 0) {
                guard = guard0;
            } else {
                const float d1 = dmax1 - D[k], d2 = D[k] - dmin1;
                if (wide && (fabsf(d1 - 700.f) < band || fabsf(d2 - 700.f) < band))
                    unsure = true;
                guard = wide && (d1 > 700.f || d2 > 700.f);
            }
            const float pk = guard ? 0.f : e[k] * ies;
            if (k == 0)
                a0 = pk;
            prev = acum;
            acum += pk;
            if (uf <= acum)
                chosen = k;
        }
    }
    const float tol = 4e-5f + 4.f * maxerr;
    const bool close = chosen >= 0 ? ((uf > acum - tol) || (chosen > 0 && uf < prev + tol)) : (uf < acum + tol);
    comp = chosen;
    a0out = a0;
    return !(unsure || close);
}

// Branch-free certified FP32 decision with a stability margin.  With
// D_k = dc_k + h_k * s (s = num^2, D_0 = 0) the component is the first k with
// u * sum(e) <= c_k (e_k = exp(D_k - max D), c_k the running sums).  Returns
// false when the 700 guards of the log-likelihood differences could matter
// (any difference beyond 600) or when u lies within the certified error tol of
// a boundary; the caller then takes the guarded or the FP64 path.
// On success *w is a margin in log-probability: while the true s moves by Delta
// with H * Delta <= w (H: largest h_k - smallest, h_0 = 0 included), every
// cumulative probability changes by a factor within exp(+-H * Delta), which
// cannot carry a boundary across u, so the decision stays the same.
template <int KM>
__device__ __forceinline__ bool pick_margin(float s, float uf, const float *__restrict__ gcf, int K, int &comp,
                                            float &w)
{
    float D[KM];
    float maxerr = 0.f;
    D[0] = 0.f;
#pragma unroll
    for (int k = 1; k < KM; ++k) {
        const float dc = gcf[2 * k], h = gcf[2 * k + 1];
        D[k] = k < K ? __fmaf_rn(h, s, dc) : -INFINITY;
        maxerr = k < K ? fmaxf(maxerr, 3.0e-7f * (fabsf(dc) + fabsf(h * s))) : maxerr;
    }
    float dmax = 0.f, dmax1 = D[1], dmin1 = D[1];
#pragma unroll
    for (int k = 1; k < KM; ++k) {
        dmax = fmaxf(dmax, D[k]);
        dmax1 = fmaxf(dmax1, D[k]);
        dmin1 = k < K ? fminf(dmin1, D[k]) : dmin1;
    }
    const bool far = (dmax1 - dmin1) < 600.f && dmax1 < 600.f && dmin1 > -600.f;
    float c[KM];
    float run = 0.f;
#pragma unroll
    for (int k = 0; k < KM; ++k) {
        run = __fadd_rn(run, __expf(D[k] - dmax));   // exp(-inf) = 0 beyond K
        c[k] = run;
    }
    const float es = run;
    const float target = uf * es;
    const float tol = (4e-5f + 4.f * maxerr) * es;
    int chosen = 0;
    bool close = false;
    float up = es, lo = 0.f;
#pragma unroll
    for (int k = 0; k < KM; ++k) {
        if (k < K) {
            const bool below = c[k] < target;
            chosen += below ? 1 : 0;
            close = close || fabsf(c[k] - target) < tol;
            lo = below ? c[k] : lo;
        }
    }
#pragma unroll
    for (int k = KM - 1; k >= 0; --k)
        up = (k < K && c[k] >= target) ? c[k] : up;
    comp = chosen < K ? chosen : -1;
    const float w1 = __logf(up - tol) - __logf(target);
    const float w2 = chosen > 0 ? __logf(target) - __logf(lo + tol) : 50.f;
    w = fminf(fminf(w1, w2) - 1e-5f, 50.f);
    return far && !close && chosen < K && w > 0.f;
}

}  // namespace brr
