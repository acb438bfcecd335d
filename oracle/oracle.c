/*
 * CPU oracle for the BayesR Gibbs-sweep path (TEST INFRASTRUCTURE ONLY).
 * Plain C11, FP64, no contraction of a*b+c into fused multiply-adds
 * (built with -ffp-contract=off so x86-64 and aarch64 hosts agree bit for bit).
 * Every function cites the reference file:line it restates; see oracle.h for
 * what is and is not pinned.
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------- */
/* Draw stream.  Philox4x32-10 as published by Salmon, Moraes, Dror and Shaw,
 * "Parallel random numbers: as easy as 1, 2, 3" (SC'11): 10 rounds of the
 * 4x32 S-box with multipliers M0, M1 and Weyl key increments W0, W1. */
#define PHILOX_M0 0xD2511F53u
#define PHILOX_M1 0xCD9E8D57u
#define PHILOX_W0 0x9E3779B9u
#define PHILOX_W1 0xBB67AE85u

void or_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4])
{
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; ++r) {
        const uint64_t p0 = (uint64_t)PHILOX_M0 * c0;
        const uint64_t p1 = (uint64_t)PHILOX_M1 * c2;
        const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        const uint32_t n0 = hi1 ^ c1 ^ k0;
        const uint32_t n1 = lo1;
        const uint32_t n2 = hi0 ^ c3 ^ k1;
        const uint32_t n3 = lo0;
        c0 = n0; c1 = n1; c2 = n2; c3 = n3;
        k0 += PHILOX_W0;
        k1 += PHILOX_W1;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* Stream purposes (the third counter word). */
enum {
    P_INIT = 1,     /* sigmaG initial uniforms        (src/BayesRBase.cpp:60-63) */
    P_MU = 2,       /* intercept normal                (src/DenseBayesRRmz.cpp:39) */
    P_MARKER = 3,   /* per-marker (u, z)               (src/BayesRBase.cpp:106-109) */
    P_PERM = 4,     /* sweep permutation               (src/BayesRBase.cpp:198) */
    P_SIGMAE = 5,   /* residual variance gamma         (src/BayesRBase.cpp:239) */
    P_SIGMAG = 6,   /* genetic variance gamma per group (src/BayesRBase.cpp:245) */
    P_PI = 7        /* Dirichlet gammas per group/comp (src/BayesRBase.cpp:246) */
};

static void block(uint32_t seed, uint32_t chain, uint32_t idx, uint32_t it,
                  uint32_t purpose, uint32_t sub, uint32_t out[4])
{
    const uint32_t ctr[4] = {idx, it, purpose, sub};
    const uint32_t key[2] = {seed, chain};
    or_philox4x32_10(ctr, key, out);
}

double or_u53(uint32_t a, uint32_t b)
{
    /* 27 + 26 random bits, offset by one half: strictly inside (0, 1). */
    return ((double)(a >> 5) * 67108864.0 + (double)(b >> 6) + 0.5) * (1.0 / 9007199254740992.0);
}

static double box_muller(double v1, double v2)
{
    return sqrt(-2.0 * log(v1)) * cos(6.283185307179586 * v2);
}

void or_marker_draws(uint32_t seed, uint32_t chain, uint32_t it, uint32_t j, double *u, double *z)
{
    uint32_t b[4], c[4];
    block(seed, chain, j, it, P_MARKER, 0, b);
    block(seed, chain, j, it, P_MARKER, 1, c);
    *u = or_u53(b[0], b[1]);
    *z = box_muller(or_u53(b[2], b[3]), or_u53(c[0], c[1]));
}

void or_permutation(uint32_t seed, uint32_t chain, uint32_t it, uint32_t M, uint32_t *perm)
{
    for (uint32_t i = 0; i < M; ++i)
        perm[i] = i;
    for (uint32_t i = M; i-- > 1;) {
        uint32_t b[4];
        block(seed, chain, i, it, P_PERM, 0, b);
        const uint64_t r = ((uint64_t)b[0] << 32) | b[1];
        const uint64_t j = (uint64_t)(((unsigned __int128)r * (uint64_t)(i + 1)) >> 64);
        const uint32_t t = perm[i];
        perm[i] = perm[j];
        perm[j] = t;
    }
}

/* Marsaglia & Tsang, "A simple method for generating gamma variables",
 * ACM TOMS 26(3), 2000; shapes below one use the G(a+1) * U^(1/a) boost. */
int or_gamma(uint32_t seed, uint32_t chain, uint32_t it, uint32_t purpose, uint32_t sub,
             double shape, double *out)
{
    if (!(shape > 0.0))
        return OR_ERR_ARG;
    const double a = shape < 1.0 ? shape + 1.0 : shape;
    const double d = a - 1.0 / 3.0;
    const double c = 1.0 / sqrt(9.0 * d);
    for (uint32_t t = 0; t < 1024; ++t) {
        uint32_t b[4], e[4];
        block(seed, chain, t, it, purpose, sub, b);
        block(seed, chain, t, it, purpose, sub | 0x80000000u, e);
        const double x = box_muller(or_u53(b[0], b[1]), or_u53(b[2], b[3]));
        double v = 1.0 + c * x;
        if (v <= 0.0)
            continue;
        v = v * v * v;
        const double u = or_u53(e[0], e[1]);
        const double x2 = x * x;
        if (u < 1.0 - 0.0331 * (x2 * x2) || log(u) < 0.5 * x2 + d * (1.0 - v + log(v))) {
            double g = d * v;
            if (shape < 1.0)
                g = g * pow(or_u53(e[2], e[3]), 1.0 / shape);
            *out = g;
            return OR_OK;
        }
    }
    return OR_ERR_STREAM;
}

/* inverse scaled chi-square (src/distributions_boost.cpp:45-47, :58-60):
 * 1 / Gamma(shape = dof/2, scale = 1 / (dof*scale/2)). */
static int inv_scaled_chisq(uint32_t seed, uint32_t chain, uint32_t it, uint32_t purpose,
                            uint32_t sub, double dof, double scale, double *out)
{
    double g;
    const int rc = or_gamma(seed, chain, it, purpose, sub, 0.5 * dof, &g);
    if (rc)
        return rc;
    const double sc = 1.0 / (0.5 * dof * scale);
    *out = 1.0 / (sc * g);
    return OR_OK;
}

/* ------------------------------------------------------------------------- */
/* Preprocess. */

static inline int64_t col_bytes(int64_t N) { return (N + 3) >> 2; }

/* 2-bit code -> genotype; the bits of a pair are (b[k], b[k+1]) read from the
 * least significant end, allele1 = !b[k], allele2 = !b[k+1]
 * (src/preprocessgraph.cpp:43-56); (allele1, allele2) == (0, 1) is missing
 * (src/densemarkerbuilder.cpp:30). */
static inline int code_to_g(unsigned code)
{
    const unsigned a1 = !(code & 1u);
    const unsigned a2 = !(code & 2u);
    if (a1 == 0 && a2 == 1)
        return -1;
    return (int)(a1 + a2);
}

static inline unsigned code_at(const uint8_t *colp, int64_t i)
{
    return (colp[i >> 2] >> (2 * (i & 3))) & 3u;
}

int or_decode_bed(const uint8_t *bed, int64_t N, int64_t M, int8_t *g)
{
    if (!bed || !g || N <= 0 || M <= 0)
        return OR_ERR_ARG;
    const int64_t cb = col_bytes(N);
    for (int64_t j = 0; j < M; ++j)
        for (int64_t i = 0; i < N; ++i)
            g[j * N + i] = (int8_t)code_to_g(code_at(bed + j * cb, i));
    return OR_OK;
}

int or_marker_counts(const uint8_t *bed, int64_t N, int64_t M, int64_t *counts)
{
    if (!bed || !counts || N <= 0 || M <= 0)
        return OR_ERR_ARG;
    const int64_t cb = col_bytes(N);
    for (int64_t j = 0; j < M; ++j) {
        int64_t c[4] = {0, 0, 0, 0};
        for (int64_t i = 0; i < N; ++i) {
            const int gv = code_to_g(code_at(bed + j * cb, i));
            c[gv < 0 ? 3 : gv] += 1;
        }
        memcpy(counts + 4 * j, c, sizeof c);
    }
    return OR_OK;
}

/* Dense builder (src/densemarkerbuilder.cpp:23-60): missing -> mean of the
 * non-missing genotypes; centre by the column mean; scale so that the squared
 * norm is N-1.  The column takes only four distinct values, so the column mean
 * and the squared norm are restated from the genotype counts in a fixed order:
 *   mean    = S / (N - nm),             S = n1 + 2 n2
 *   colmean = (S + nm*mean) / N
 *   sqn     = n0 c0^2 + n1 c1^2 + n2 c2^2 + nm cm^2,   c_v = v - colmean
 *   x_v     = c_v * (1 / sqrt(sqn / (N - 1)))
 * lut is indexed by the 2-bit BED code: {0: g=2, 1: missing, 2: g=1, 3: g=0}. */
static int dense_lut_from_counts(const int64_t c[4], int64_t N, double lut[4])
{
    const int64_t n0 = c[0], n1 = c[1], n2 = c[2], nm = c[3];
    if (nm >= N)
        return OR_ERR_MARKER;
    const double S = (double)(n1 + 2 * n2);
    const double mean = S / ((double)N - (double)nm);
    const double colmean = (S + (double)nm * mean) / (double)N;
    const double c0 = 0.0 - colmean, c1 = 1.0 - colmean, c2 = 2.0 - colmean, cm = mean - colmean;
    const double sqn = (((double)n0 * (c0 * c0) + (double)n1 * (c1 * c1)) + (double)n2 * (c2 * c2))
                       + (double)nm * (cm * cm);
    if (!(sqn > 0.0))
        return OR_ERR_MARKER;
    const double sigma = 1.0 / sqrt(sqn / ((double)N - 1.0));
    lut[0] = c2 * sigma;
    lut[1] = cm * sigma;
    lut[2] = c1 * sigma;
    lut[3] = c0 * sigma;
    return OR_OK;
}

int or_dense_lut(const uint8_t *bed, int64_t N, int64_t M, double *lut)
{
    if (!bed || !lut || N < 2 || M <= 0)
        return OR_ERR_ARG;
    int64_t *cnt = (int64_t *)malloc(sizeof(int64_t) * 4 * (size_t)M);
    if (!cnt)
        return OR_ERR_ARG;
    int rc = or_marker_counts(bed, N, M, cnt);
    for (int64_t j = 0; rc == OR_OK && j < M; ++j)
        rc = dense_lut_from_counts(cnt + 4 * j, N, lut + 4 * j);
    free(cnt);
    return rc;
}

int or_dense_columns(const uint8_t *bed, int64_t N, int64_t M, double *x)
{
    double *lut = (double *)malloc(sizeof(double) * 4 * (size_t)M);
    if (!lut)
        return OR_ERR_ARG;
    int rc = or_dense_lut(bed, N, M, lut);
    const int64_t cb = col_bytes(N);
    for (int64_t j = 0; rc == OR_OK && j < M; ++j)
        for (int64_t i = 0; i < N; ++i)
            x[j * N + i] = lut[4 * j + code_at(bed + j * cb, i)];
    free(lut);
    return rc;
}

/* Ragged builder statistics (src/sparsemarker.cpp:8-19 accumulates value and
 * value^2 of non-missing genotypes; src/raggedsparsemarkerbuilder.cpp:43-55
 * divides by N including missing and forms the sd). */
static int sparse_stats_from_counts(const int64_t c[4], int64_t N, int eigen, double st[4])
{
    double Zsum = (double)(c[1] + 2 * c[2]);
    double sqrdZ = (double)(c[1] + 4 * c[2]);
    const double Nd = (double)N;
    const double mean = Zsum / Nd;
    if (eigen) {
        /* src/eigensparsemarkerbuilder.cpp:46-56: missing genotypes imputed at
         * the mean in sqrdZ and Zsum before the sd */
        sqrdZ += (mean * mean) * (double)c[3];
        Zsum += mean * (double)c[3];
    }
    const double sd = sqrt(((sqrdZ - (2.0 * mean) * Zsum) + (Nd * mean) * mean) / (Nd - 1.0));
    st[0] = mean;
    st[1] = sd;
    st[2] = sqrdZ;
    st[3] = Zsum;
    /* src/raggedsparsemarker.cpp:68-77 rejects markers with no ones and no twos;
     * a marker with sd == 0 would divide by zero in the sampler. */
    if (c[1] + c[2] == 0 || !(sd > 0.0))
        return OR_ERR_MARKER;
    return OR_OK;
}

static int sparse_stats(const uint8_t *bed, int64_t N, int64_t M, int eigen, double *stats)
{
    if (!bed || !stats || N < 2 || M <= 0)
        return OR_ERR_ARG;
    int64_t *cnt = (int64_t *)malloc(sizeof(int64_t) * 4 * (size_t)M);
    if (!cnt)
        return OR_ERR_ARG;
    int rc = or_marker_counts(bed, N, M, cnt);
    for (int64_t j = 0; rc == OR_OK && j < M; ++j)
        rc = sparse_stats_from_counts(cnt + 4 * j, N, eigen, stats + 4 * j);
    free(cnt);
    return rc;
}

int or_ragged_stats(const uint8_t *bed, int64_t N, int64_t M, double *stats)
{
    return sparse_stats(bed, N, M, 0, stats);
}

int or_eigen_stats(const uint8_t *bed, int64_t N, int64_t M, double *stats)
{
    return sparse_stats(bed, N, M, 1, stats);
}

/* Index lists in ascending individual order (src/raggedsparsemarkerbuilder.cpp:25-41). */
int or_ragged_lists(const uint8_t *bed, int64_t N, int64_t M,
                    int64_t *off_ones, int32_t *ones,
                    int64_t *off_twos, int32_t *twos,
                    int64_t *off_miss, int32_t *miss)
{
    if (!bed || N <= 0 || M <= 0)
        return OR_ERR_ARG;
    const int64_t cb = col_bytes(N);
    int64_t a = 0, b = 0, m = 0;
    for (int64_t j = 0; j < M; ++j) {
        off_ones[j] = a;
        off_twos[j] = b;
        off_miss[j] = m;
        for (int64_t i = 0; i < N; ++i) {
            const int gv = code_to_g(code_at(bed + j * cb, i));
            if (gv == 1)
                ones[a++] = (int32_t)i;
            else if (gv == 2)
                twos[b++] = (int32_t)i;
            else if (gv < 0)
                miss[m++] = (int32_t)i;
        }
    }
    off_ones[M] = a;
    off_twos[M] = b;
    off_miss[M] = m;
    return OR_OK;
}

/* ------------------------------------------------------------------------- */
/* Chain. */

struct or_markers {
    int kind;
    int64_t N, M;
    double *x;          /* dense: M x N standardized columns (dense_lut == 0) */
    double *lut;        /* dense: M x 4 standardized value per 2-bit code (dense_lut != 0) */
    const uint8_t *bed; /* dense_lut != 0: the problem's BED payload */
    double *stats;      /* ragged: M x {mean, sd, sqrdZ, Zsum} */
    int64_t *off[3];    /* ragged: ones, twos, missing offsets (M+1 each) */
    int32_t *idx[3];
};

void or_markers_destroy(or_markers *m)
{
    if (!m)
        return;
    free(m->x);
    free(m->lut);
    free(m->stats);
    for (int k = 0; k < 3; ++k) {
        free(m->off[k]);
        free(m->idx[k]);
    }
    free(m);
}

int or_markers_create(const or_problem *p, or_markers **out)
{
    if (!p || !out || p->N < 2 || p->M <= 0)
        return OR_ERR_ARG;
    or_markers *m = (or_markers *)calloc(1, sizeof(or_markers));
    if (!m)
        return OR_ERR_ARG;
    m->kind = p->kind;
    m->N = p->N;
    m->M = p->M;
    int rc = OR_OK;
    if (p->kind == OR_KIND_DENSE && p->dense_lut) {
        m->lut = (double *)malloc(sizeof(double) * 4 * (size_t)p->M);
        m->bed = p->bed;
        rc = m->lut ? or_dense_lut(p->bed, p->N, p->M, m->lut) : OR_ERR_ARG;
    } else if (p->kind == OR_KIND_DENSE) {
        m->x = (double *)malloc(sizeof(double) * (size_t)p->N * (size_t)p->M);
        rc = m->x ? or_dense_columns(p->bed, p->N, p->M, m->x) : OR_ERR_ARG;
    } else if (p->kind == OR_KIND_RAGGED || p->kind == OR_KIND_EIGEN) {
        int64_t *cnt = (int64_t *)malloc(sizeof(int64_t) * 4 * (size_t)p->M);
        m->stats = (double *)malloc(sizeof(double) * 4 * (size_t)p->M);
        rc = (cnt && m->stats) ? or_marker_counts(p->bed, p->N, p->M, cnt) : OR_ERR_ARG;
        int64_t tot[3] = {0, 0, 0};
        for (int64_t j = 0; rc == OR_OK && j < p->M; ++j) {
            tot[0] += cnt[4 * j + 1];
            tot[1] += cnt[4 * j + 2];
            tot[2] += cnt[4 * j + 3];
            rc = sparse_stats_from_counts(cnt + 4 * j, p->N, p->kind == OR_KIND_EIGEN, m->stats + 4 * j);
        }
        for (int k = 0; rc == OR_OK && k < 3; ++k) {
            m->off[k] = (int64_t *)malloc(sizeof(int64_t) * (size_t)(p->M + 1));
            m->idx[k] = (int32_t *)malloc(sizeof(int32_t) * (size_t)(tot[k] + 1));
            if (!m->off[k] || !m->idx[k])
                rc = OR_ERR_ARG;
        }
        if (rc == OR_OK)
            rc = or_ragged_lists(p->bed, p->N, p->M, m->off[0], m->idx[0], m->off[1], m->idx[1],
                                 m->off[2], m->idx[2]);
        free(cnt);
    } else {
        rc = OR_ERR_ARG;
    }
    if (rc != OR_OK) {
        or_markers_destroy(m);
        return rc;
    }
    *out = m;
    return OR_OK;
}

/* src/BayesRBase.cpp:39-99 (plus runGibbs zeroing m_components, :181). */
int or_init(const or_problem *p, or_state *s)
{
    if (!p || !s || p->N < 2 || p->M <= 0 || p->n_groups <= 0 || p->n_groups > OR_MAX_GROUPS)
        return OR_ERR_ARG;
    const int64_t N = p->N, M = p->M;
    for (int g = 0; g < p->n_groups; ++g) {
        const int K = p->K[g];
        if (K < 2 || K > OR_MAX_K)
            return OR_ERR_ARG;
        /* prior pi: every entry 0.5/K, then entry 0 set to 0.5 (src/BayesRBase.cpp:43-48) */
        for (int k = 0; k < OR_MAX_K; ++k)
            s->pi[g * OR_MAX_K + k] = k < K ? 0.5 / (double)K : 0.0;
        s->pi[g * OR_MAX_K] = 0.5;
        uint32_t b[4];
        block(p->seed, p->chain, (uint32_t)g, 0, P_INIT, 0, b);
        s->sigmaG[g] = or_u53(b[0], b[1]);
    }
    for (int64_t j = 0; j < M; ++j) {
        s->beta[j] = 0.0;
        s->acum[j] = 0.0;
        s->comp[j] = 0;
    }
    s->mu = 0.0;
    /* y standardized (src/BayesRBase.cpp:85-86); y was read as float (src/data.cpp:348). */
    double ysum = 0.0;
    for (int64_t i = 0; i < N; ++i)
        ysum += (double)p->y[i];
    const double ymean = ysum / (double)N;
    double sq = 0.0;
    for (int64_t i = 0; i < N; ++i) {
        const double d = (double)p->y[i] - ymean;
        s->eps[i] = d;
        sq += d * d;
    }
    const double scale = sqrt(sq / (double)(N - 1));
    double esq = 0.0, esum = 0.0;
    for (int64_t i = 0; i < N; ++i) {
        s->eps[i] = s->eps[i] / scale;
        s->eps[i] = s->eps[i] - s->mu;           /* (src/BayesRBase.cpp:88) */
        esq += s->eps[i] * s->eps[i];
        esum += s->eps[i];
    }
    s->sigmaE = esq / (double)N * 0.5;           /* (src/BayesRBase.cpp:89) */
    s->epsSum = esum;                            /* (src/BayesRBase.cpp:90) */
    s->m0 = 0.0;
    memset(s->v, 0, sizeof s->v);
    memset(s->betasqnG, 0, sizeof s->betasqnG);
    return OR_OK;
}

/* BayesRBase::processColumn (src/BayesRBase.cpp:287-392) with the dense
 * kernel (src/densebayesrkernel.cpp:10-20) or the ragged kernel
 * (src/sparsebayesrkernel.cpp:10-34, src/raggedbayesrkernel.cpp:10-35,
 * src/SparseBayesRRG.cpp:76-92). */
/* The sampling half of processColumn (src/BayesRBase.cpp:287-366) for marker j
 * against the current residual: the new beta, component, component counts and
 * squared effects; acum (P(component 0)) is stored when write_acum is set, as
 * the synchronous processColumn does (:341) and processColumnAsync does not
 * (:394-496).  Returns the new beta; *beta_old_out gets the old one. */
static double column_pick(const or_problem *p, const or_markers *mk, or_state *s,
                          uint32_t j, double p_u, double z, int write_acum, double *beta_old_out)
{
    const int64_t N = p->N;
    const double NM1 = (double)(N - 1);
    const int g = p->group[j];
    const int K = p->K[g];
    const int km1 = K - 1;
    const double *Srow = p->S + (size_t)g * (OR_MAX_K - 1);
    double cVa[OR_MAX_K], cVaI[OR_MAX_K], denom[OR_MAX_K], muk[OR_MAX_K], logL[OR_MAX_K + 1];
    const double beta_old = s->beta[j];
    const double sigmaG = s->sigmaG[g];
    cVa[0] = 0.0;
    cVaI[0] = 0.0;
    for (int k = 1; k < K; ++k) {
        cVa[k] = Srow[k - 1];
        cVaI[k] = 1.0 / cVa[k];
    }
    const double sigmaEOverSigmaG = s->sigmaE / sigmaG;
    for (int k = 1; k < K; ++k)
        denom[k - 1] = NM1 + sigmaEOverSigmaG * cVaI[k];

    double num;
    if (mk->kind == OR_KIND_DENSE && mk->lut) {
        /* the same column values as below, read through the code table */
        const double *lut = mk->lut + 4 * (size_t)j;
        const uint8_t *col = mk->bed + (size_t)j * (size_t)col_bytes(N);
        double dot = 0.0;
        for (int64_t i = 0; i < N; ++i)
            dot += lut[code_at(col, i)] * s->eps[i];
        num = dot + beta_old * (double)(N - 1);
    } else if (mk->kind == OR_KIND_DENSE) {
        const double *x = mk->x + (size_t)j * (size_t)N;
        double dot = 0.0;
        for (int64_t i = 0; i < N; ++i)
            dot += x[i] * s->eps[i];
        num = dot + beta_old * (double)(N - 1);
    } else {
        const double mean = mk->stats[4 * j + 0], sd = mk->stats[4 * j + 1];
        double s1 = 0.0, s2 = 0.0;
        for (int64_t q = mk->off[0][j]; q < mk->off[0][j + 1]; ++q)
            s1 += s->eps[mk->idx[0][q]];
        for (int64_t q = mk->off[1][j]; q < mk->off[1][j + 1]; ++q)
            s2 += s->eps[mk->idx[1][q]];
        double zdot = s1 + 2.0 * s2;
        if (mk->kind == OR_KIND_EIGEN) {
            /* Zg.dot(epsilon) over the stored entries in ascending individual
             * order, Zg = 1, 2, or the mean at missing genotypes
             * (src/eigensparsemarkerbuilder.cpp:62-72, src/eigenbayesrkernel.cpp:17-20) */
            int64_t q[3], e[3];
            for (int k = 0; k < 3; ++k) {
                q[k] = mk->off[k][j];
                e[k] = mk->off[k][j + 1];
            }
            const double val[3] = {1.0, 2.0, mean};
            zdot = 0.0;
            for (;;) {
                int kb = -1;
                for (int k = 0; k < 3; ++k)
                    if (q[k] < e[k] && (kb < 0 || mk->idx[k][q[k]] < mk->idx[kb][q[kb]]))
                        kb = k;
                if (kb < 0)
                    break;
                zdot += val[kb] * s->eps[mk->idx[kb][q[kb]++]];
            }
        }
        const double dot = zdot / sd;
        num = (beta_old * ((double)N - 1.0) - (mean * s->epsSum) / sd) + dot;
    }

    muk[0] = 0.0;
    for (int k = 1; k < K; ++k)
        muk[k] = num / denom[k - 1];
    const double logLScale = sigmaG / s->sigmaE * NM1;
    for (int k = 0; k < K; ++k)
        logL[k] = log(s->pi[g * OR_MAX_K + k]);
    for (int k = 1; k < K; ++k)
        logL[k] = (logL[k] - 0.5 * log(logLScale * cVa[k] + 1.0)) + (0.5 * (muk[k] * num)) / s->sigmaE;

    /* acum = P(component 0), zero when any log-likelihood gap exceeds 700 (:335-339) */
    double acum;
    int big = 0;
    for (int k = 1; k < K; ++k)
        if (fabs(logL[k] - logL[0]) > 700.0)
            big = 1;
    if (big) {
        acum = 0.0;
    } else {
        double sum = 0.0;
        for (int k = 0; k < K; ++k)
            sum += exp(logL[k] - logL[0]);
        acum = 1.0 / sum;
    }
    if (write_acum)
        s->acum[j] = acum;

    /* inverse-CDF walk (:346-366).  The reference evaluates the guard for
     * k = K-1 against logL[K], one past the end; the resulting acum is never
     * read again, so that step is omitted. */
    double beta_new = beta_old;
    for (int k = 0; k < K; ++k) {
        if (p_u <= acum) {
            if (k == 0) {
                beta_new = 0.0;
            } else {
                beta_new = z * sqrt(s->sigmaE / denom[k - 1]) + muk[k];
                s->betasqnG[g] += beta_new * beta_new;
            }
            s->v[g * OR_MAX_K + k] += 1.0;
            s->comp[j] = k;
            break;
        } else if (k + 1 < K) {
            int over = 0;
            for (int q = 1; q < K; ++q)
                if (fabs(logL[q] - logL[k + 1]) > 700.0)
                    over = 1;
            if (!over) {
                double sum = 0.0;
                for (int q = 0; q < K; ++q)
                    sum += exp(logL[q] - logL[k + 1]);
                acum += 1.0 / sum;
            }
        }
    }
    s->beta[j] = beta_new;
    *beta_old_out = beta_old;
    return beta_new;
}

/* The residual half (src/BayesRBase.cpp:368-378, the kernels' epsilon change
 * and the running epsilon sum): nothing when the marker stays out of the
 * model. */
static void column_update(const or_problem *p, const or_markers *mk, or_state *s,
                          uint32_t j, double beta_old, double beta_new)
{
    const int64_t N = p->N;
    if (beta_old == 0.0 && beta_new == 0.0)
        return;                                   /* (:372) */
    const double dBeta = beta_old - beta_new;
    if (mk->kind == OR_KIND_DENSE && mk->lut) {
        const double *lut = mk->lut + 4 * (size_t)j;
        const uint8_t *col = mk->bed + (size_t)j * (size_t)col_bytes(N);
        for (int64_t i = 0; i < N; ++i)
            s->eps[i] = s->eps[i] + dBeta * lut[code_at(col, i)];
    } else if (mk->kind == OR_KIND_DENSE) {
        const double *x = mk->x + (size_t)j * (size_t)N;
        for (int64_t i = 0; i < N; ++i)
            s->eps[i] = s->eps[i] + dBeta * x[i];
    } else {
        const double mean = mk->stats[4 * j + 0], sd = mk->stats[4 * j + 1];
        const double Zsum = mk->stats[4 * j + 3];
        const double meanAdj = dBeta * mean / sd;
        const double oneAdj = dBeta / sd;
        /* delta starts at -meanAdj everywhere; ones/twos/missing adjusted in turn */
        double *delta = (double *)malloc(sizeof(double) * (size_t)N);
        for (int64_t i = 0; i < N; ++i)
            delta[i] = -meanAdj;
        for (int64_t q = mk->off[0][j]; q < mk->off[0][j + 1]; ++q)
            delta[mk->idx[0][q]] += oneAdj;
        for (int64_t q = mk->off[1][j]; q < mk->off[1][j + 1]; ++q)
            delta[mk->idx[1][q]] += 2.0 * oneAdj;
        for (int64_t q = mk->off[2][j]; q < mk->off[2][j + 1]; ++q)
            delta[mk->idx[2][q]] += meanAdj;
        for (int64_t i = 0; i < N; ++i)
            s->eps[i] = s->eps[i] + delta[i];
        free(delta);
        /* running epsilon sum (src/sparsebayesrkernel.cpp:29-34, src/SparseBayesRRG.cpp:91) */
        s->epsSum += (dBeta * Zsum) / sd - ((dBeta * mean) * (double)N) / sd;
    }
}

static void process_column(const or_problem *p, const or_markers *mk, or_state *s,
                           uint32_t j, double p_u, double z)
{
    double beta_old;
    const double beta_new = column_pick(p, mk, s, j, p_u, z, 1, &beta_old);
    column_update(p, mk, s, j, beta_old, beta_new);
}

int or_sweep(const or_problem *p, const or_markers *mk, or_state *s,
             const uint32_t *order, const double *u, const double *z)
{
    if (p->async_batch <= 0) {
        for (int64_t q = 0; q < p->M; ++q) {
            const uint32_t j = order[q];
            process_column(p, mk, s, j, u[j], z[j]);
        }
        return OR_OK;
    }
    /* asyncppbayes (src/parallelgraph.cpp:51-150, src/BayesRBase.cpp:394-524):
     * the ParallelGraph keeps up to analysisTokens markers in flight and lets the
     * next ones start when all have returned.  The schedule restated here is
     * the one where every marker of a batch of async_batch consecutive markers
     * reads the residual (and the running residual sum) before any of them
     * writes: all picks of the batch first, then the updates in sweep order. */
    const int64_t T = p->async_batch;
    double bo[OR_MAX_ASYNC], bn[OR_MAX_ASYNC];
    if (T > OR_MAX_ASYNC)
        return OR_ERR_ARG;
    for (int64_t q0 = 0; q0 < p->M; q0 += T) {
        const int64_t q1 = q0 + T < p->M ? q0 + T : p->M;
        for (int64_t q = q0; q < q1; ++q) {
            const uint32_t j = order[q];
            bn[q - q0] = column_pick(p, mk, s, j, u[j], z[j], 0, &bo[q - q0]);
        }
        for (int64_t q = q0; q < q1; ++q)
            column_update(p, mk, s, order[q], bo[q - q0], bn[q - q0]);
    }
    return OR_OK;
}

int or_iterate(const or_problem *p, const or_markers *mk, or_state *s, uint32_t it)
{
    const int64_t N = p->N, M = p->M;
    const double Nd = (double)N;
    /* updateMu: dense src/DenseBayesRRmz.cpp:36-42, sparse src/SparseBayesRRG.cpp:106-113 */
    {
        const double old_mu = s->mu;
        for (int64_t i = 0; i < N; ++i)
            s->eps[i] = s->eps[i] + s->mu;
        double mean;
        if (p->kind == OR_KIND_DENSE) {
            double sum = 0.0;
            for (int64_t i = 0; i < N; ++i)
                sum += s->eps[i];
            mean = sum / Nd;
        } else {
            s->epsSum += old_mu * Nd;
            mean = s->epsSum / Nd;
        }
        uint32_t b[4];
        block(p->seed, p->chain, 0, it, P_MU, 0, b);
        const double zmu = box_muller(or_u53(b[0], b[1]), or_u53(b[2], b[3]));
        s->mu = mean + sqrt(s->sigmaE / Nd) * zmu;
        for (int64_t i = 0; i < N; ++i)
            s->eps[i] = s->eps[i] - s->mu;
        if (p->kind != OR_KIND_DENSE)
            s->epsSum -= s->mu * Nd;
    }
    /* per-marker draws and permutation (src/BayesRBase.cpp:196-198) */
    double *u = (double *)malloc(sizeof(double) * (size_t)M);
    double *z = (double *)malloc(sizeof(double) * (size_t)M);
    uint32_t *order = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)M);
    if (!u || !z || !order) {
        free(u); free(z); free(order);
        return OR_ERR_ARG;
    }
    for (int64_t j = 0; j < M; ++j)
        or_marker_draws(p->seed, p->chain, it, (uint32_t)j, &u[j], &z[j]);
    or_permutation(p->seed, p->shared_perm ? p->perm_chain : p->chain, it, (uint32_t)M, order);
    s->m0 = 0.0;
    memset(s->v, 0, sizeof s->v);
    memset(s->betasqnG, 0, sizeof s->betasqnG);
    or_sweep(p, mk, s, order, u, z);
    free(u); free(z); free(order);

    /* sigmaE (src/BayesRBase.cpp:238-239) */
    double esq = 0.0;
    for (int64_t i = 0; i < N; ++i)
        esq += s->eps[i] * s->eps[i];
    int rc = inv_scaled_chisq(p->seed, p->chain, it, P_SIGMAE, 0, p->v0E + Nd,
                              (esq + p->v0E * p->s02E) / (p->v0E + Nd), &s->sigmaE);
    if (rc)
        return rc;
    /* sigmaG and pi per group (src/BayesRBase.cpp:243-247) */
    for (int g = 0; g < p->n_groups; ++g) {
        const int K = p->K[g];
        double vs = 0.0;
        for (int k = 0; k < K; ++k)
            vs += s->v[g * OR_MAX_K + k];
        const double m0 = vs - s->v[g * OR_MAX_K];
        s->m0 = m0;
        rc = inv_scaled_chisq(p->seed, p->chain, it, P_SIGMAG, (uint32_t)g, p->v0G + m0,
                              (s->betasqnG[g] * m0 + p->v0G * p->s02G) / (p->v0G + m0),
                              &s->sigmaG[g]);
        if (rc)
            return rc;
        double r[OR_MAX_K], rs = 0.0;
        for (int k = 0; k < K; ++k) {
            double gk;
            rc = or_gamma(p->seed, p->chain, it, P_PI, (uint32_t)(g * 256 + k),
                          s->v[g * OR_MAX_K + k] + 1.0, &gk);
            if (rc)
                return rc;
            r[k] = 1.0 * gk;
            rs += r[k];
        }
        for (int k = 0; k < K; ++k)
            s->pi[g * OR_MAX_K + k] = r[k] / rs;
    }
    return OR_OK;
}
