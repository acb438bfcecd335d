// Test driver of the GPU adapter: a stand-in for the reference's BayesRBase
// that runs the runGibbs loop body (src/BayesRBase.cpp:186-247) on the host,
// with its state in host vectors as the reference keeps it, and hands the
// sweep to GpuSweepGraph::exec.  The markers come through GpuMarkerBuilder,
// fed from a PLINK .bed file the way the preprocess graph decodes it
// (src/preprocessgraph.cpp:24-60).  The draws replay the counter-based stream
// of brr_stream.h, so the chain is comparable with the FP64 oracle.
//
//   adapter_harness <file.bed> <pheno.f32> <groups.i32> N M kind form gram
//                   "S1;S2;..." seed iterations <trace.out>
//
// trace.out: per iteration M betas, M components, sigmaE, the G sigmaG, mu
// (doubles).
#include <array>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "../bayesrrcmd_gb300/adapter/gpu_adapter.h"
#include "../bayesrrcmd_gb300/csrc/brr_stream.h"

namespace {

std::vector<std::vector<double>> parse_S(const std::string &spec)
{
    std::vector<std::vector<double>> out;
    std::stringstream groups(spec);
    std::string g;
    while (std::getline(groups, g, ';')) {
        std::vector<double> row;
        std::stringstream vals(g);
        std::string v;
        while (std::getline(vals, v, ','))
            row.push_back(std::atof(v.c_str()));
        out.push_back(row);
    }
    return out;
}

// Fisher-Yates over the stream (the permutation the library and the oracle use)
void permutation(brr::StreamKey key, uint32_t it, uint32_t M, std::vector<unsigned> &perm)
{
    perm.resize(M);
    for (uint32_t i = 0; i < M; ++i)
        perm[i] = i;
    for (uint32_t i = M; i-- > 1;) {
        const brr::U4 b = brr::stream_block(key, i, it, brr::kPurposePerm, 0);
        const uint64_t r = ((uint64_t)b.x << 32) | b.y;
        const uint64_t j = (uint64_t)(((unsigned __int128)r * (uint64_t)(i + 1)) >> 64);
        std::swap(perm[i], perm[j]);
    }
}

class HarnessBayesR : public Analysis, public BayesRSweepAccess
{
public:
    HarnessBayesR(unsigned N, unsigned M, int kind, const std::vector<float> &y, const std::vector<int32_t> &group,
                  const std::vector<std::vector<double>> &S, uint32_t seed)
        : N(N), M(M), kind(kind), group(group), S(S), key{seed, 0u}
    {
        const int G = (int)S.size();
        // BayesRBase::init (src/BayesRBase.cpp:39-99)
        m_pi.assign(G, std::vector<double>());
        for (int g = 0; g < G; ++g) {
            const int K = (int)S[g].size() + 1;
            m_pi[g].assign(K, 0.5 / K);
            m_pi[g][0] = 0.5;
        }
        m_v.assign(G, std::vector<double>(BRR_MAX_K, 0.0));
        m_betasqnG.assign(G, 0.0);
        m_sigmaG.resize(G);
        for (int g = 0; g < G; ++g)
            m_sigmaG[g] = brr::uniform_init(key, (uint32_t)g);
        m_beta.assign(M, 0.0);
        m_acum.assign(M, 0.0);
        m_components.assign(M, 0.0);
        double mean = 0.0;
        for (float v : y)
            mean += (double)v;
        mean /= (double)N;
        std::vector<double> ys(N);
        double sq = 0.0;
        for (unsigned i = 0; i < N; ++i) {
            ys[i] = (double)y[i] - mean;
            sq += ys[i] * ys[i];
        }
        const double sd = std::sqrt(sq / (double)(N - 1));
        m_epsilon.resize(N);
        double esq = 0.0, esum = 0.0;
        for (unsigned i = 0; i < N; ++i) {
            m_epsilon[i] = ys[i] / sd - m_mu;
            esq += m_epsilon[i] * m_epsilon[i];
            esum += m_epsilon[i];
        }
        m_sigmaE = esq / (double)N * 0.5;
        m_epsilonSum = esum;
        m_randomNumbers.resize(M);
    }

    // ---- BayesRSweepAccess
    const std::vector<std::array<double, 2>> &markerDraws() const override { return m_randomNumbers; }
    double mu() const override { return m_mu; }
    double sigmaE() const override { return m_sigmaE; }
    double sigmaG(int g) const override { return m_sigmaG[g]; }
    double pi(int g, int k) const override { return m_pi[g][k]; }
    int mixtureSize(int g) const override { return g < (int)S.size() ? (int)S[g].size() + 1 : 0; }
    double *beta() override { return m_beta.data(); }
    double *components() override { return m_components.data(); }
    double *acum() override { return m_acum.data(); }
    double *epsilon() override { return m_epsilon.data(); }
    double &epsilonSum() override { return m_epsilonSum; }
    void setComponentCount(int g, int k, double c) override { m_v[g][k] = c; }
    void setBetaSquaredNorm(int g, double v) override { m_betasqnG[g] = v; }

    void processColumn(const KernelPtr &) override {}

    // the runGibbs loop body with the analysis graph's exec in its place
    int runGibbs(AnalysisGraph *graph) override
    {
        const double Nd = (double)N;
        std::vector<unsigned> order;
        for (unsigned it = 0; it < iterations; ++it) {
            // updateMu: dense src/DenseBayesRRmz.cpp:36-42, sparse src/SparseBayesRRG.cpp:106-113
            const double old_mu = m_mu;
            for (auto &e : m_epsilon)
                e = e + m_mu;
            double mean;
            if (kind == BRR_KIND_DENSE) {
                double s = 0.0;
                for (double e : m_epsilon)
                    s += e;
                mean = s / Nd;
            } else {
                m_epsilonSum += old_mu * Nd;
                mean = m_epsilonSum / Nd;
            }
            m_mu = mean + std::sqrt(m_sigmaE / Nd) * brr::normal_mu(key, it);
            for (auto &e : m_epsilon)
                e = e - m_mu;
            if (kind != BRR_KIND_DENSE)
                m_epsilonSum -= m_mu * Nd;
            // prepareForAnylsis and the shuffle (src/BayesRBase.cpp:101-110, :198)
            for (unsigned j = 0; j < M; ++j)
                brr::marker_draws(key, it, j, &m_randomNumbers[j][0], &m_randomNumbers[j][1]);
            permutation(key, it, M, order);
            for (auto &row : m_v)
                std::fill(row.begin(), row.end(), 0.0);
            std::fill(m_betasqnG.begin(), m_betasqnG.end(), 0.0);
            graph->exec(this, N, M, order);
            if (static_cast<GpuSweepGraph *>(graph)->status() != BRR_OK)
                return 1;
            // sigmaE, sigmaG, pi (src/BayesRBase.cpp:237-247)
            double esq = 0.0;
            for (double e : m_epsilon)
                esq += e * e;
            if (!brr::inv_scaled_chisq(key, it, brr::kPurposeSigmaE, 0, v0E + Nd, (esq + v0E * s02E) / (v0E + Nd),
                                       &m_sigmaE))
                return 2;
            for (size_t g = 0; g < S.size(); ++g) {
                const int K = (int)S[g].size() + 1;
                double vs = 0.0;
                for (int k = 0; k < K; ++k)
                    vs += m_v[g][k];
                const double m0 = vs - m_v[g][0];
                if (!brr::inv_scaled_chisq(key, it, brr::kPurposeSigmaG, (uint32_t)g, v0G + m0,
                                           (m_betasqnG[g] * m0 + v0G * s02G) / (v0G + m0), &m_sigmaG[g]))
                    return 2;
                double r[BRR_MAX_K], rs = 0.0;
                for (int k = 0; k < K; ++k) {
                    double gk;
                    if (!brr::gamma_draw(key, it, brr::kPurposePi, (uint32_t)(g * 256 + k), m_v[g][k] + 1.0, &gk))
                        return 2;
                    r[k] = 1.0 * gk;
                    rs += r[k];
                }
                for (int k = 0; k < K; ++k)
                    m_pi[g][k] = r[k] / rs;
            }
            // the sample row (src/BayesRBase.cpp:250-253)
            trace.insert(trace.end(), m_beta.begin(), m_beta.end());
            trace.insert(trace.end(), m_components.begin(), m_components.end());
            trace.push_back(m_sigmaE);
            trace.insert(trace.end(), m_sigmaG.begin(), m_sigmaG.end());
            trace.push_back(m_mu);
        }
        return 0;
    }

    unsigned iterations = 0;
    std::vector<double> trace;

private:
    unsigned N, M;
    int kind;
    std::vector<int32_t> group;
    std::vector<std::vector<double>> S;
    brr::StreamKey key;
    const double v0E = 1e-4, s02E = 1e-4, v0G = 1e-4, s02G = 1e-4;
    double m_mu = 0.0, m_sigmaE = 0.0, m_epsilonSum = 0.0;
    std::vector<double> m_sigmaG, m_beta, m_acum, m_components, m_epsilon, m_betasqnG;
    std::vector<std::vector<double>> m_pi, m_v;
    std::vector<std::array<double, 2>> m_randomNumbers;
};

template <class T>
std::vector<T> read_raw(const char *path, size_t n)
{
    std::vector<T> v(n);
    std::ifstream f(path, std::ios::binary);
    f.read(reinterpret_cast<char *>(v.data()), (std::streamsize)(n * sizeof(T)));
    if (!f)
        v.clear();
    return v;
}

}  // namespace

int main(int argc, char **argv)
{
    if (argc != 13) {
        std::cerr << "usage: adapter_harness bed pheno groups N M kind form gram S seed iterations out" << std::endl;
        return 64;
    }
    const unsigned N = (unsigned)std::atoi(argv[4]), M = (unsigned)std::atoi(argv[5]);
    const int kind = std::atoi(argv[6]), form = std::atoi(argv[7]), gram = std::atoi(argv[8]);
    const auto S = parse_S(argv[9]);
    const uint32_t seed = (uint32_t)std::atoi(argv[10]);
    const unsigned iterations = (unsigned)std::atoi(argv[11]);
    const auto y = read_raw<float>(argv[2], N);
    const auto group = read_raw<int32_t>(argv[3], M);
    if (y.empty() || group.empty() || S.empty()) {
        std::cerr << "cannot read the phenotype, the groups or S" << std::endl;
        return 65;
    }

    // the preprocess graph's decode loop feeding the GPU marker builder
    GpuMarkerBuilder builder(N, M);
    {
        std::ifstream bed(argv[1], std::ios::binary);
        char magic[3];
        bed.read(magic, 3);
        if (!bed || magic[0] != 0x6c || magic[1] != 0x1b || magic[2] != 0x01) {
            std::cerr << "not a SNP-major PLINK .bed file" << std::endl;
            return 65;
        }
        for (unsigned j = 0; j < M; ++j) {
            builder.initialise(j, N);
            for (unsigned i = 0; i < N;) {
                char ch;
                bed.read(&ch, 1);
                if (!bed) {
                    std::cerr << "Error: problem with the BED file" << std::endl;
                    return 65;
                }
                const unsigned b = (unsigned char)ch;
                for (unsigned k = 0; k < 7 && i < N; k += 2, ++i)
                    builder.processAllele(i, !((b >> k) & 1u), !((b >> (k + 1)) & 1u));
            }
            builder.endColumn();
            if (!builder.build())
                return 66;
        }
    }

    brr_config cfg{};
    cfg.N = N;
    cfg.M = M;
    cfg.kind = kind;
    cfg.form = form;
    cfg.n_groups = (int32_t)S.size();
    for (size_t g = 0; g < S.size(); ++g) {
        cfg.K[g] = (int32_t)S[g].size() + 1;
        for (size_t k = 0; k < S[g].size(); ++k)
            cfg.S[g * (BRR_MAX_K - 1) + k] = S[g][k];
    }
    cfg.seed = seed;
    cfg.chain = 0;
    cfg.v0E = cfg.s02E = cfg.v0G = cfg.s02G = 1e-4;
    cfg.refresh_every = form == BRR_FORM_FP32C ? 3 : 0;
    cfg.gram = gram;
    brr_ctx *ctx = nullptr;
    if (brr_ctx_create(&cfg, &ctx) != BRR_OK) {
        std::cerr << brr_last_error() << std::endl;
        return 67;
    }
    int rc = builder.pack(ctx);
    GpuSweepGraph graph(ctx);
    if (!rc)
        rc = graph.setGroups(group.data());
    if (!rc)
        rc = graph.setPhenotype(y.data());
    HarnessBayesR analysis(N, M, kind, y, group, S, seed);
    analysis.iterations = iterations;
    if (!rc)
        rc = analysis.runGibbs(&graph);
    brr_ctx_destroy(ctx);
    if (rc) {
        std::cerr << "chain failed (" << rc << ")" << std::endl;
        return 68;
    }
    std::ofstream out(argv[12], std::ios::binary);
    out.write(reinterpret_cast<const char *>(analysis.trace.data()),
              (std::streamsize)(analysis.trace.size() * sizeof(double)));
    std::printf("adapter chain: %u iterations, last sweep %.3f ms\n", iterations, graph.lastSweepMs());
    return out ? 0 : 69;
}
