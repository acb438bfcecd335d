// GpuMarkerBuilder and GpuSweepGraph over libbrr_gpu.so (interfaces in
// gpu_adapter.h).
#include "gpu_adapter.h"

#include <cstring>
#include <iostream>

// ---------------------------------------------------------------------------
// GpuMarkerBuilder

GpuMarkerBuilder::GpuMarkerBuilder(unsigned int numInds, unsigned int numSnps)
    : m_inds(numInds), m_snps(numSnps), m_colBytes((numInds + 3u) / 4u),
      // 0x55: the missing code 01 in all four slots, so individuals the
      // preprocess graph skips (not kept) stay missing
      m_bed((size_t)numSnps * ((numInds + 3u) / 4u), 0x55), m_ended(numSnps, 0)
{
}

void GpuMarkerBuilder::initialise(const unsigned int snp, const unsigned int numInds)
{
    MarkerBuilder::initialise(snp, numInds);
    if (snp >= m_snps || numInds != m_inds) {
        std::cerr << "GpuMarkerBuilder: column " << snp << " of " << numInds << " individuals does not fit the "
                  << m_snps << " x " << m_inds << " batch" << std::endl;
        m_marker.reset();
        return;
    }
    std::memset(m_bed.data() + (size_t)snp * m_colBytes, 0x55, m_colBytes);
    m_ended[snp] = 0;
    auto mk = std::make_unique<GpuMarker>();
    mk->i = snp;
    mk->numInds = numInds;
    m_marker = std::move(mk);
}

void GpuMarkerBuilder::processAllele(unsigned int individual, unsigned int allele1, unsigned int allele2)
{
    if (!m_marker || individual >= m_inds)
        return;
    // the BED bits are the negated alleles: bit 2i = !allele1, bit 2i+1 = !allele2
    const unsigned code = (allele1 ? 0u : 1u) | (allele2 ? 0u : 2u);
    uint8_t &byte = m_bed[(size_t)m_snp * m_colBytes + (individual >> 2)];
    const unsigned shift = 2u * (individual & 3u);
    byte = (uint8_t)((byte & ~(3u << shift)) | (code << shift));
}

void GpuMarkerBuilder::endColumn()
{
    if (!m_marker)
        return;
    m_ended[m_snp] = 1;
    static_cast<GpuMarker *>(m_marker.get())->valid = true;
}

std::unique_ptr<Marker> GpuMarkerBuilder::build()
{
    if (!m_marker) {
        std::cerr << "Not building Marker, was MarkerBuilder::initialise called?" << std::endl;
        return nullptr;
    }
    if (!m_marker->isValid()) {
        std::cerr << "Marker is not valid!" << std::endl;
        return nullptr;
    }
    return std::move(m_marker);
}

int GpuMarkerBuilder::pack(brr_ctx *ctx) const
{
    for (unsigned j = 0; j < m_snps; ++j)
        if (!m_ended[j]) {
            std::cerr << "GpuMarkerBuilder: column " << j << " was never ended" << std::endl;
            return BRR_ERR_ARG;
        }
    const int rc = brr_pack_bed(ctx, m_bed.data(), (int64_t)m_bed.size());
    if (rc != BRR_OK)
        std::cerr << "GpuMarkerBuilder: packing failed: " << brr_last_error() << std::endl;
    return rc;
}

// ---------------------------------------------------------------------------
// GpuSweepGraph

GpuSweepGraph::GpuSweepGraph(brr_ctx *ctx) : AnalysisGraph(1), m_ctx(ctx) {}

int GpuSweepGraph::fail(int rc, const char *what)
{
    m_status = rc;
    m_error = std::string(what) + ": " + brr_last_error();
    std::cerr << "GpuSweepGraph: " << m_error << std::endl;
    return rc;
}

int GpuSweepGraph::setPhenotype(const float *y)
{
    const int rc = brr_set_phenotype(m_ctx, y);
    return rc ? fail(rc, "brr_set_phenotype") : BRR_OK;
}

int GpuSweepGraph::setGroups(const int32_t *group)
{
    const int rc = brr_set_groups(m_ctx, group);
    return rc ? fail(rc, "brr_set_groups") : BRR_OK;
}

void GpuSweepGraph::exec(Analysis *analysis, unsigned int numInds, unsigned int numSnps,
                         const std::vector<unsigned int> &markerIndices)
{
    m_status = BRR_OK;
    m_error.clear();
    auto *st = dynamic_cast<BayesRSweepAccess *>(analysis);
    if (!st) {
        m_status = BRR_ERR_ARG;
        m_error = "the analysis does not implement BayesRSweepAccess";
        std::cerr << "GpuSweepGraph: " << m_error << std::endl;
        return;
    }
    m_analysis = analysis;
    const auto &draws = st->markerDraws();
    if (markerIndices.size() != numSnps || draws.size() != numSnps) {
        m_status = BRR_ERR_ARG;
        m_error = "one marker index and one (p, randomNorm) pair per marker are required";
        std::cerr << "GpuSweepGraph: " << m_error << std::endl;
        return;
    }
    // the analysis's state onto the device (updateMu, the scalar draws and
    // any fixed effects changed it on the host since the last sweep)
    m_comp.resize(numSnps);
    const double *cd = st->components();
    for (unsigned j = 0; j < numSnps; ++j)
        m_comp[j] = (int32_t)cd[j];
    brr_state s{};
    s.beta = st->beta();
    s.comp = m_comp.data();
    s.acum = st->acum();
    s.eps = st->epsilon();
    s.mu = st->mu();
    s.sigmaE = st->sigmaE();
    s.epsSum = st->epsilonSum();
    for (int g = 0; g < BRR_MAX_GROUPS; ++g) {
        const int K = st->mixtureSize(g);
        if (K <= 0)
            break;
        s.sigmaG[g] = st->sigmaG(g);
        for (int k = 0; k < K && k < BRR_MAX_K; ++k)
            s.pi[g * BRR_MAX_K + k] = st->pi(g, k);
    }
    int rc = brr_set_state(m_ctx, &s);
    if (rc) {
        fail(rc, "brr_set_state");
        return;
    }
    m_u.resize(numSnps);
    m_z.resize(numSnps);
    for (unsigned j = 0; j < numSnps; ++j) {
        m_u[j] = draws[j][0];
        m_z[j] = draws[j][1];
    }
    brr_sweep_out out{};
    rc = brr_sweep(m_ctx, markerIndices.data(), m_u.data(), m_z.data(), &out);
    if (rc) {
        fail(rc, "brr_sweep");
        return;
    }
    // results back where runGibbs reads them: the sample row (beta,
    // components, acum, residual), the residual's norm (sigmaE draw) and
    // the component counts and squared effects per group (sigmaG, pi draws)
    rc = brr_get_state(m_ctx, &s);
    if (rc) {
        fail(rc, "brr_get_state");
        return;
    }
    double *comp = st->components();
    for (unsigned j = 0; j < numSnps; ++j)
        comp[j] = (double)m_comp[j];
    st->epsilonSum() = s.epsSum;
    for (int g = 0; g < BRR_MAX_GROUPS; ++g) {
        const int K = st->mixtureSize(g);
        if (K <= 0)
            break;
        for (int k = 0; k < K; ++k)
            st->setComponentCount(g, k, out.v[g * BRR_MAX_K + k]);
        st->setBetaSquaredNorm(g, out.betasqnG[g]);
    }
    double ms = 0.0, total = 0.0;
    int64_t rounds = 0;
    if (brr_get_timing(m_ctx, &ms, &total, &rounds) == BRR_OK)
        m_sweepMs = ms;
    (void)numInds;
}
