// GPU implementations of the reference's sweep-path interfaces, over the C ABI
// of libbrr_gpu.so:
//
//   GpuMarkerBuilder : MarkerBuilder   collects the 2-bit genotype codes that
//       the preprocess graph feeds through processAllele (src/preprocessgraph.cpp:24-70)
//       column by column, and packs all columns on the device in one
//       brr_pack_bed call (decode, counts, standardisation or index lists);
//   GpuSweepGraph : AnalysisGraph      runs the whole sweep of
//       AnalysisGraph::exec (src/analysisgraph.hpp:18-21; the reference's
//       Sequential graph calls processColumn per marker, src/sequential.cpp:10-27)
//       as one brr_sweep, then writes the sweep's results back into the
//       analysis, where runGibbs reads them (src/BayesRBase.cpp:237-253).
//
// The reference's BayesRBase keeps the chain state in protected members
// (src/BayesRBase.hpp:63-96) and has no accessors for them.  To plug in a
// GPU graph it implements BayesRSweepAccess below: every accessor returns or
// sets an existing member, nothing else changes in runGibbs.
#pragma once

#include <array>
#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include "../../include/brr_gpu.h"
#include "reference_iface.h"

// What BayesRBase would add (each a one-line accessor of an existing member).
class BayesRSweepAccess
{
public:
    virtual ~BayesRSweepAccess() = default;

    // m_randomNumbers[j] = {p, randomNorm}, indexed by marker id, drawn by
    // prepareForAnylsis before the sweep (src/BayesRBase.cpp:101-110)
    virtual const std::vector<std::array<double, 2>> &markerDraws() const = 0;
    virtual double mu() const = 0;                       // m_mu
    virtual double sigmaE() const = 0;                   // m_sigmaE
    virtual double sigmaG(int group) const = 0;          // m_sigmaG[group]
    virtual double pi(int group, int k) const = 0;       // m_pi(group, k)
    virtual int mixtureSize(int group) const = 0;        // K of the group (m_pi.cols() for one K)
    virtual double *beta() = 0;                          // m_beta.data(), M values
    virtual double *components() = 0;                    // m_components.data(), M values (component as double)
    virtual double *acum() = 0;                          // m_acum.data(), M values
    virtual double *epsilon() = 0;                       // m_epsilon.data(), N values
    virtual double &epsilonSum() = 0;                    // m_epsilonSum (running sum of the sparse kinds)
    // after the sweep: m_v(group, k) and m_betasqnG[group] as processColumn
    // accumulates them (src/BayesRBase.cpp:353-355)
    virtual void setComponentCount(int group, int k, double count) = 0;
    virtual void setBetaSquaredNorm(int group, double value) = 0;
};

// Marker handed back by GpuMarkerBuilder::build: the values stay on the
// device once packed; the object carries the marker's index and size, and is
// valid once its column was ended (a column that does not vary is refused
// when the batch is packed, with BRR_ERR_MARKER).
struct GpuMarker : public Marker
{
    bool valid = false;

    std::streamsize size() const override { return 0; }
    void read(std::istream *) override {}
    void write(std::ostream *) const override {}
    bool isValid() const override { return valid; }
};

class GpuMarkerBuilder : public MarkerBuilder
{
public:
    // numSnps columns of numInds individuals each
    GpuMarkerBuilder(unsigned int numInds, unsigned int numSnps);

    void initialise(const unsigned int snp, const unsigned int numInds) override;
    // allele1 = !bit(2i), allele2 = !bit(2i+1) of the BED code
    // (src/preprocessgraph.cpp:43-56); (0, 1) is missing
    void processAllele(unsigned int individual, unsigned int allele1, unsigned int allele2) override;
    void endColumn() override;
    std::unique_ptr<Marker> build() override;

    // Uploads every column to the context and packs it on the device (one
    // brr_pack_bed call); BRR_ERR_ARG if a column was never ended.
    int pack(brr_ctx *ctx) const;
    const std::vector<uint8_t> &payload() const { return m_bed; }

private:
    unsigned int m_inds, m_snps;
    size_t m_colBytes;
    std::vector<uint8_t> m_bed;       // SNP-major BED payload, no header
    std::vector<uint8_t> m_ended;     // per column: endColumn seen
};

class GpuSweepGraph : public AnalysisGraph
{
public:
    // ctx: markers packed (GpuMarkerBuilder::pack or brr_pack_bed); the
    // graph does not own it
    explicit GpuSweepGraph(brr_ctx *ctx);

    // The phenotype as read (float, NA rows removed) and the marker groups:
    // the device needs them for the FP64 residual refresh and the per-group
    // mixtures.  Call once before the first exec.
    int setPhenotype(const float *y);
    int setGroups(const int32_t *group);

    bool isAsynchronous() const override { return false; }

    // One sweep over markerIndices in order with the analysis's current
    // state and draws; the updated beta, components, acum, residual, running
    // residual sum and the sweep statistics are written back into the
    // analysis.  Errors are reported on std::cerr as the reference's graphs
    // do, and by status().
    void exec(Analysis *analysis, unsigned int numInds, unsigned int numSnps,
              const std::vector<unsigned int> &markerIndices) override;

    int status() const { return m_status; }
    const std::string &error() const { return m_error; }
    double lastSweepMs() const { return m_sweepMs; }

private:
    brr_ctx *m_ctx;
    int m_status = BRR_OK;
    std::string m_error;
    double m_sweepMs = 0.0;
    std::vector<double> m_u, m_z;
    std::vector<int32_t> m_comp;

    int fail(int rc, const char *what);
};
