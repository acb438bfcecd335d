// Stand-in declarations of the reference's interfaces on the Gibbs-sweep
// path, with the same names, signatures and ownership, but no Eigen, TBB or
// Boost (which the reference's own headers pull in):
//   AnalysisGraph   src/analysisgraph.hpp:9-26
//   Marker          src/marker.h:19-35 (without compress/decompress)
//   MarkerBuilder   src/markerbuilder.h:11-42 (without read/decompress)
//   Kernel          src/kernel.h:8-14
//   Analysis        src/analysis.h:25-52 (the members a sweep graph uses)
// A maintainer compiles gpu_adapter.cpp against the reference's own headers
// instead; nothing in the adapter depends on what is left out here.
#pragma once

#include <cstddef>
#include <iosfwd>
#include <memory>
#include <vector>

class Analysis;

class AnalysisGraph
{
public:
    explicit AnalysisGraph(size_t maxParallel = 0) : m_maxParallel(maxParallel) {}
    virtual ~AnalysisGraph() = default;

    // true if the analysis calls BayesRBase::processColumnAsync
    virtual bool isAsynchronous() const = 0;

    virtual void exec(Analysis *analysis, unsigned int numInds, unsigned int numSnps,
                      const std::vector<unsigned int> &markerIndices) = 0;

protected:
    Analysis *m_analysis = nullptr;
    size_t m_maxParallel = 0;
};

struct Marker
{
    virtual ~Marker() = default;

    unsigned int i = 0;
    unsigned int numInds = 0;

    virtual std::streamsize size() const = 0;
    virtual void read(std::istream *inStream) = 0;
    virtual void write(std::ostream *outStream) const = 0;
    virtual bool isValid() const = 0;
};

using ConstMarkerPtr = std::shared_ptr<const Marker>;

class MarkerBuilder
{
public:
    virtual ~MarkerBuilder() = default;

    virtual void initialise(const unsigned int snp, const unsigned int numInds)
    {
        m_snp = snp;
        m_numInds = numInds;
    }
    virtual void processAllele(unsigned int individual, unsigned int allele1, unsigned int allele2) = 0;
    virtual void endColumn() = 0;
    // nullptr (with a message on std::cerr) when the column is not valid
    virtual std::unique_ptr<Marker> build() { return std::move(m_marker); }

protected:
    std::unique_ptr<Marker> m_marker = nullptr;
    unsigned int m_snp = 0;
    double m_numInds = 0;
};

struct Kernel
{
    explicit Kernel(const ConstMarkerPtr &m) : marker(m) {}
    virtual ~Kernel() = default;

    ConstMarkerPtr marker = nullptr;
};

using KernelPtr = std::shared_ptr<Kernel>;

class AnalysisGraph;

class Analysis
{
public:
    virtual ~Analysis() = default;

    virtual int runGibbs(AnalysisGraph *analysis) = 0;
    virtual void processColumn(const KernelPtr &kernel) = 0;
};
