// `brr`: command-line entry of the GB300 BayesR path (the reference's
// src/main.cpp:8-48 + AnalysisRunner::run, src/analysisrunner.cpp:278-306,
// restricted to --preprocess and --analysis-type ppbayes over PLINK BED).
// Compute runs in libbrr_gpu.so through the C ABI of include/brr_gpu.h.
#include <charconv>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <deque>
#include <future>
#include <mutex>
#include <thread>
#include <cstdio>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <sstream>
#include <vector>

#include "../../include/brr_gpu.h"
#include "data.h"
#include "options.h"

using namespace brr;

namespace {

void check(int rc, const char *what)
{
    if (rc != BRR_OK)
        throw std::string("Error: ") + what + " failed (" + std::to_string(rc) + "): " + brr_last_error();
}

// src/analysisrunner.cpp:20-45
void readMetaData(Data &data, const Options &opt)
{
    if (opt.inputType != InputType::BED)
        throw std::string("Error: the GB300 path reads PLINK BED input (--bfile PREFIX or --data-file X.bed)");
    data.readFamFile(fileWithSuffix(opt.dataFile, ".fam"));
    data.readBimFile(fileWithSuffix(opt.dataFile, ".bim"));
    if (!opt.phenotypeFile.empty())
        data.readPhenotypeFile(opt.phenotypeFile);
    if (!opt.groupFile.empty()) {
        data.readGroupFile(opt.groupFile);
        if (opt.S.size() != data.numGroups)
            std::cerr << "Number of groups " << data.numGroups << " does not match the number of variance sets: "
                      << opt.S.size() << std::endl;
    }
}

brr_config makeConfig(const Options &opt, const Data &data)
{
    brr_config c{};
    c.N = data.numInds();
    c.M = data.numSnps();
    c.kind = opt.preprocessDataType == PreprocessDataType::SparseRagged  ? BRR_KIND_RAGGED
             : opt.preprocessDataType == PreprocessDataType::SparseEigen ? BRR_KIND_EIGEN
                                                                          : BRR_KIND_DENSE;
    c.form = opt.form == "fp32c" ? BRR_FORM_FP32C : BRR_FORM_FP64;
    c.n_groups = (int)opt.S.size();
    if (c.n_groups < 1 || c.n_groups > BRR_MAX_GROUPS)
        throw std::string("Error: the variance components could not be parsed (--S)");
    for (int g = 0; g < c.n_groups; ++g) {
        c.K[g] = (int)opt.S[g].size() + 1;
        for (std::size_t k = 0; k < opt.S[g].size() && k < BRR_MAX_K - 1; ++k)
            c.S[g * (BRR_MAX_K - 1) + k] = opt.S[g][k];
    }
    c.seed = opt.seed;
    c.chain = 0;
    c.v0E = opt.v0E;
    c.s02E = opt.s02E;
    c.v0G = opt.v0G;
    c.s02G = opt.s02G;
    c.refresh_every = opt.refreshEvery;
    c.spec_width = opt.specWidth;
    c.device = opt.device;
    if (opt.analysisType == AnalysisType::AsyncPpBayes) {
        // the reference's ParallelGraph with --analysis-tokens markers in flight
        // (src/analysisrunner.cpp:259-268, src/parallelgraph.cpp:51-150)
        if (opt.analysisTokens < 1 || opt.analysisTokens > 64)
            throw std::string("Error: --analysis-tokens must be in 1..64 for the GPU asyncppbayes sweep");
        if (c.form != BRR_FORM_FP64)
            throw std::string("Error: asyncppbayes runs the FP64 form (--form fp64)");
        c.async_batch = opt.analysisTokens;
    }
    return c;
}

struct Ctx {
    brr_ctx *h = nullptr;
    ~Ctx() { brr_ctx_destroy(h); }
};

// Genotype codes of the analysis: the reference's ppbayes maps the file its
// --preprocess wrote (src/analysisrunner.cpp:186-196); when that file and its
// index exist they are read back into 2-bit codes, otherwise the BED is read.
std::vector<uint8_t> readPreprocessedAsBed(const Options &opt, int64_t N, int64_t M)
{
    const std::string pp = ppFileForType(opt.preprocessDataType, opt.dataFile);
    const std::string ix = ppIndexFileForType(opt.preprocessDataType, opt.dataFile);
    switch (opt.preprocessDataType) {
    case PreprocessDataType::Dense: return readDensePreprocessedAsBed(pp, ix, N, M, opt.compress);
    case PreprocessDataType::SparseEigen: return readEigenPreprocessedAsBed(pp, ix, N, M, opt.compress);
    case PreprocessDataType::SparseRagged: return readRaggedPreprocessedAsBed(pp, ix, N, M, opt.compress);
    default: throw std::string("Error: unsupported --sparse-data type (dense, eigen or ragged)");
    }
}

std::vector<uint8_t> readGenotypes(const Options &opt, int64_t N, int64_t M, bool preprocessed)
{
    const std::string pp = ppFileForType(opt.preprocessDataType, opt.dataFile);
    const std::string ix = ppIndexFileForType(opt.preprocessDataType, opt.dataFile);
    if (preprocessed && std::ifstream(pp).good() && std::ifstream(ix).good()) {
        std::cout << "Start reading preprocessed bed file: " << pp << std::endl;
        return readPreprocessedAsBed(opt, N, M);
    }
    return readBedPayload(opt.dataFile, N, M);
}

void packFromBed(Ctx &ctx, const Options &opt, const Data &data, const brr_config &cfg, std::vector<uint8_t> &bed,
                 bool preprocessed = false)
{
    check(brr_ctx_create(&cfg, &ctx.h), "brr_ctx_create");
    bed = readGenotypes(opt, cfg.N, cfg.M, preprocessed);
    check(brr_pack_bed(ctx.h, bed.data(), (int64_t)bed.size()), "brr_pack_bed");
}

// src/analysisrunner.cpp:47-78 + src/preprocessgraph.cpp:152-244
bool preprocess(const Options &opt)
{
    if (opt.preprocessDataType == PreprocessDataType::None)
        throw std::string("Error: unsupported --sparse-data type (dense, eigen or ragged)");
    if (opt.compress && !canReadCompressed())
        throw std::string("Error: --compress needs zlib, which this build of brr does not have");
    const auto t0 = std::chrono::steady_clock::now();
    Data data;
    readMetaData(data, opt);
    const brr_config cfg = makeConfig(opt, data);
    Ctx ctx;
    std::vector<uint8_t> bed;
    packFromBed(ctx, opt, data, cfg, bed);
    const int64_t M = cfg.M;
    std::vector<double> table((size_t)M * 4);
    std::vector<int64_t> counts((size_t)M * 4);
    check(brr_get_marker_table(ctx.h, table.data(), counts.data()), "brr_get_marker_table");
    const std::string pp = ppFileForType(opt.preprocessDataType, opt.dataFile);
    const std::string ix = ppIndexFileForType(opt.preprocessDataType, opt.dataFile);
    if (cfg.kind == BRR_KIND_DENSE) {
        writeDensePreprocessed(pp, ix, cfg.N, M, table.data(), bed.data());
    } else {
        int64_t tot[3] = {0, 0, 0};
        for (int64_t j = 0; j < M; ++j) {
            tot[0] += counts[4 * j + 1];
            tot[1] += counts[4 * j + 2];
            tot[2] += counts[4 * j + 3];
        }
        std::vector<int64_t> off[3];
        std::vector<int32_t> idx[3];
        for (int k = 0; k < 3; ++k) {
            off[k].resize(M + 1);
            idx[k].resize(tot[k] + 1);
        }
        check(brr_get_ragged_lists(ctx.h, off[0].data(), idx[0].data(), off[1].data(), idx[1].data(), off[2].data(),
                                   idx[2].data()),
              "brr_get_ragged_lists");
        const int64_t *offs[3] = {off[0].data(), off[1].data(), off[2].data()};
        const int32_t *idxs[3] = {idx[0].data(), idx[1].data(), idx[2].data()};
        if (cfg.kind == BRR_KIND_EIGEN)
            writeEigenPreprocessed(pp, ix, M, table.data(), offs, idxs);
        else
            writeRaggedPreprocessed(pp, ix, M, table.data(), offs, idxs);
    }
    // --compress: every record deflated, as the reference's PreprocessGraph
    // writes them (src/preprocessgraph.cpp:63-67, :110-122)
    if (opt.compress)
        compressPreprocessed(pp, ix, M);
    const double s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    std::printf("Finished preprocessing the bed file in %.3f sec.\n\n", s);
    return true;
}

// Sample file of SampleWriter::openGroups / Writer::write
// (src/samplewriter.cpp:82-118, src/writer.cpp:9-22): header with ',' and rows
// with ", " in the stream's default precision.
// Rows are formatted and written by a background thread, so that a saved
// iteration costs the chain only the copy of its state (the reference writes
// synchronously, which at N = M = 100k is several times a sweep's time); the
// writer formats each row in eight slices on eight threads.  Up to two rows
// wait; a third waits for the writer.  Numbers are printed as the default
// ostream does (6 significant digits, %g style).
class SampleWriter {
public:
    void open(const std::string &file, int64_t M, int64_t N, int G)
    {
        std::cout << "Opening results file " << file << std::endl;
        out_.open(file);
        if (!out_)
            throw("Error: can not open the sample file [" + file + "] for writing.");
        M_ = M;
        N_ = N;
        G_ = G;
        out_ << "iteration," << "mu,";
        for (int64_t i = 0; i < M; ++i)
            out_ << "beta[" << (i + 1) << "],";
        out_ << "sigmaE,";
        for (int g = 0; g < G; ++g)
            out_ << "sigmaG[" << (g + 1) << "],";
        for (int64_t i = 0; i < M; ++i)
            out_ << "comp[" << (i + 1) << "],";
        for (int64_t i = 0; i < M; ++i)
            out_ << "acum[" << (i + 1) << "],";
        int64_t i;
        for (i = 0; i < N - 1; ++i)
            out_ << "epsilon[" << (i + 1) << "],";
        out_ << "epsilon[" << (i + 1) << "]" << std::endl;
        thread_ = std::thread([this] { run(); });
    }
    // Copies the state; returns as soon as a buffer is free.
    void write(unsigned iteration, const brr_state &st)
    {
        std::unique_lock<std::mutex> lk(mu_);
        cv_.wait(lk, [this] { return queue_.size() < 2 || failed_; });
        if (failed_)
            throw std::string("Error: writing the sample file failed");
        Row r;
        if (!free_.empty()) {
            r = std::move(free_.back());
            free_.pop_back();
        }
        lk.unlock();
        r.iteration = iteration;
        r.mu = st.mu;
        r.sigmaE = st.sigmaE;
        r.sigmaG.assign(st.sigmaG, st.sigmaG + G_);
        r.beta.assign(st.beta, st.beta + M_);
        r.comp.assign(st.comp, st.comp + M_);
        r.acum.assign(st.acum, st.acum + M_);
        r.eps.assign(st.eps, st.eps + N_);
        lk.lock();
        queue_.push_back(std::move(r));
        cv_.notify_all();
    }
    // Waits for the queued rows and closes the file.
    void close()
    {
        if (!thread_.joinable())
            return;
        {
            std::lock_guard<std::mutex> lk(mu_);
            done_ = true;
        }
        cv_.notify_all();
        thread_.join();
        out_.close();
        if (failed_)
            throw std::string("Error: writing the sample file failed");
    }
    ~SampleWriter()
    {
        try {
            close();
        } catch (...) {
        }
    }

private:
    struct Row {
        unsigned iteration = 0;
        double mu = 0, sigmaE = 0;
        std::vector<double> sigmaG, beta, acum, eps;
        std::vector<int32_t> comp;
    };
    static void put(std::string &s, double v)
    {
        char buf[64];
        const auto r = std::to_chars(buf, buf + sizeof buf, v, std::chars_format::general, 6);
        s.append(buf, r.ptr);
    }
    // Value k of the row in file order: iteration, mu, beta[M], sigmaE,
    // sigmaG[G], comp[M], acum[M], epsilon[N].
    double value(const Row &r, int64_t k) const
    {
        if (k == 0)
            return (double)r.iteration;
        if (k == 1)
            return r.mu;
        k -= 2;
        if (k < M_)
            return r.beta[(size_t)k];
        k -= M_;
        if (k == 0)
            return r.sigmaE;
        k -= 1;
        if (k < G_)
            return r.sigmaG[(size_t)k];
        k -= G_;
        if (k < M_)
            return (double)r.comp[(size_t)k];
        k -= M_;
        if (k < M_)
            return r.acum[(size_t)k];
        return r.eps[(size_t)(k - M_)];
    }
    // Values [lo, hi) of the row, each followed by ", " except the row's last.
    void format_range(const Row &r, int64_t lo, int64_t hi, std::string &s) const
    {
        s.clear();
        const int64_t last = 3 + G_ + 3 * M_ + N_ - 1;
        for (int64_t k = lo; k < hi; ++k) {
            put(s, value(r, k));
            if (k != last)
                s += ", ";
        }
        if (hi == last + 1)
            s += '\n';
    }
    // Formats each row in kParts slices on as many threads (a row at
    // N = M = 100,000 holds 400,000 numbers) and writes the slices in order.
    void run()
    {
        const int64_t total = 3 + G_ + 3 * M_ + N_;
        const int parts = total < 65536 ? 1 : kParts;
        std::vector<std::string> slice((size_t)parts);
        for (;;) {
            Row r;
            {
                std::unique_lock<std::mutex> lk(mu_);
                cv_.wait(lk, [this] { return !queue_.empty() || done_; });
                if (queue_.empty())
                    break;
                r = std::move(queue_.front());
                queue_.pop_front();
            }
            std::vector<std::future<void>> work;
            for (int t = 1; t < parts; ++t)
                work.push_back(std::async(std::launch::async, [&, t] {
                    format_range(r, total * t / parts, total * (t + 1) / parts, slice[(size_t)t]);
                }));
            format_range(r, 0, total / parts, slice[0]);
            for (auto &w : work)
                w.get();
            for (const std::string &sl : slice)
                out_.write(sl.data(), (std::streamsize)sl.size());
            std::lock_guard<std::mutex> lk(mu_);
            if (!out_)
                failed_ = true;
            free_.push_back(std::move(r));
            cv_.notify_all();
        }
        out_.flush();
    }

    static constexpr int kParts = 8;
    std::ofstream out_;
    int64_t M_ = 0, N_ = 0;
    int G_ = 0;
    std::thread thread_;
    std::mutex mu_;
    std::condition_variable cv_;
    std::deque<Row> queue_;
    std::vector<Row> free_;
    bool done_ = false, failed_ = false;
};

// runBayesRAnalysis + BayesRBase::runGibbs (src/analysisrunner.cpp:123-152,
// src/BayesRBase.cpp:130-285)
bool ppbayes(const Options &opt)
{
    if (opt.fixedEffectNumber != 0)
        throw std::string("Error: --fixedEffectNumber " + std::to_string(opt.fixedEffectNumber) +
                          ": fixed effects are not supported by the GPU sampler");
    Data data;
    readMetaData(data, opt);
    if (opt.S.empty())
        throw std::string("Error: variance components must be given for ppbayes (--S)");
    if ((int64_t)data.y.size() != data.numInds())
        throw std::string("Error: " + std::to_string(data.y.size()) + " phenotype values for " +
                          std::to_string(data.numInds()) + " individuals (missing phenotypes must be removed)");
    if ((int64_t)data.G.size() != data.numSnps())
        throw std::string("Error: the group file lists " + std::to_string(data.G.size()) + " SNPs, the BIM " +
                          std::to_string(data.numSnps()));
    const brr_config cfg = makeConfig(opt, data);
    Ctx ctx;
    std::vector<uint8_t> bed;
    packFromBed(ctx, opt, data, cfg, bed, true);
    check(brr_set_groups(ctx.h, data.G.data()), "brr_set_groups");
    check(brr_set_phenotype(ctx.h, data.y.data()), "brr_set_phenotype");
    check(brr_init_chain(ctx.h), "brr_init_chain");

    const int64_t M = cfg.M, N = cfg.N;
    const int G = cfg.n_groups;
    SampleWriter writer;
    writer.open(opt.mcmcSampleFile, M, N, G);
    std::ofstream iterLog;
    if (opt.iterLog)
        iterLog.open(opt.iterLogFile);
    // The reference's column log holds per-marker microseconds of num, beta and
    // the epsilon update (src/BayesRBase.cpp:381-389).  On the GPU markers are
    // swept in blocks by many warps at once, so its counterpart is the sweep's
    // phase counters: the counting kernel variant (the same chain bit for bit)
    // and one row per iteration of the 16 counters of brr_get_phase_cycles.
    std::ofstream colLog;
    if (opt.colLog) {
        colLog.open(opt.colLogFile);
        if (!colLog)
            throw std::string("Error: cannot open the column log " + opt.colLogFile);
        check(brr_set_profiling(ctx.h, 1), "brr_set_profiling");
        colLog << "iter";
        for (int k = 0; k < 16; ++k)
            colLog << ",phase" << k;
        colLog << std::endl;
    }
    std::vector<double> beta(M), acum(M), eps(N);
    std::vector<int32_t> comp(M);
    brr_state st{};
    st.beta = beta.data();
    st.comp = comp.data();
    st.acum = acum.data();
    st.eps = eps.data();
    std::cout << "Number of groups: " << G << std::endl << "Running Gibbs sampling" << std::endl;
    double meanIter = 0.0, meanSweep = 0.0;
    const auto t1 = std::chrono::steady_clock::now();
    for (unsigned it = 0; it < opt.chainLength; ++it) {
        const auto s0 = std::chrono::steady_clock::now();
        std::cout << "iteration " << it << ": ";
        check(brr_iterate(ctx.h, 1), "brr_iterate");
        double sweep_ms = 0, total_ms = 0;
        int64_t rounds = 0;
        brr_get_timing(ctx.h, &sweep_ms, &total_ms, &rounds);
        if (it >= opt.burnin && it % opt.thin == 0) {
            check(brr_get_state(ctx.h, &st), "brr_get_state");
            writer.write(it, st);
        }
        const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - s0).count();
        std::cout << secs << "s (" << sweep_ms / 1000.0 << "s)" << std::endl;
        meanIter += secs;
        meanSweep += sweep_ms / 1000.0;
        if (opt.colLog) {
            int64_t cyc[16] = {0};
            check(brr_get_phase_cycles(ctx.h, cyc), "brr_get_phase_cycles");
            colLog << it;
            for (int k = 0; k < 16; ++k)
                colLog << "," << cyc[k];
            colLog << std::endl;
        }
        if (opt.iterLog) {
            brr_state sc{};
            check(brr_get_state(ctx.h, &sc), "brr_get_state");
            iterLog << it << ", " << sc.mu << ", " << sc.sigmaE;
            for (int g = 0; g < G; ++g)
                iterLog << ", " << sc.sigmaG[g];
            iterLog << ", " << sweep_ms << ", " << total_ms << ", " << rounds << std::endl;
        }
    }
    writer.close();
    const double dur = std::chrono::duration<double>(std::chrono::steady_clock::now() - t1).count();
    std::cout << "duration: " << (long)dur << "s" << std::endl;
    const double n = opt.chainLength ? (double)opt.chainLength : 1.0;
    std::cout << "mean iteration duration: " << meanIter / n << "s" << std::endl
              << "mean flowgraph duration: " << meanSweep / n << "s" << std::endl;
    return true;
}

void printOptions(const Options &o)
{
    std::cout << "{\"analysis\": " << (int)o.analysisType << ", \"input\": " << (int)o.inputType
              << ", \"data\": \"" << o.dataFile << "\", \"pheno\": \"" << o.phenotypeFile << "\", \"chain\": "
              << o.chainLength << ", \"burnin\": " << o.burnin << ", \"thin\": " << o.thin << ", \"seed\": " << o.seed
              << ", \"samples\": \"" << o.mcmcSampleFile << "\", \"sparse\": " << (int)o.preprocessDataType
              << ", \"form\": \"" << o.form << "\", \"colLog\": \"" << (o.colLog ? o.colLogFile : "")
              << "\", \"tokens\": " << o.analysisTokens << ", \"fixed\": " << o.fixedEffectNumber << ", \"failure\": \"" << o.failureFile
              << "\", \"compress\": " << (o.compress ? "true" : "false")
              << ", \"zlib\": " << (canReadCompressed() ? "true" : "false") << ", \"S\": [";
    for (std::size_t g = 0; g < o.S.size(); ++g) {
        std::cout << (g ? ", " : "") << "[";
        for (std::size_t k = 0; k < o.S[g].size(); ++k)
            std::cout << (k ? ", " : "") << std::setprecision(17) << o.S[g][k];
        std::cout << "]";
    }
    std::cout << "]}" << std::endl;
}

}  // namespace

int main(int argc, const char *argv[])
{
    std::cout << "***********************************************\n"
              << "* brr (GB300 sm_103a BayesR Gibbs sampler)    *\n"
              << "***********************************************" << std::endl;
    try {
        Options opt;
        opt.inputOptions(argc, argv);
        if (opt.printOptions) {
            printOptions(opt);
            return 0;
        }
        if (!opt.exportBedFile.empty()) {
            // preprocessed input (per --sparse-data) back to a PLINK BED: no GPU needed
            Data data;
            data.readFamFile(fileWithSuffix(opt.dataFile, ".fam"));
            data.readBimFile(fileWithSuffix(opt.dataFile, ".bim"));
            writeBedFile(opt.exportBedFile, readPreprocessedAsBed(opt, data.numInds(), data.numSnps()));
            std::cout << "Wrote " << opt.exportBedFile << std::endl;
            return 0;
        }
        switch (opt.analysisType) {
        case AnalysisType::Preprocess:
            return preprocess(opt) ? 0 : 1;
        case AnalysisType::PpBayes:
            if (opt.S.empty()) {
                std::cerr << "Variance components `--S` are missing or could not be parsed!" << std::endl;
                return 1;
            }
            return ppbayes(opt) ? 0 : 1;
        case AnalysisType::AsyncPpBayes:
            if (opt.S.empty()) {
                std::cerr << "Variance components `--S` are missing or could not be parsed!" << std::endl;
                return 1;
            }
            return ppbayes(opt) ? 0 : 1;
        case AnalysisType::Gauss:
        case AnalysisType::AsyncGauss:
            // the BayesW (Gauss) analyses of the reference
            // (src/analysisrunner.cpp:219-268) are not on this path
            std::cerr << "Error: this GPU sampler runs --analysis-type ppbayes and asyncppbayes (and preprocess); "
                         "gauss and asyncgauss are not supported" << std::endl;
            return 1;
        default:
            std::cerr << "unknown analysis type" << std::endl;
            return 1;
        }
    } catch (const std::string &err) {
        std::cerr << err << std::endl;
    } catch (const char *err) {
        std::cerr << err << std::endl;
    }
    return 1;
}
