// Command-line options of `brr`, mirroring the reference Options class
// (src/options.hpp:21-105, parser src/options.cpp:95-332) for the BayesR path.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace brr {

enum class AnalysisType { Unknown = 0, Preprocess, PpBayes, AsyncPpBayes, Gauss, AsyncGauss };   // src/common.h:8-15
enum class InputType { Unknown = 0, BED, CSV };                  // src/common.h:19-23
enum class PreprocessDataType { None = 0, Dense, SparseEigen, SparseRagged };  // src/common.h:27-32

// Variance components: one row per group; rows may differ in length (the
// reference requires equal lengths, src/options.cpp:46-55; a group with its
// own mixture size is the generalisation the two-group configurations need).
using VarianceComponents = std::vector<std::vector<double>>;

// src/options.cpp:23-73: groups separated by ';', components by ','.  Returns
// an empty matrix on any parse error, as the reference does.
VarianceComponents parseVarianceComponentsFromString(const std::string &s, bool require_equal_rows = false);
// src/options.cpp:86-93: a path to an existing regular file is read, else the
// argument itself is parsed.
VarianceComponents parseVarianceComponents(const std::string &arg);

struct Options {
    unsigned chainLength = 10000;          // src/options.hpp:67-77 defaults
    unsigned burnin = 5000;
    unsigned seed = 0;
    unsigned thin = 5;
    VarianceComponents S = {{0.01, 0.001, 0.0001}};
    std::string groupFile;
    std::string title = "brr";
    AnalysisType analysisType = AnalysisType::Unknown;
    std::string phenotypeFile;
    std::string dataFile;
    InputType inputType = InputType::Unknown;
    std::string mcmcSampleFile = "bayesOutput.csv";
    std::string optionFile;
    bool compress = false;
    PreprocessDataType preprocessDataType = PreprocessDataType::Dense;
    std::string iterLogFile;
    bool iterLog = false;
    std::string colLogFile;                // src/options.hpp:57-58
    bool colLog = false;
    unsigned fixedEffectNumber = 0;        // src/options.hpp:44: fixed effects are not on this path
    std::string failureFile;               // src/options.hpp:40: BayesW only
    bool useMarkerCache = false;
    unsigned numThread = 0;
    double v0E = 0.0001, s02E = 0.0001, v0G = 0.0001, s02G = 0.0001;
    // GB300 additions
    std::string form = "fp64";             // fp64 (drop-in) | fp32c
    int refreshEvery = 50;
    int analysisTokens = 20;    // asyncppbayes: markers in flight (src/options.hpp:33)
    int specWidth = 0;
    int device = 0;
    bool printOptions = false;
    std::string exportBedFile;             // --export-bed: preprocessed input back to PLINK BED, then exit

    Options();
    // Throws std::string on an invalid option, like the reference.
    void inputOptions(int argc, const char *argv[]);
    void readFile(const std::string &file);
};

InputType getInputType(const std::string &dataFile);                      // src/common.cpp:118-134
std::string fileWithSuffix(const std::string &dataFile, const std::string &suffix);  // src/common.cpp:67-70
std::string ppFileForType(PreprocessDataType type, const std::string &dataFile);     // src/common.cpp:72-93
std::string ppIndexFileForType(PreprocessDataType type, const std::string &dataFile);

}  // namespace brr
