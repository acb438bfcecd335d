#include "options.h"

#include <cstdlib>
#include <cstring>
#include <ctime>
#include <fstream>
#include <iostream>
#include <iterator>
#include <sstream>
#include <sys/stat.h>

namespace brr {

namespace {

std::vector<std::string> tokens(const std::string &s, const std::string &sep)
{
    std::vector<std::string> out;
    std::string::size_type b = s.find_first_not_of(sep);
    while (b != std::string::npos) {
        std::string::size_type e = s.find_first_of(sep, b);
        if (e == std::string::npos)
            e = s.size();
        out.push_back(s.substr(b, e - b));
        b = s.find_first_not_of(sep, e);
    }
    return out;
}

bool isRegularFile(const std::string &p)
{
    struct stat st;
    return ::stat(p.c_str(), &st) == 0 && S_ISREG(st.st_mode);
}

}  // namespace

VarianceComponents parseVarianceComponentsFromString(const std::string &s, bool require_equal_rows)
{
    std::vector<std::string> groups = tokens(s, ";");
    if (groups.empty())
        groups.push_back(s);
    VarianceComponents S;
    std::size_t expected = 0;
    for (std::size_t g = 0; g < groups.size(); ++g) {
        const std::vector<std::string> comps = tokens(groups[g], ",");
        if (comps.empty()) {
            std::cout << "Failed to parse variance components: " << s << std::endl;
            return {};
        }
        if (g == 0)
            expected = comps.size();
        else if (require_equal_rows && comps.size() != expected) {
            std::cout << "Incorrect number of variance components! Got: " << comps.size()
                      << ", expected: " << expected << std::endl;
            return {};
        }
        std::vector<double> row;
        for (const auto &c : comps) {
            try {
                std::size_t used = 0;
                const double v = std::stod(c, &used);
                row.push_back(v);
            } catch (const std::invalid_argument &) {
                std::cerr << "Could not parse variance component: " << c << std::endl;
                return {};
            } catch (const std::out_of_range &) {
                std::cerr << "Variance component is out of range: " << c << std::endl;
                return {};
            }
        }
        S.push_back(row);
    }
    return S;
}

VarianceComponents parseVarianceComponents(const std::string &arg)
{
    if (isRegularFile(arg)) {
        std::ifstream in(arg);
        if (!in.is_open()) {
            std::cout << "Error opening variance components file: " << arg << std::endl;
            return {};
        }
        return parseVarianceComponentsFromString({std::istreambuf_iterator<char>(in), std::istreambuf_iterator<char>()});
    }
    return parseVarianceComponentsFromString(arg);
}

static AnalysisType parseAnalysisType(const std::string &t)
{
    if (t == "preprocess")
        return AnalysisType::Preprocess;
    if (t == "ppbayes")
        return AnalysisType::PpBayes;
    if (t == "asyncppbayes")
        return AnalysisType::AsyncPpBayes;
    if (t == "gauss")
        return AnalysisType::Gauss;
    if (t == "asyncgauss")
        return AnalysisType::AsyncGauss;
    return AnalysisType::Unknown;
}

Options::Options() { seed = static_cast<unsigned>(std::time(nullptr)); }

InputType getInputType(const std::string &f)
{
    auto ends = [&](const std::string &e) { return f.size() >= e.size() && f.compare(f.size() - e.size(), e.size(), e) == 0; };
    if (ends(".bed"))
        return InputType::BED;
    if (ends(".csv"))
        return InputType::CSV;
    return InputType::Unknown;
}

std::string fileWithSuffix(const std::string &dataFile, const std::string &suffix)
{
    const auto pos = dataFile.find_last_of('.');
    return (pos == std::string::npos ? dataFile : dataFile.substr(0, pos)) + suffix;
}

std::string ppFileForType(PreprocessDataType type, const std::string &dataFile)
{
    switch (type) {
    case PreprocessDataType::Dense: return fileWithSuffix(dataFile, ".ppbed");
    case PreprocessDataType::SparseEigen: return fileWithSuffix(dataFile, ".eigen.sparsebed");
    case PreprocessDataType::SparseRagged: return fileWithSuffix(dataFile, ".ragged.sparsebed");
    default: return {};
    }
}

std::string ppIndexFileForType(PreprocessDataType type, const std::string &dataFile)
{
    switch (type) {
    case PreprocessDataType::Dense: return fileWithSuffix(dataFile, ".ppbedindex");
    case PreprocessDataType::SparseEigen: return fileWithSuffix(dataFile, ".eigen.sparsebedindex");
    case PreprocessDataType::SparseRagged: return fileWithSuffix(dataFile, ".ragged.sparsebedindex");
    default: return {};
    }
}

// src/options.cpp:95-278; unknown flags throw.  `--bfile PREFIX` selects
// PREFIX.bed/.bim/.fam (the reference README uses it, its parser lacks it).
void Options::inputOptions(int argc, const char *argv[])
{
    auto need = [&](int &i) -> const char * {
        if (i + 1 >= argc) {
            std::stringstream e;
            e << "\nError: option \"" << argv[i] << "\" needs a value.\n";
            throw e.str();
        }
        return argv[++i];
    };
    for (int i = 1; i < argc; ++i) {
        const char *a = argv[i];
        if (!std::strcmp(a, "--inp-file")) {
            optionFile = need(i);
            readFile(optionFile);
            return;
        } else if (!std::strcmp(a, "--analysis-type")) {
            analysisType = parseAnalysisType(need(i));
        } else if (!std::strcmp(a, "--preprocess")) {
            analysisType = AnalysisType::Preprocess;
        } else if (!std::strcmp(a, "--compress")) {
            compress = true;
        } else if (!std::strcmp(a, "--data-file")) {
            dataFile = need(i);
            inputType = getInputType(dataFile);
        } else if (!std::strcmp(a, "--bfile")) {
            dataFile = std::string(need(i)) + ".bed";
            inputType = InputType::BED;
        } else if (!std::strcmp(a, "--pheno")) {
            phenotypeFile = need(i);
        } else if (!std::strcmp(a, "--mcmc-samples")) {
            mcmcSampleFile = need(i);
        } else if (!std::strcmp(a, "--chain-length")) {
            chainLength = std::atoi(need(i));
        } else if (!std::strcmp(a, "--burn-in")) {
            burnin = std::atoi(need(i));
        } else if (!std::strcmp(a, "--seed")) {
            seed = std::atoi(need(i));
        } else if (!std::strcmp(a, "--out")) {
            title = need(i);
        } else if (!std::strcmp(a, "--thin")) {
            thin = std::atoi(need(i));
        } else if (!std::strcmp(a, "--S")) {
            S = parseVarianceComponents(need(i));
        } else if (!std::strcmp(a, "--group")) {
            groupFile = need(i);
        } else if (!std::strcmp(a, "--thread")) {
            numThread = std::atoi(need(i));
        } else if (!std::strcmp(a, "--sparse-data")) {
            const std::string t = need(i);
            if (t == "eigen")
                preprocessDataType = PreprocessDataType::SparseEigen;
            else if (t == "ragged")
                preprocessDataType = PreprocessDataType::SparseRagged;
            else
                preprocessDataType = PreprocessDataType::None;
        } else if (!std::strcmp(a, "--iterLog")) {
            iterLog = true;
            iterLogFile = need(i);
        } else if (!std::strcmp(a, "--colLog")) {
            colLog = true;
            colLogFile = need(i);
        } else if (!std::strcmp(a, "--fixedEffectNumber")) {
            fixedEffectNumber = (unsigned)std::atoi(need(i));
        } else if (!std::strcmp(a, "--failure")) {
            failureFile = need(i);
        } else if (!std::strcmp(a, "--marker-cache")) {
            useMarkerCache = true;
        } else if (!std::strcmp(a, "--v0E")) {
            v0E = std::atof(need(i));
        } else if (!std::strcmp(a, "--s02E")) {
            s02E = std::atof(need(i));
        } else if (!std::strcmp(a, "--v0G")) {
            v0G = std::atof(need(i));
        } else if (!std::strcmp(a, "--s02G")) {
            s02G = std::atof(need(i));
        } else if (!std::strcmp(a, "--analysis-tokens")) {
            // asyncppbayes: the markers the reference's ParallelGraph keeps in
            // flight (src/options.cpp:216-219), the GPU sweep's batch
            analysisTokens = std::atoi(need(i));
        } else if (!std::strcmp(a, "--thread-spawned") || !std::strcmp(a, "--decompression-concurrency") ||
                   !std::strcmp(a, "--decompression-tokens") || !std::strcmp(a, "--analysis-concurrency") ||
                   !std::strcmp(a, "--preprocess-chunks")) {
            need(i);   // host-thread tuning of the reference's TBB graphs: accepted, no effect on the GPU path
        } else if (!std::strcmp(a, "--form")) {
            form = need(i);
            if (form != "fp64" && form != "fp32c")
                throw std::string("\nError: --form must be fp64 or fp32c.\n");
        } else if (!std::strcmp(a, "--refresh")) {
            refreshEvery = std::atoi(need(i));
        } else if (!std::strcmp(a, "--spec-width")) {
            specWidth = std::atoi(need(i));
        } else if (!std::strcmp(a, "--device")) {
            device = std::atoi(need(i));
        } else if (!std::strcmp(a, "--print-options")) {
            printOptions = true;
        } else if (!std::strcmp(a, "--export-bed")) {
            exportBedFile = need(i);
        } else {
            std::stringstream e;
            e << "\nError: invalid option \"" << a << "\".\n";
            throw e.str();
        }
    }
}

// src/options.cpp:280-324: "key value" pairs; comments start with // or #.
void Options::readFile(const std::string &file)
{
    optionFile = file;
    const auto pos = file.rfind('.');
    title = pos == std::string::npos ? file : file.substr(0, pos);
    std::ifstream in(file.c_str());
    if (!in)
        throw("Error: can not open the file [" + file + "] to read.");
    std::string key, value;
    while (in >> key >> value) {
        if (key == "phenotypeFile")
            phenotypeFile = value;
        else if (key == "analysisType")
            analysisType = parseAnalysisType(value);
        else if (key == "mcmcSampleFile")
            mcmcSampleFile = value;
        else if (key == "chainLength")
            chainLength = std::stoi(value);
        else if (key == "burnin")
            burnin = std::stoi(value);
        else if (key == "seed")
            seed = std::stoi(value);
        else if (key == "thin")
            thin = std::stoi(value);
        else if (key == "S")
            S = parseVarianceComponents(value);
        else if (key == "numThread")
            numThread = std::stoi(value);
        else if (key.substr(0, 2) == "//" || key.substr(0, 1) == "#")
            continue;
        else
            throw("\nError: invalid option " + key + " " + value + "\n");
    }
}

}  // namespace brr
