// PLINK metadata, phenotype and group readers and the preprocessed-file
// formats of the reference, for the host side of `brr`.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace brr {

struct IndexEntry {          // src/common.h:57-61: one per marker in the index file
    uint64_t pos = 0;
    uint64_t compressedSize = 0;
    uint64_t originalSize = 0;
};

struct Data {
    std::vector<std::string> indIds;     // "FID:IID", src/data.cpp:85-107
    std::vector<std::string> snpIds;     // src/data.cpp:109-133
    std::vector<float> y;                // src/data.cpp:334-365 (NA skipped, packed)
    std::vector<int32_t> G;              // group per marker, default 0
    unsigned numGroups = 1;
    int64_t numInds() const { return (int64_t)indIds.size(); }
    int64_t numSnps() const { return (int64_t)snpIds.size(); }

    void readFamFile(const std::string &famFile);        // throws std::string
    void readBimFile(const std::string &bimFile);        // throws std::string
    void readPhenotypeFile(const std::string &phenFile); // throws std::string
    void readGroupFile(const std::string &groupFile);    // throws std::string
};

// SNP-major BED payload without the 3-byte magic; throws on a bad magic or size
// (src/preprocessgraph.cpp:195-200, :36-41).
std::vector<uint8_t> readBedPayload(const std::string &bedFile, int64_t N, int64_t M);

// Preprocessed marker files (uncompressed layout of src/preprocessgraph.cpp:92-126):
// dense records are N doubles (src/densemarker.cpp:34-49); ragged records are
// {mean, sd, sqrdZ, Zsum} doubles then three (u64 count, int32[count]) lists
// (src/sparsemarker.cpp:43-58, src/raggedsparsemarker.cpp:43-66).
void writeDensePreprocessed(const std::string &ppFile, const std::string &indexFile, int64_t N, int64_t M,
                            const double *lut, const uint8_t *bedPayload);
void writeRaggedPreprocessed(const std::string &ppFile, const std::string &indexFile, int64_t M,
                             const double *stats, const int64_t *off[3], const int32_t *idx[3]);
// Eigen sparse records (src/eigensparsemarker.cpp:39-58): the four statistics,
// an int64 entry count, the entries' double values (1, 2, or the mean at
// missing genotypes) and their int32 individual indices, ascending.
void writeEigenPreprocessed(const std::string &ppFile, const std::string &indexFile, int64_t M,
                            const double *stats, const int64_t *off[3], const int32_t *idx[3]);
std::vector<IndexEntry> readIndex(const std::string &indexFile, int64_t M);

// Genotype codes in the BED payload layout (M x ceil(N/4) bytes, padding bits
// zero) rebuilt from a preprocessed file, so that `brr` consumes the files of
// the reference's --preprocess (src/analysisrunner.cpp:186-196 maps them for
// ppbayes).  Ragged records give the codes directly (ones, twos, missing lists);
// a dense record is the standardised column, whose at most four distinct values
// are matched to genotype classes by recomputing the dense builder's values
// (src/densemarkerbuilder.cpp:44-59) from the class counts each assignment
// implies.  With `compressed` (the reference's --compress, which decides how
// its LimitSequenceGraph reads records, src/limitsequencegraph.cpp:19-23 and
// src/analysis.cpp:21-24) every record is a zlib stream of the same bytes
// (src/marker.cpp:10-34, src/compression.cpp:101-126) and is inflated to its
// index entry's originalSize; a record that does not inflate but whose two
// sizes are equal is taken as stored (files written without compression).
// Without `compressed` a record whose sizes differ is an error.  Throws
// std::string on a malformed file.
std::vector<uint8_t> readRaggedPreprocessedAsBed(const std::string &ppFile, const std::string &indexFile, int64_t N,
                                                 int64_t M, bool compressed = false);
std::vector<uint8_t> readDensePreprocessedAsBed(const std::string &ppFile, const std::string &indexFile, int64_t N,
                                                int64_t M, bool compressed = false);
// Eigen sparse records give the codes from the entry values; when a marker's
// mean is exactly 1 its missing entries (stored as 1.0) are told apart from
// heterozygotes by count only, which leaves the chain unchanged.
std::vector<uint8_t> readEigenPreprocessedAsBed(const std::string &ppFile, const std::string &indexFile, int64_t N,
                                                int64_t M, bool compressed = false);
// Whether this build can inflate compressed records (zlib found when it was built).
bool canReadCompressed();
// Rewrites an uncompressed preprocessed file and its index in the layout of
// the reference's --compress (src/preprocessgraph.cpp:63-67, :104-122): each
// record deflated at the default level into one zlib stream, the index
// holding {pos, compressedSize, originalSize}.  Throws std::string on error or
// when this build has no zlib.
void compressPreprocessed(const std::string &ppFile, const std::string &indexFile, int64_t M);
// Writes a PLINK BED file (magic + SNP-major payload).
void writeBedFile(const std::string &bedFile, const std::vector<uint8_t> &payload);

}  // namespace brr
