#include "data.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <set>
#include <sstream>
#include <unordered_set>

#if defined(BRR_WITH_ZLIB)
#include <zlib.h>
#endif

namespace brr {

void Data::readFamFile(const std::string &famFile)
{
    std::ifstream in(famFile.c_str());
    if (!in)
        throw("Error: can not open the file [" + famFile + "] to read.");
    std::cout << "Reading PLINK FAM file from [" + famFile + "]." << std::endl;
    indIds.clear();
    std::unordered_set<std::string> seen;
    std::string fid, pid, dad, mom, sex, phen;
    while (in >> fid >> pid >> dad >> mom >> sex >> phen) {
        const std::string id = fid + ":" + pid;
        if (!seen.insert(id).second)
            throw("Error: Duplicate individual ID found: \"" + fid + "\t" + pid + "\".");
        indIds.push_back(id);
    }
    std::cout << indIds.size() << " individuals to be included from [" + famFile + "]." << std::endl;
}

void Data::readBimFile(const std::string &bimFile)
{
    std::ifstream in(bimFile.c_str());
    if (!in)
        throw("Error: can not open the file [" + bimFile + "] to read.");
    std::cout << "Reading PLINK BIM file from [" + bimFile + "]." << std::endl;
    snpIds.clear();
    std::unordered_set<std::string> seen;
    std::string chr, id, gen, phys, a1, a2;
    while (in >> chr >> id >> gen >> phys >> a1 >> a2) {
        if (!seen.insert(id).second)
            throw("Error: Duplicate SNP ID found: \"" + id + "\".");
        snpIds.push_back(id);
    }
    G.assign(snpIds.size(), 0);
    std::cout << snpIds.size() << " SNPs to be included from [" + bimFile + "]." << std::endl;
}

// The value of every listed, known individual whose phenotype is not "NA", in
// file order; the reference packs these values without re-aligning them to
// the .fam order (src/data.cpp:350-361).
void Data::readPhenotypeFile(const std::string &phenFile)
{
    std::ifstream in(phenFile.c_str());
    if (!in)
        throw("Error: can not open the phenotype file [" + phenFile + "] to read.");
    std::cout << "Reading phenotypes from [" + phenFile + "]." << std::endl;
    std::unordered_set<std::string> known(indIds.begin(), indIds.end());
    y.clear();
    std::string line;
    while (std::getline(in, line)) {
        std::istringstream ss(line);
        std::string f, i, v;
        if (!(ss >> f >> i >> v))
            continue;
        if (known.count(f + ":" + i) && v != "NA")
            y.push_back((float)std::atof(v.c_str()));
    }
}

void Data::readGroupFile(const std::string &groupFile)
{
    std::ifstream in(groupFile);
    if (!in.is_open())
        throw("Error: can not open the group file [" + groupFile + "] to read.");
    G.clear();
    std::string snp;
    int g;
    while (in >> snp >> g)
        G.push_back(g);
    std::set<int> distinct(G.begin(), G.end());
    numGroups = (unsigned)distinct.size();
    std::cout << "Groups read from file: " << numGroups << std::endl;
}

std::vector<uint8_t> readBedPayload(const std::string &bedFile, int64_t N, int64_t M)
{
    std::ifstream in(bedFile, std::ios::binary);
    if (!in)
        throw("Error: can not open the file [" + bedFile + "] to read.");
    char header[3];
    in.read(header, 3);
    if (!in || (unsigned char)header[0] != 0x6c || (unsigned char)header[1] != 0x1b ||
        (unsigned char)header[2] != 0x01)
        throw std::string("Error: Incorrect first three bytes of bed file");
    const int64_t bytes = M * ((N + 3) / 4);
    std::vector<uint8_t> payload((size_t)bytes);
    in.read(reinterpret_cast<char *>(payload.data()), bytes);
    if (in.gcount() != bytes)
        throw std::string("Error: problem with the BED file ... has the FAM/BIM file been changed?");
    char extra;
    if (in.read(&extra, 1))
        throw std::string("Error: problem with the BED file ... has the FAM/BIM file been changed?");
    return payload;
}

namespace {
void writeIndexEntry(std::ofstream &idx, uint64_t pos, uint64_t size)
{
    idx.write(reinterpret_cast<const char *>(&pos), sizeof pos);
    idx.write(reinterpret_cast<const char *>(&size), sizeof size);
    idx.write(reinterpret_cast<const char *>(&size), sizeof size);
}
}  // namespace

void writeDensePreprocessed(const std::string &ppFile, const std::string &indexFile, int64_t N, int64_t M,
                            const double *lut, const uint8_t *bed)
{
    std::ofstream out(ppFile, std::ios::binary), idx(indexFile, std::ios::binary);
    if (!out || !idx)
        throw("Error: Unable to open the preprocessed bed file [" + ppFile + "] for writing.");
    const int64_t cb = (N + 3) / 4;
    std::vector<double> col((size_t)N);
    uint64_t pos = 0;
    for (int64_t j = 0; j < M; ++j) {
        const uint8_t *c = bed + j * cb;
        for (int64_t i = 0; i < N; ++i)
            col[i] = lut[4 * j + ((c[i >> 2] >> (2 * (i & 3))) & 3)];
        const uint64_t size = (uint64_t)N * sizeof(double);
        out.write(reinterpret_cast<const char *>(col.data()), (std::streamsize)size);
        writeIndexEntry(idx, pos, size);
        pos += size;
    }
}

void writeRaggedPreprocessed(const std::string &ppFile, const std::string &indexFile, int64_t M, const double *stats,
                             const int64_t *off[3], const int32_t *idx3[3])
{
    std::ofstream out(ppFile, std::ios::binary), idx(indexFile, std::ios::binary);
    if (!out || !idx)
        throw("Error: Unable to open the preprocessed bed file [" + ppFile + "] for writing.");
    uint64_t pos = 0;
    for (int64_t j = 0; j < M; ++j) {
        out.write(reinterpret_cast<const char *>(stats + 4 * j), 4 * sizeof(double));
        uint64_t size = 4 * sizeof(double);
        for (int k = 0; k < 3; ++k) {
            const uint64_t n = (uint64_t)(off[k][j + 1] - off[k][j]);
            out.write(reinterpret_cast<const char *>(&n), sizeof n);
            if (n)
                out.write(reinterpret_cast<const char *>(idx3[k] + off[k][j]), (std::streamsize)(n * sizeof(int32_t)));
            size += sizeof n + n * sizeof(int32_t);
        }
        writeIndexEntry(idx, pos, size);
        pos += size;
    }
}

void writeEigenPreprocessed(const std::string &ppFile, const std::string &indexFile, int64_t M, const double *stats,
                            const int64_t *off[3], const int32_t *idx3[3])
{
    std::ofstream out(ppFile, std::ios::binary), idx(indexFile, std::ios::binary);
    if (!out || !idx)
        throw("Error: Unable to open the preprocessed bed file [" + ppFile + "] for writing.");
    uint64_t pos = 0;
    std::vector<double> values;
    std::vector<int32_t> rows;
    for (int64_t j = 0; j < M; ++j) {
        // entries in ascending individual order: 1, 2, or the mean at missing genotypes
        const double val[3] = {1.0, 2.0, stats[4 * j]};
        int64_t q[3], e[3];
        for (int k = 0; k < 3; ++k) {
            q[k] = off[k][j];
            e[k] = off[k][j + 1];
        }
        values.clear();
        rows.clear();
        for (;;) {
            int kb = -1;
            for (int k = 0; k < 3; ++k)
                if (q[k] < e[k] && (kb < 0 || idx3[k][q[k]] < idx3[kb][q[kb]]))
                    kb = k;
            if (kb < 0)
                break;
            values.push_back(val[kb]);
            rows.push_back(idx3[kb][q[kb]++]);
        }
        const int64_t count = (int64_t)values.size();
        out.write(reinterpret_cast<const char *>(stats + 4 * j), 4 * sizeof(double));
        out.write(reinterpret_cast<const char *>(&count), sizeof count);
        if (count) {
            out.write(reinterpret_cast<const char *>(values.data()), (std::streamsize)(count * sizeof(double)));
            out.write(reinterpret_cast<const char *>(rows.data()), (std::streamsize)(count * sizeof(int32_t)));
        }
        const uint64_t size = 4 * sizeof(double) + sizeof count + (uint64_t)count * (sizeof(double) + sizeof(int32_t));
        writeIndexEntry(idx, pos, size);
        pos += size;
    }
}

std::vector<IndexEntry> readIndex(const std::string &indexFile, int64_t M)
{
    std::vector<IndexEntry> v((size_t)M);
    std::ifstream in(indexFile, std::ios::binary);
    if (!in)
        throw std::string("Error: Failed to open compressed preprocessed bed file index");
    in.read(reinterpret_cast<char *>(v.data()), (std::streamsize)(M * sizeof(IndexEntry)));
    if (in.gcount() != (std::streamsize)(M * sizeof(IndexEntry)))
        throw std::string("Error: preprocessed index is shorter than the number of SNPs");
    return v;
}

namespace {

void setCode(std::vector<uint8_t> &bed, int64_t cb, int64_t j, int64_t i, unsigned code)
{
    uint8_t &b = bed[(size_t)(j * cb + (i >> 2))];
    const unsigned sh = 2u * (unsigned)(i & 3);
    b = (uint8_t)((b & ~(3u << sh)) | (code << sh));
}

std::vector<uint8_t> allHomozygousMajor(int64_t N, int64_t M)
{
    const int64_t cb = (N + 3) / 4;
    std::vector<uint8_t> bed((size_t)(M * cb), 0);
    for (int64_t j = 0; j < M; ++j)
        for (int64_t i = 0; i < N; ++i)
            setCode(bed, cb, j, i, 3u);   // code 11: genotype 0
    return bed;
}

std::ifstream openPreprocessed(const std::string &ppFile)
{
    std::ifstream in(ppFile, std::ios::binary);
    if (!in)
        throw std::string("Error: Failed to open preprocessed bed file [" + ppFile + "]");
    return in;
}

// Inflates a zlib stream (the format deflateInit writes) into exactly
// plain.size() bytes; false when the bytes are not such a stream or this build
// has no zlib.
bool inflateRecord(const std::vector<char> &packed, std::vector<char> &plain)
{
#if defined(BRR_WITH_ZLIB)
    uLongf got = (uLongf)plain.size();
    const int rc = uncompress(reinterpret_cast<Bytef *>(plain.data()), &got,
                              reinterpret_cast<const Bytef *>(packed.data()), (uLong)packed.size());
    return rc == Z_OK && got == (uLongf)plain.size();
#else
    (void)packed;
    (void)plain;
    return false;
#endif
}

// Positions a stream at a marker's record: the file itself for uncompressed
// files, or an in-memory copy of the inflated record for compressed ones
// (Marker::decompress then read, src/marker.cpp:36-55).
class RecordReader {
public:
    RecordReader(const std::string &ppFile, bool compressed) : file_(openPreprocessed(ppFile)), compressed_(compressed) {}

    std::istream &open(const IndexEntry &e, int64_t j)
    {
        const std::string which = " of marker " + std::to_string(j);
        if (!compressed_) {
            if (e.compressedSize != e.originalSize)
                throw std::string("Error: the record" + which +
                                  " of the preprocessed file is compressed; read it with --compress");
            file_.clear();
            file_.seekg((std::streamoff)e.pos);
            return file_;
        }
        packed_.resize((size_t)e.compressedSize);
        file_.clear();
        file_.seekg((std::streamoff)e.pos);
        file_.read(packed_.data(), (std::streamsize)packed_.size());
        if (!file_)
            throw std::string("Error: the preprocessed bed file ends before the record" + which);
        plain_.resize((size_t)e.originalSize);
        if (!inflateRecord(packed_, plain_)) {
            if (e.compressedSize != e.originalSize)
                throw std::string(canReadCompressed()
                                      ? "Error: the compressed record" + which + " does not inflate to its size"
                                      : "Error: the record" + which +
                                            " is compressed and this build of brr has no zlib to read it");
            plain_ = packed_;   // stored without compression
        }
        mem_.str(std::string(plain_.data(), plain_.size()));
        mem_.clear();
        return mem_;
    }

private:
    std::ifstream file_;
    bool compressed_;
    std::vector<char> packed_, plain_;
    std::istringstream mem_;
};

// Standardised value per 2-bit code (0: genotype 2, 1: missing, 2: genotype 1,
// 3: genotype 0) of a dense column with the given class counts: missing values
// take the mean of the non-missing ones, the column is centred and scaled to
// a squared norm of N-1 (src/densemarkerbuilder.cpp:44-59).
bool standardisedValues(int64_t N, const int64_t n[4], double v[4])
{
    const int64_t n2 = n[0], nm = n[1], n1 = n[2], n0 = n[3];
    if (N - nm <= 0 || N < 2)
        return false;
    const double S = (double)n1 + 2.0 * (double)n2;
    const double mean = S / (double)(N - nm);
    const double colmean = (S + (double)nm * mean) / (double)N;
    const double d2 = 2.0 - colmean, d1 = 1.0 - colmean, d0 = -colmean, dm = mean - colmean;
    const double sqn = (double)n2 * d2 * d2 + (double)n1 * d1 * d1 + (double)n0 * d0 * d0 + (double)nm * dm * dm;
    if (!(sqn > 0.0))
        return false;
    const double sigma = 1.0 / std::sqrt(sqn / (double)(N - 1));
    v[0] = d2 * sigma;
    v[1] = dm * sigma;
    v[2] = d1 * sigma;
    v[3] = d0 * sigma;
    return true;
}

}  // namespace

std::vector<uint8_t> readRaggedPreprocessedAsBed(const std::string &ppFile, const std::string &indexFile, int64_t N,
                                                 int64_t M, bool compressed)
{
    const std::vector<IndexEntry> index = readIndex(indexFile, M);
    RecordReader records(ppFile, compressed);
    std::vector<uint8_t> bed = allHomozygousMajor(N, M);
    const int64_t cb = (N + 3) / 4;
    const unsigned listCode[3] = {2u, 0u, 1u};   // Zones: genotype 1, Ztwos: genotype 2, Zmissing
    std::vector<int32_t> ids;
    for (int64_t j = 0; j < M; ++j) {
        std::istream &in = records.open(index[(size_t)j], j);
        double stats[4];
        in.read(reinterpret_cast<char *>(stats), sizeof stats);
        uint64_t used = sizeof stats;
        for (int k = 0; k < 3; ++k) {
            uint64_t n = 0;
            in.read(reinterpret_cast<char *>(&n), sizeof n);
            if (!in || n > (uint64_t)N)
                throw std::string("Error: malformed ragged record of marker " + std::to_string(j));
            ids.resize((size_t)n);
            if (n)
                in.read(reinterpret_cast<char *>(ids.data()), (std::streamsize)(n * sizeof(int32_t)));
            if (!in)
                throw std::string("Error: malformed ragged record of marker " + std::to_string(j));
            for (int32_t i : ids) {
                if (i < 0 || i >= N)
                    throw std::string("Error: individual index out of range in marker " + std::to_string(j));
                setCode(bed, cb, j, i, listCode[k]);
            }
            used += sizeof n + n * sizeof(int32_t);
        }
        if (used != index[(size_t)j].originalSize)
            throw std::string("Error: ragged record size of marker " + std::to_string(j) + " does not match the index");
    }
    return bed;
}

std::vector<uint8_t> readEigenPreprocessedAsBed(const std::string &ppFile, const std::string &indexFile, int64_t N,
                                                int64_t M, bool compressed)
{
    const std::vector<IndexEntry> index = readIndex(indexFile, M);
    RecordReader records(ppFile, compressed);
    std::vector<uint8_t> bed = allHomozygousMajor(N, M);
    const int64_t cb = (N + 3) / 4;
    std::vector<double> values;
    std::vector<int32_t> rows;
    std::vector<int64_t> ones;
    for (int64_t j = 0; j < M; ++j) {
        const std::string which = " of marker " + std::to_string(j);
        std::istream &in = records.open(index[(size_t)j], j);
        double stats[4];
        int64_t count = -1;
        in.read(reinterpret_cast<char *>(stats), sizeof stats);
        in.read(reinterpret_cast<char *>(&count), sizeof count);
        if (!in || count < 0 || count > N)
            throw std::string("Error: malformed Eigen sparse record" + which);
        values.resize((size_t)count);
        rows.resize((size_t)count);
        if (count) {
            in.read(reinterpret_cast<char *>(values.data()), (std::streamsize)(count * sizeof(double)));
            in.read(reinterpret_cast<char *>(rows.data()), (std::streamsize)(count * sizeof(int32_t)));
        }
        if (!in)
            throw std::string("Error: malformed Eigen sparse record" + which);
        const uint64_t used = 4 * sizeof(double) + sizeof count + (uint64_t)count * (sizeof(double) + sizeof(int32_t));
        if (used != index[(size_t)j].originalSize)
            throw std::string("Error: Eigen sparse record size" + which + " does not match the index");
        // Zg holds 1, 2, or the mean (stats[0]) at missing genotypes
        // (src/eigensparsemarkerbuilder.cpp:62-72)
        const double mean = stats[0];
        int64_t twos = 0;
        ones.clear();
        for (int64_t q = 0; q < count; ++q) {
            const int32_t i = rows[(size_t)q];
            if (i < 0 || i >= N || (q > 0 && i <= rows[(size_t)q - 1]))
                throw std::string("Error: individual index out of range or out of order" + which);
            const double v = values[(size_t)q];
            if (v == 1.0) {
                setCode(bed, cb, j, i, 2u);
                ones.push_back(q);
            } else if (v == 2.0) {
                setCode(bed, cb, j, i, 0u);
                ++twos;
            } else if (v == mean) {
                setCode(bed, cb, j, i, 1u);
            } else {
                throw std::string("Error: value other than 1, 2 or the marker mean" + which);
            }
        }
        if (mean == 1.0) {
            // a missing genotype stored as the mean 1.0 looks like a heterozygote;
            // the genotype sum is N, so N - 2*twos of the 1.0 entries are
            // heterozygotes and the rest are missing.  Which ones are missing
            // does not change the chain: Zg, the statistics, the dot products
            // and the residual updates (zero for a value equal to the mean) are
            // the same, so the last entries are marked missing.
            const int64_t het = N - 2 * twos;
            if (het < 0 || het > (int64_t)ones.size())
                throw std::string("Error: Eigen sparse record" + which + " does not match its mean");
            for (size_t q = (size_t)het; q < ones.size(); ++q)
                setCode(bed, cb, j, rows[(size_t)ones[q]], 1u);
        }
    }
    return bed;
}

std::vector<uint8_t> readDensePreprocessedAsBed(const std::string &ppFile, const std::string &indexFile, int64_t N,
                                                int64_t M, bool compressed)
{
    const std::vector<IndexEntry> index = readIndex(indexFile, M);
    RecordReader records(ppFile, compressed);
    std::vector<uint8_t> bed((size_t)(M * ((N + 3) / 4)), 0);
    const int64_t cb = (N + 3) / 4;
    std::vector<double> col((size_t)N);
    for (int64_t j = 0; j < M; ++j) {
        if (index[(size_t)j].originalSize != (uint64_t)N * sizeof(double))
            throw std::string("Error: dense record of marker " + std::to_string(j) + " is not N doubles");
        std::istream &in = records.open(index[(size_t)j], j);
        in.read(reinterpret_cast<char *>(col.data()), (std::streamsize)(N * sizeof(double)));
        if (!in)
            throw std::string("Error: the preprocessed bed file ends before marker " + std::to_string(j));
        // distinct values (one per genotype class present, identical within a class)
        double val[4];
        int64_t cnt[4] = {0, 0, 0, 0};
        int nd = 0;
        std::vector<uint8_t> cls((size_t)N);
        for (int64_t i = 0; i < N; ++i) {
            int k = 0;
            while (k < nd && !(val[k] == col[(size_t)i]))
                ++k;
            if (k == nd) {
                if (nd == 4 || std::isnan(col[(size_t)i]))
                    throw std::string("Error: marker " + std::to_string(j) +
                                      " of the preprocessed file is not a standardised genotype column");
                val[nd++] = col[(size_t)i];
            }
            ++cnt[k];
            cls[(size_t)i] = (uint8_t)k;
        }
        // the first assignment of distinct values to codes whose recomputed
        // standardised values reproduce the column
        int best[4] = {-1, -1, -1, -1};
        int perm[4] = {0, 1, 2, 3};
        bool found = false;
        do {
            int64_t n[4] = {0, 0, 0, 0};
            for (int k = 0; k < nd; ++k)
                n[perm[k]] = cnt[k];
            double v[4];
            if (!standardisedValues(N, n, v))
                continue;
            bool ok = true;
            for (int k = 0; k < nd && ok; ++k)
                ok = std::fabs(v[perm[k]] - val[k]) <= 1e-9 * std::max(1.0, std::fabs(val[k]));
            if (ok) {
                for (int k = 0; k < nd; ++k)
                    best[k] = perm[k];
                found = true;
            }
        } while (!found && std::next_permutation(perm, perm + 4));
        if (!found)
            throw std::string("Error: marker " + std::to_string(j) +
                              " of the preprocessed file does not match a standardised genotype column");
        for (int64_t i = 0; i < N; ++i)
            setCode(bed, cb, j, i, (unsigned)best[cls[(size_t)i]]);
    }
    return bed;
}

void compressPreprocessed(const std::string &ppFile, const std::string &indexFile, int64_t M)
{
#if defined(BRR_WITH_ZLIB)
    const std::vector<IndexEntry> index = readIndex(indexFile, M);
    const std::string tmpFile = ppFile + ".compressing";
    {
        std::ifstream in = openPreprocessed(ppFile);
        std::ofstream out(tmpFile, std::ios::binary | std::ios::trunc);
        if (!out)
            throw std::string("Error: Unable to open [" + tmpFile + "] for writing");
        std::ofstream idx(indexFile + ".compressing", std::ios::binary | std::ios::trunc);
        if (!idx)
            throw std::string("Error: Unable to open [" + indexFile + ".compressing] for writing");
        std::vector<char> plain;
        std::vector<Bytef> packed;
        uint64_t pos = 0;
        for (int64_t j = 0; j < M; ++j) {
            const IndexEntry &e = index[(size_t)j];
            if (e.compressedSize != e.originalSize)
                throw std::string("Error: marker " + std::to_string(j) + " is compressed already");
            plain.resize((size_t)e.originalSize);
            in.clear();
            in.seekg((std::streamoff)e.pos);
            in.read(plain.data(), (std::streamsize)plain.size());
            if (!in)
                throw std::string("Error: the preprocessed bed file ends before marker " + std::to_string(j));
            uLongf size = compressBound((uLong)plain.size());
            packed.resize((size_t)size);
            if (compress2(packed.data(), &size, reinterpret_cast<const Bytef *>(plain.data()), (uLong)plain.size(),
                          Z_DEFAULT_COMPRESSION) != Z_OK)
                throw std::string("Error: compressing marker " + std::to_string(j) + " failed");
            out.write(reinterpret_cast<const char *>(packed.data()), (std::streamsize)size);
            const IndexEntry ne{pos, (uint64_t)size, e.originalSize};
            idx.write(reinterpret_cast<const char *>(&ne), sizeof ne);
            pos += size;
        }
        if (!out || !idx)
            throw std::string("Error: writing the compressed preprocessed files failed");
    }
    if (std::rename(tmpFile.c_str(), ppFile.c_str()) != 0 ||
        std::rename((indexFile + ".compressing").c_str(), indexFile.c_str()) != 0)
        throw std::string("Error: replacing the preprocessed files with their compressed form failed");
#else
    (void)ppFile;
    (void)indexFile;
    (void)M;
    throw std::string("Error: --compress needs zlib, which this build of brr does not have");
#endif
}

bool canReadCompressed()
{
#if defined(BRR_WITH_ZLIB)
    return true;
#else
    return false;
#endif
}

void writeBedFile(const std::string &bedFile, const std::vector<uint8_t> &payload)
{
    std::ofstream out(bedFile, std::ios::binary);
    if (!out)
        throw std::string("Error: Unable to open [" + bedFile + "] for writing");
    const unsigned char magic[3] = {0x6c, 0x1b, 0x01};
    out.write(reinterpret_cast<const char *>(magic), 3);
    out.write(reinterpret_cast<const char *>(payload.data()), (std::streamsize)payload.size());
}

}  // namespace brr
