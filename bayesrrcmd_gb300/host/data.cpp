#include "data.h"

#include <algorithm>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <set>
#include <sstream>
#include <unordered_set>

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

}  // namespace brr
