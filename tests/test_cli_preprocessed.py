"""Reading the reference's preprocessed files back into genotype codes (CPU).

The reference's ppbayes maps the file its --preprocess wrote
(src/analysisrunner.cpp:186-196, src/data.cpp:52-75): dense records of N
standardised doubles (src/densemarker.cpp:34-49) or ragged records of four
statistics and the Zones/Ztwos/Zmissing index lists
(src/raggedsparsemarker.cpp:43-66), or Eigen sparse records of the statistics
and the Zg entries (src/eigensparsemarker.cpp:39-58), with a
{pos, compressedSize, originalSize} index per marker (src/common.h:57-61).  Files are written here in that layout
from the oracle's builders; `brr --export-bed` must return the original BED
payload bit for bit from ragged and Eigen files, and from dense files codes that
standardise to the same columns (identical codes where all three genotype
classes occur), including markers where genotype classes are absent.
"""
import json
import subprocess

import numpy as np
import pytest

import oracle_lib as O
from bayesrrcmd_gb300 import plink
from bayesrrcmd_gb300.build import build_cli


@pytest.fixture(scope="module")
def brr():
    return str(build_cli())


def dataset(tmp_path, N=333, M=60, missing=0.02, seed=5):
    g, _ = plink.synth_genotypes(N, M, seed=seed, missing=missing)
    # rare and one-sided markers: genotype 2 absent, genotype 0 absent
    rng = np.random.default_rng(seed + 1)
    g[0] = (rng.random(N) < 0.01).astype(np.int8)
    g[0, 0] = 1
    g[1] = 2 - (rng.random(N) < 0.05).astype(np.int8)
    g[1, 1] = 1
    g[2] = np.where(rng.random(N) < 0.5, 0, 2).astype(np.int8)
    if missing > 0:
        g[0, 5] = -1
        g[2, 7] = -1
    payload = plink.encode_bed(g)
    prefix = tmp_path / "pp"
    plink.write_plink(prefix, payload, N)
    return prefix, payload, N, M


def write_index(path, sizes):
    pos = np.concatenate([[0], np.cumsum(sizes)[:-1]]).astype(np.uint64)
    idx = np.stack([pos, np.asarray(sizes, np.uint64), np.asarray(sizes, np.uint64)], axis=1)
    idx.astype(np.uint64).tofile(path)


def write_dense(prefix, payload, N):
    cols = O.dense_columns(payload, N)
    cols.astype(np.float64).tofile(str(prefix) + ".ppbed")
    write_index(str(prefix) + ".ppbedindex", [N * 8] * cols.shape[0])
    return cols


def write_ragged(prefix, payload, N):
    rc, stats = O.ragged_stats(payload, N)
    lists = O.ragged_lists(payload, N)
    M = payload.shape[0]
    sizes = []
    with open(str(prefix) + ".ragged.sparsebed", "wb") as f:
        for j in range(M):
            f.write(stats[j].astype(np.float64).tobytes())
            size = 32
            for off, ix in lists:
                part = ix[off[j]:off[j + 1]].astype(np.int32)
                f.write(np.uint64(part.size).tobytes())
                f.write(part.tobytes())
                size += 8 + 4 * part.size
            sizes.append(size)
    write_index(str(prefix) + ".ragged.sparsebedindex", sizes)


def write_eigen(prefix, payload, N):
    """Records of src/eigensparsemarker.cpp:39-58: stats, int64 count, double
    values (1, 2, or the mean at missing genotypes), int32 indices."""
    rc, stats = O.eigen_stats(payload, N)
    assert rc == 0
    lists = O.ragged_lists(payload, N)
    M = payload.shape[0]
    sizes = []
    with open(str(prefix) + ".eigen.sparsebed", "wb") as f:
        for j in range(M):
            parts = [ix[off[j]:off[j + 1]] for off, ix in lists]
            vals = [np.full(len(parts[0]), 1.0), np.full(len(parts[1]), 2.0), np.full(len(parts[2]), stats[j, 0])]
            rows = np.concatenate(parts).astype(np.int32)
            order = np.argsort(rows, kind="stable")
            f.write(stats[j].astype(np.float64).tobytes())
            f.write(np.int64(rows.size).tobytes())
            f.write(np.concatenate(vals)[order].astype(np.float64).tobytes())
            f.write(rows[order].tobytes())
            sizes.append(40 + 12 * rows.size)
    write_index(str(prefix) + ".eigen.sparsebedindex", sizes)
    return stats


def export(brr, prefix, out, *extra):
    return subprocess.run([brr, "--bfile", str(prefix), "--export-bed", str(out), *extra],
                          capture_output=True, text=True)


def read_payload(path, N, M):
    raw = np.fromfile(path, np.uint8)
    assert raw[:3].tolist() == [0x6C, 0x1B, 0x01]
    return raw[3:].reshape(M, (N + 3) // 4)


@pytest.mark.parametrize("missing", [0.0, 0.02])
def test_dense_preprocessed_back_to_bed(brr, tmp_path, missing):
    """A standardised column does not change under g -> a*g + b with a > 0, so
    with two genotype classes present {0,1}, {1,2} and {0,2} give the same
    column: codes are pinned where all three classes occur, the standardised
    columns everywhere (the sampler sees only those)."""
    prefix, payload, N, M = dataset(tmp_path, missing=missing)
    cols = write_dense(prefix, payload, N)
    r = export(brr, prefix, tmp_path / "back.bed")
    assert r.returncode == 0, r.stderr
    back = read_payload(tmp_path / "back.bed", N, M)
    np.testing.assert_allclose(O.dense_columns(back, N), cols, rtol=1e-12, atol=1e-12)
    g = plink.decode_bed(payload, N)
    full = np.array([all((g[j] == c).any() for c in (0, 1, 2)) for j in range(M)])
    assert full.sum() > M // 2
    np.testing.assert_array_equal(back[full], payload[full])


@pytest.mark.parametrize("missing", [0.0, 0.02])
def test_ragged_preprocessed_back_to_bed(brr, tmp_path, missing):
    prefix, payload, N, M = dataset(tmp_path, missing=missing)
    write_ragged(prefix, payload, N)
    r = export(brr, prefix, tmp_path / "back.bed", "--sparse-data", "ragged")
    assert r.returncode == 0, r.stderr
    np.testing.assert_array_equal(read_payload(tmp_path / "back.bed", N, M), payload)


def test_dense_column_that_is_not_a_genotype_column_is_an_error(brr, tmp_path):
    prefix, payload, N, M = dataset(tmp_path, missing=0.0)
    cols = write_dense(prefix, payload, N)
    cols[3, :5] = [0.1, 0.2, 0.3, 0.4, 0.5]   # five distinct values
    cols.astype(np.float64).tofile(str(prefix) + ".ppbed")
    r = export(brr, prefix, tmp_path / "back.bed")
    assert r.returncode == 1 and "marker 3" in r.stderr


def test_dense_column_with_wrong_values_is_an_error(brr, tmp_path):
    prefix, payload, N, M = dataset(tmp_path, missing=0.0)
    cols = write_dense(prefix, payload, N)
    cols[4] *= 1.5   # three classes, but not standardised
    cols.astype(np.float64).tofile(str(prefix) + ".ppbed")
    r = export(brr, prefix, tmp_path / "back.bed")
    assert r.returncode == 1 and "marker 4" in r.stderr


def test_compressed_records_are_refused(brr, tmp_path):
    prefix, payload, N, M = dataset(tmp_path, missing=0.0)
    write_dense(prefix, payload, N)
    idx = np.fromfile(str(prefix) + ".ppbedindex", np.uint64).reshape(M, 3)
    idx[0, 1] -= 8   # compressedSize != originalSize, as with --compress
    idx.tofile(str(prefix) + ".ppbedindex")
    r = export(brr, prefix, tmp_path / "back.bed")
    assert r.returncode == 1 and "compressed" in r.stderr


def test_ragged_index_out_of_range_is_an_error(brr, tmp_path):
    prefix, payload, N, M = dataset(tmp_path, missing=0.0)
    write_ragged(prefix, payload, N)
    raw = bytearray(open(str(prefix) + ".ragged.sparsebed", "rb").read())
    n_ones = int(np.frombuffer(raw, np.uint64, 1, 32)[0])
    assert n_ones > 0
    raw[40:44] = np.int32(N + 5).tobytes()   # first index of marker 0's Zones
    open(str(prefix) + ".ragged.sparsebed", "wb").write(bytes(raw))
    r = export(brr, prefix, tmp_path / "back.bed", "--sparse-data", "ragged")
    assert r.returncode == 1 and "out of range" in r.stderr


@pytest.mark.parametrize("missing", [0.0, 0.02])
def test_eigen_preprocessed_back_to_bed(brr, tmp_path, missing):
    prefix, payload, N, M = dataset(tmp_path, missing=missing)
    write_eigen(prefix, payload, N)
    r = export(brr, prefix, tmp_path / "back.bed", "--sparse-data", "eigen")
    assert r.returncode == 0, r.stderr
    np.testing.assert_array_equal(read_payload(tmp_path / "back.bed", N, M), payload)


def test_eigen_marker_with_mean_one(brr, tmp_path):
    """Genotype sum N: missing genotypes are stored as 1.0 like heterozygotes.
    The reader recovers the counts (hence the statistics) exactly; which
    entries it marks missing does not change Zg."""
    prefix, payload, N, M = dataset(tmp_path, missing=0.02)
    g = plink.decode_bed(payload, N)
    rng = np.random.default_rng(3)
    row = np.zeros(N, np.int8)
    perm = rng.permutation(N)
    row[perm[:100]] = 2
    row[perm[100:233]] = 1            # 2*100 + 133 = 333 = N
    row[perm[233:253]] = -1
    g[5] = row
    payload = plink.encode_bed(g)
    plink.write_plink(prefix, payload, N)
    stats = write_eigen(prefix, payload, N)
    assert stats[5, 0] == 1.0
    r = export(brr, prefix, tmp_path / "back.bed", "--sparse-data", "eigen")
    assert r.returncode == 0, r.stderr
    back = read_payload(tmp_path / "back.bed", N, M)
    keep = np.arange(M) != 5
    np.testing.assert_array_equal(back[keep], payload[keep])
    np.testing.assert_array_equal(O.counts(back, N)[5], O.counts(payload, N)[5])
    assert np.array_equal(O.eigen_stats(back, N)[1][5], stats[5])
    gb = plink.decode_bed(back, N)[5]
    Zg = lambda r: np.where(r < 0, 1.0, r.astype(float))
    np.testing.assert_array_equal(Zg(gb), Zg(row))


def test_eigen_value_that_is_not_a_genotype_is_an_error(brr, tmp_path):
    prefix, payload, N, M = dataset(tmp_path, missing=0.0)
    write_eigen(prefix, payload, N)
    raw = bytearray(open(str(prefix) + ".eigen.sparsebed", "rb").read())
    assert int(np.frombuffer(raw, np.int64, 1, 32)[0]) > 0
    raw[40:48] = np.float64(1.5).tobytes()   # marker 0's first value
    open(str(prefix) + ".eigen.sparsebed", "wb").write(bytes(raw))
    r = export(brr, prefix, tmp_path / "back.bed", "--sparse-data", "eigen")
    assert r.returncode == 1 and "marker 0" in r.stderr


# Compressed files: the reference's --preprocess --compress writes each record
# as a zlib stream at the default level (deflateInit(-1), src/compression.cpp:5-11,
# src/marker.cpp:10-34) and the index holds {pos, compressedSize, originalSize};
# its ppbayes inflates every record when --compress is given
# (src/limitsequencegraph.cpp:19-23).
PP_FILES = {None: (".ppbed", ".ppbedindex"), "ragged": (".ragged.sparsebed", ".ragged.sparsebedindex"),
            "eigen": (".eigen.sparsebed", ".eigen.sparsebedindex")}


def needs_zlib(brr):
    r = subprocess.run([brr, "--print-options"], capture_output=True, text=True)
    if not json.loads(r.stdout.strip().splitlines()[-1])["zlib"]:
        pytest.skip("brr was built without zlib")


def write_kind(prefix, payload, N, sparse):
    {None: write_dense, "ragged": write_ragged, "eigen": write_eigen}[sparse](prefix, payload, N)


def compress_files(prefix, sparse, M):
    import zlib
    pp, ix = (str(prefix) + s for s in PP_FILES[sparse])
    idx = np.fromfile(ix, np.uint64).reshape(M, 3)
    raw = open(pp, "rb").read()
    out, entries, pos = [], [], 0
    for j in range(M):
        rec = raw[int(idx[j, 0]):int(idx[j, 0]) + int(idx[j, 2])]
        z = zlib.compress(rec)
        out.append(z)
        entries.append((pos, len(z), len(rec)))
        pos += len(z)
    open(pp, "wb").write(b"".join(out))
    np.array(entries, np.uint64).tofile(ix)
    return np.array(entries, np.uint64)


def sparse_args(sparse):
    return [] if sparse is None else ["--sparse-data", sparse]


@pytest.mark.parametrize("sparse", [None, "ragged", "eigen"])
def test_compressed_files_are_read_with_compress(brr, tmp_path, sparse):
    needs_zlib(brr)
    prefix, payload, N, M = dataset(tmp_path, missing=0.02)
    write_kind(prefix, payload, N, sparse)
    r = export(brr, prefix, tmp_path / "plain.bed", *sparse_args(sparse))
    assert r.returncode == 0, r.stderr
    entries = compress_files(prefix, sparse, M)
    assert (entries[:, 1] != entries[:, 2]).all()
    r = export(brr, prefix, tmp_path / "no_flag.bed", *sparse_args(sparse))
    assert r.returncode == 1 and "--compress" in r.stderr
    r = export(brr, prefix, tmp_path / "inflated.bed", "--compress", *sparse_args(sparse))
    assert r.returncode == 0, r.stderr
    np.testing.assert_array_equal(read_payload(tmp_path / "inflated.bed", N, M),
                                  read_payload(tmp_path / "plain.bed", N, M))


def test_uncompressed_files_are_read_as_stored_with_compress(brr, tmp_path):
    needs_zlib(brr)
    prefix, payload, N, M = dataset(tmp_path, missing=0.02)
    write_ragged(prefix, payload, N)
    r = export(brr, prefix, tmp_path / "back.bed", "--compress", "--sparse-data", "ragged")
    assert r.returncode == 0, r.stderr
    np.testing.assert_array_equal(read_payload(tmp_path / "back.bed", N, M), payload)


def test_corrupt_compressed_record_is_an_error(brr, tmp_path):
    needs_zlib(brr)
    prefix, payload, N, M = dataset(tmp_path, missing=0.0)
    write_ragged(prefix, payload, N)
    entries = compress_files(prefix, "ragged", M)
    pp = str(prefix) + ".ragged.sparsebed"
    data = bytearray(open(pp, "rb").read())
    at = int(entries[3, 0] + entries[3, 1] // 2)
    data[at] ^= 0x5A
    open(pp, "wb").write(bytes(data))
    r = export(brr, prefix, tmp_path / "back.bed", "--compress", "--sparse-data", "ragged")
    assert r.returncode == 1 and "marker 3" in r.stderr and "inflate" in r.stderr


COMPRESS_DRIVER = r"""
#include <cstdio>
#include <cstdlib>
#include <string>
#include "data.h"
int main(int argc, char **argv)
{
    try {
        brr::compressPreprocessed(argv[1], argv[2], std::atoll(argv[3]));
    } catch (const std::string &e) {
        std::fprintf(stderr, "%s\n", e.c_str());
        return 1;
    }
    return 0;
}
"""


@pytest.fixture(scope="module")
def compressor(brr, tmp_path_factory):
    """compressPreprocessed (the writer side of --preprocess --compress) built
    from the brr sources with zlib, as a small driver."""
    import shutil
    needs_zlib(brr)
    from bayesrrcmd_gb300.build import HOST
    d = tmp_path_factory.mktemp("compress")
    (d / "driver.cpp").write_text(COMPRESS_DRIVER)
    cxx = shutil.which("g++") or shutil.which("c++")
    r = subprocess.run([cxx, "-O2", "-std=c++17", "-DBRR_WITH_ZLIB", f"-I{HOST}", str(d / "driver.cpp"),
                        str(HOST / "data.cpp"), "-o", str(d / "compress"), "-lz"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return str(d / "compress")


@pytest.mark.parametrize("sparse", [None, "ragged", "eigen"])
def test_written_compressed_files_round_trip(brr, compressor, tmp_path, sparse):
    import zlib
    prefix, payload, N, M = dataset(tmp_path, missing=0.02)
    write_kind(prefix, payload, N, sparse)
    pp, ix = (str(prefix) + s for s in PP_FILES[sparse])
    before = np.fromfile(ix, np.uint64).reshape(M, 3)
    raw = open(pp, "rb").read()
    records = [raw[int(e[0]):int(e[0]) + int(e[2])] for e in before]
    r = export(brr, prefix, tmp_path / "plain.bed", *sparse_args(sparse))
    assert r.returncode == 0, r.stderr
    r = subprocess.run([compressor, pp, ix, str(M)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    after = np.fromfile(ix, np.uint64).reshape(M, 3)
    np.testing.assert_array_equal(after[:, 2], before[:, 2])
    np.testing.assert_array_equal(after[1:, 0], np.cumsum(after[:-1, 1]))
    packed = open(pp, "rb").read()
    assert len(packed) == int(after[-1, 0] + after[-1, 1])
    for j, e in enumerate(after):
        assert zlib.decompress(packed[int(e[0]):int(e[0] + e[1])]) == records[j]
    r = export(brr, prefix, tmp_path / "back.bed", "--compress", *sparse_args(sparse))
    assert r.returncode == 0, r.stderr
    np.testing.assert_array_equal(read_payload(tmp_path / "back.bed", N, M),
                                  read_payload(tmp_path / "plain.bed", N, M))
    # a second pass refuses records that are compressed already
    r = subprocess.run([compressor, pp, ix, str(M)], capture_output=True, text=True)
    assert r.returncode == 1 and "compressed already" in r.stderr
