"""Reading the reference's preprocessed files back into genotype codes (CPU).

The reference's ppbayes maps the file its --preprocess wrote
(src/analysisrunner.cpp:186-196, src/data.cpp:52-75): dense records of N
standardised doubles (src/densemarker.cpp:34-49) or ragged records of four
statistics and the Zones/Ztwos/Zmissing index lists
(src/raggedsparsemarker.cpp:43-66), with a {pos, compressedSize, originalSize}
index per marker (src/common.h:57-61).  Files are written here in that layout
from the oracle's builders; `brr --export-bed` must return the original BED
payload bit for bit from ragged files, and from dense files codes that
standardise to the same columns (identical codes where all three genotype
classes occur), including markers where genotype classes are absent.
"""
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
