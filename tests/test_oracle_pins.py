"""Pins of the CPU oracle against what the reference itself provides.

The reference cannot be compiled here (Eigen, Boost.Random and TBB are
absent), so its chain outputs cannot be regenerated.  These tests pin the
oracle against the checkable facts the reference ships: the GeneFrq column of
its uk10k fixture, the sparse epsilon-update identity of its unit test, the
published Philox4x32-10 known-answer vectors for the replacement draw stream,
and the algebraic invariants of its dense standardisation.
"""
import io
import zipfile
from pathlib import Path

import numpy as np
import pytest

import oracle_lib as O
from refdir import reference_dir
from bayesrrcmd_gb300 import plink

REF = reference_dir()
GOLDEN = Path(__file__).resolve().parent / "golden"


def test_philox_known_answers():
    # Random123 kat_vectors for philox4x32_10 (Salmon et al., SC'11)
    assert O.philox([0, 0, 0, 0], [0, 0]) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert O.philox([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]
    assert O.philox([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0]) == \
        [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


def test_bed_decode_matches_reference_code_table():
    # src/preprocessgraph.cpp:43-56: allele1 = !b[k], allele2 = !b[k+1]; (0,1) missing
    # single bytes with all four codes 0,1,2,3 in the four slots
    bed = np.array([[0b11100100]], np.uint8)
    assert O.decode(bed, 4).tolist() == [[2, -1, 1, 0]]
    # ragged: ones at code 2, twos at code 0, missing at code 1 (src/raggedsparsemarkerbuilder.cpp:34-40)
    (o1, i1), (o2, i2), (om, im) = O.ragged_lists(bed, 4)
    assert i1.tolist() == [2] and i2.tolist() == [0] and im.tolist() == [1]


def test_trailing_padding_is_ignored():
    g = np.array([[0, 1, 2, 0, 1]], np.int8)
    bed = plink.encode_bed(g)
    bed[0, -1] |= 0b10101000   # garbage in the unused fields of the last byte
    assert O.decode(bed, 5).tolist() == g.tolist()
    assert O.counts(bed, 5).tolist() == [[2, 2, 1, 0]]


@pytest.mark.parametrize("N,M,miss", [(7, 5, 0.0), (64, 30, 0.1), (203, 41, 0.03), (1000, 20, 0.0)])
def test_dense_standardisation_invariants(N, M, miss):
    g, _ = plink.synth_genotypes(N, M, seed=N + M, missing=miss)
    bed = plink.encode_bed(g)
    x = O.dense_columns(bed, N)
    # centred columns with squared norm N-1 (src/densemarkerbuilder.cpp:56-59)
    np.testing.assert_allclose(x.sum(1), 0.0, atol=1e-9 * N)
    np.testing.assert_allclose((x * x).sum(1), N - 1.0, rtol=1e-12)
    np.testing.assert_allclose(x, plink.standardize_dense(g), rtol=1e-12, atol=1e-12)


def test_ragged_stats_formula():
    g, _ = plink.synth_genotypes(301, 17, seed=4, missing=0.05)
    bed = plink.encode_bed(g)
    rc, st = O.ragged_stats(bed, 301)
    assert rc == 0
    gz = np.where(g < 0, 0, g).astype(float)
    mean = gz.sum(1) / 301
    sd = np.sqrt(((gz ** 2).sum(1) - 2 * mean * gz.sum(1) + 301 * mean ** 2) / 300)
    np.testing.assert_allclose(st[:, 0], mean, rtol=1e-15)
    np.testing.assert_allclose(st[:, 1], sd, rtol=1e-14)
    np.testing.assert_array_equal(st[:, 3], gz.sum(1))


def test_sparse_update_identity_of_reference_unit_test():
    # test/eigenSparseTest.cpp:69-81: with no missing genotypes, the ragged
    # epsilon update dBeta*(Z - mean)/sd equals dBeta times the centred,
    # scaled column; the dense builder's column equals it exactly in law.
    g, _ = plink.synth_genotypes(500, 6, seed=9)
    bed = plink.encode_bed(g)
    rc, st = O.ragged_stats(bed, 500)
    x = O.dense_columns(bed, 500)
    dbeta = 0.37
    for j in range(6):
        upd_sparse = dbeta * g[j] / st[j, 1] - dbeta * st[j, 0] / st[j, 1]
        np.testing.assert_allclose(upd_sparse, dbeta * x[j], rtol=1e-12, atol=1e-14)


def test_monomorphic_marker_rejected():
    g = np.zeros((2, 40), np.int8)
    g[1, 3] = 1
    bed = plink.encode_bed(g)
    assert O.marker_table_dense(bed, 40)[0] == -2
    assert O.ragged_stats(bed, 40)[0] == -2


def test_permutation_and_draws():
    p = O.permutation(3, 0, 7, 1000)
    assert sorted(p.tolist()) == list(range(1000))
    assert not np.array_equal(p, O.permutation(3, 0, 8, 1000))
    u, z = O.marker_draws(3, 0, 1, 20000)
    assert 0 < u.min() and u.max() < 1
    assert abs(u.mean() - 0.5) < 0.01 and abs(z.mean()) < 0.03 and abs(z.std() - 1) < 0.03


@pytest.mark.parametrize("shape", [0.3, 1.0, 2.5, 50.0, 5000.0])
def test_gamma_moments(shape):
    xs = np.array([O.gamma(1, 0, it, 5, 0, shape)[1] for it in range(4000)])
    assert abs(xs.mean() / shape - 1) < 0.1
    assert abs(xs.var() / shape - 1) < 0.25


def _uk10k():
    z = REF / "test.zip"
    if not z.exists():
        pytest.skip("reference fixtures not mounted")
    zf = zipfile.ZipFile(z)
    raw = np.frombuffer(zf.read("test/data/uk10k_chr1_1mb.bed"), np.uint8)
    snpres = zf.read("test/res/test.snpRes").decode().splitlines()
    return raw, snpres


def test_uk10k_decode_matches_reference_fixture_allele_frequencies():
    """BED decode + per-marker allele counting against the GeneFrq column the
    reference ships for its uk10k fixture (test.zip:test/res/test.snpRes,
    written by GCTB from the same .bed): frequency of the counted allele =
    (n1 + 2 n2) / (2 (N - nmissing)) agrees to the printed 6 decimals."""
    raw, snpres = _uk10k()
    N, M = 3642, 6717
    assert bytes(raw[:3]) == plink.BED_MAGIC
    bed = raw[3:].reshape(M, (N + 3) // 4)
    c = O.counts(bed, N)
    freq = (c[:, 1] + 2 * c[:, 2]) / (2.0 * (N - c[:, 3]))
    gf = np.array([float(line.split()[4]) for line in snpres[1:] if line.strip()])
    assert gf.size == M
    np.testing.assert_allclose(freq, gf, atol=1e-6)
    # the committed digest pins these counts for hosts without the fixture
    digest = np.load(GOLDEN / "uk10k_counts_digest.npz")
    np.testing.assert_array_equal(c.sum(0), digest["col_sums"])
    np.testing.assert_array_equal(c[:64], digest["head"])
