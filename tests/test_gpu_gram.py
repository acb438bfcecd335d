"""The marker Gram of the blocked FP32C sweep against a direct FP64
evaluation, through the C ABI.

G[j,k] = x_j . x_k with x_j(i) = sigma_j (g_j(i) - colmean_j) for a genotype
that is present and 0 for a missing one (the dense table's value of each code).
The build forms the integer sums P, Q, R with FP4, FP8 or BF16 GEMMs (the first
the library has algorithms for) whose products and partial sums are integers
below 2^24, so they are exact; a unit
error in any of them moves G by sigma_j sigma_k >= 2, far above the bar
(absolute 1e-8, against entries up to N).  Cases: N = 100,000 with markers of
allele frequency 0.6-0.99 (P up to 4N), N = 100,000 with 1 % missing genotypes
(all four sums), and M = 8,300 (two tiles of 8,192 markers, a last tile of 108).
"""
import numpy as np
import pytest

from bayesrrcmd_gb300 import gpu, plink

pytestmark = pytest.mark.gpu


def chain_with_gram(g):
    M, N = g.shape
    bed = plink.encode_bed(g)
    ch = gpu.Chain(gpu.ChainConfig(N=N, M=M, form=gpu.FORM_FP32C, gram=1, seed=1))
    ch.pack_bed(bed)
    y = np.linspace(-1.0, 1.0, N).astype(np.float32)
    ch.set_phenotype(y)
    ch.init()
    info = ch.gram_info()
    assert info["blocked"] and info["operand_bits"] in (4, 8, 16)
    return ch


def standardised(g, table):
    code = np.select([g == 2, g == 1, g == 0], [0, 2, 3], 1)
    x = np.take_along_axis(table, code, axis=1)
    x[code == 1] = 0.0
    return x


@pytest.mark.parametrize("N,M,miss,p", [(100_000, 300, 0.0, (0.6, 0.99)), (100_000, 300, 0.01, (0.01, 0.5))])
def test_gram_entries_match_direct_products(gpu_lib, N, M, miss, p):
    g, _ = plink.synth_genotypes(N, M, seed=N + M, missing=miss, p_lo=p[0], p_hi=p[1])
    ch = chain_with_gram(g)
    t, _ = ch.marker_table()
    x = standardised(g, t)
    j, k = np.tril_indices(M, -1)
    ref = (x @ x.T)[j, k]
    got = ch.gram_entries(j, k)
    np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-8)
    ch.close()


def test_gram_entries_across_tiles(gpu_lib):
    N, M = 2003, 8300
    g, _ = plink.synth_genotypes(N, M, seed=7, missing=0.01)
    ch = chain_with_gram(g)
    t, _ = ch.marker_table()
    x = standardised(g, t)
    rng = np.random.default_rng(3)
    j = rng.integers(1, M, 3000)
    k = (rng.random(3000) * j).astype(np.int64)
    # entries on both sides of the tile edge at 8,192 and in the last, partial tile
    j = np.concatenate([j, [8192, 8192, 8299, 8299, 8200, 8191]])
    k = np.concatenate([k, [8191, 0, 8298, 8192, 8191, 8190]])
    ref = np.einsum("ij,ij->i", x[j], x[k])
    got = ch.gram_entries(j, k)
    np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-9)
    ch.close()
