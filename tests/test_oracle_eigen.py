"""The Eigen sparse kind of the oracle against a numpy restatement (CPU).

The reference's Eigen sparse marker (src/eigensparsemarkerbuilder.cpp:40-75)
stores Zg = 1, 2 at heterozygous / homozygous-minor genotypes and the marker
mean (sum over non-missing genotypes / N) at missing ones; sqrdZ, Zsum and the
sd include those imputed values.  Its kernel (src/eigenbayesrkernel.cpp:10-20,
src/sparsebayesrkernel.cpp:10-34) takes dot = Zg.eps / sd,
num = beta_old (N-1) - mean epsSum / sd + dot, and moves the residual by
dBeta Zg / sd - dBeta mean / sd, which leaves missing genotypes unchanged.
Here the oracle's sweep is replayed marker by marker from a dense imputed Zg
matrix: every marker's P(component 0) follows from num, and the residual and
running sum follow from the chosen betas.
"""
import numpy as np
import pytest

import oracle_lib as O
from bayesrrcmd_gb300 import plink

EIGEN = 2
S1 = [[0.01, 0.001, 0.0001]]


def imputed(g):
    gz = np.where(g < 0, 0, g).astype(float)
    N = g.shape[1]
    mean = gz.sum(1) / N
    Zg = np.where(g < 0, mean[:, None], gz)
    return Zg, mean


def test_eigen_stats_formula():
    g, _ = plink.synth_genotypes(301, 17, seed=4, missing=0.05)
    g[0] = np.where(g[0] < 0, 1, g[0])   # one marker without missing genotypes
    bed = plink.encode_bed(g)
    rc, st = O.eigen_stats(bed, 301)
    assert rc == 0
    Zg, mean = imputed(g)
    nm = (g < 0).sum(1)
    assert nm.sum() > 0
    sqrdZ = (Zg ** 2).sum(1)
    Zsum = Zg.sum(1)
    sd = np.sqrt((sqrdZ - 2 * mean * Zsum + 301 * mean ** 2) / 300)
    np.testing.assert_allclose(st[:, 0], mean, rtol=1e-15)
    np.testing.assert_allclose(st[:, 2], sqrdZ, rtol=1e-14)
    np.testing.assert_allclose(st[:, 3], Zsum, rtol=1e-14)
    np.testing.assert_allclose(st[:, 1], sd, rtol=1e-13)
    # the sd is the root mean square of Zg about the mean of the non-imputed
    # genotypes (Zsum / N is not that mean once missing values are imputed)
    np.testing.assert_allclose(st[:, 1], np.sqrt(((Zg - mean[:, None]) ** 2).sum(1) / 300), rtol=1e-12)
    # without missing genotypes the Eigen and ragged statistics coincide
    rc_r, st_r = O.ragged_stats(bed, 301)
    same = nm == 0
    assert same[0] and not same.all()
    np.testing.assert_array_equal(st[same], st_r[same])


def test_eigen_monomorphic_marker_rejected():
    g = np.zeros((2, 40), np.int8)
    g[1, 3] = 1
    g[0, 5] = -1   # zeros and a missing genotype: mean 0, sd 0
    bed = plink.encode_bed(g)
    assert O.eigen_stats(bed, 40)[0] == -2


def acum_of(num, sigmaE, sigmaG, pi, S, N):
    """P(component 0) of src/BayesRBase.cpp:316-339 for a given num."""
    K = len(S) + 1
    cVa = np.array([0.0] + list(S))
    denom = (N - 1) + sigmaE / sigmaG / cVa[1:]
    muk = np.concatenate([[0.0], num / denom])
    scale = sigmaG / sigmaE * (N - 1)
    logL = np.log(pi[:K]).copy()
    logL[1:] = logL[1:] - 0.5 * np.log(scale * cVa[1:] + 1.0) + 0.5 * muk[1:] * num / sigmaE
    if np.any(np.abs(logL[1:] - logL[0]) > 700):
        return 0.0
    return 1.0 / np.exp(logL - logL[0]).sum()


@pytest.mark.parametrize("N,M,miss", [(157, 40, 0.05), (90, 25, 0.2)])
def test_eigen_sweep_replayed_from_imputed_columns(N, M, miss):
    g, _ = plink.synth_genotypes(N, M, seed=N + M, missing=miss)
    bed = plink.encode_bed(g)
    y, _, _ = plink.synth_phenotype(g, 3, 5, 0.6)
    oc = O.OracleChain(bed, N, y, S1, kind=EIGEN, seed=11)
    for it in range(2):
        oc.iterate(it)
    s0 = oc.state()
    order = O.permutation(11, 0, 50, M)
    u, z = O.marker_draws(11, 0, 50, M)
    oc.sweep(order, u, z)
    s1 = oc.state()

    _, st = O.eigen_stats(bed, N)
    Zg, mean = imputed(g)
    sd = st[:, 1]
    eps = s0["eps"].copy()
    epsSum = s0["epsSum"]
    # epsSum tracks the residual total for Eigen markers (Zsum includes the imputed values)
    np.testing.assert_allclose(epsSum, eps.sum(), rtol=0, atol=1e-9)
    pi = s0["pi"][0]
    changed = 0
    for j in order:
        b_old = s0["beta"][j]
        num = b_old * (N - 1) - mean[j] * epsSum / sd[j] + Zg[j] @ eps / sd[j]
        a0 = acum_of(num, s0["sigmaE"], s0["sigmaG"][0], pi, S1[0], N)
        np.testing.assert_allclose(s1["acum"][j], a0, rtol=1e-9, atol=1e-15, err_msg=f"marker {j}")
        dB = b_old - s1["beta"][j]
        if dB != 0.0:
            changed += 1
            upd = dB * Zg[j] / sd[j] - dB * mean[j] / sd[j]
            assert np.all(upd[g[j] < 0] == 0.0)
            eps += upd
            epsSum += dB * st[j, 3] / sd[j] - dB * mean[j] * N / sd[j]
    assert changed > 0
    np.testing.assert_allclose(s1["eps"], eps, rtol=0, atol=1e-12)
    np.testing.assert_allclose(s1["epsSum"], epsSum, rtol=0, atol=1e-10)


def test_eigen_chain_equals_ragged_without_missing():
    """test/eigenSparseTest.cpp:69-81: with no missing genotypes the Eigen
    update is the centred, scaled column, as for the ragged marker."""
    N, M = 200, 30
    g, _ = plink.synth_genotypes(N, M, seed=8, missing=0.0)
    bed = plink.encode_bed(g)
    y, _, _ = plink.synth_phenotype(g, 8, 4, 0.5)
    e = O.OracleChain(bed, N, y, S1, kind=EIGEN, seed=2)
    r = O.OracleChain(bed, N, y, S1, kind=1, seed=2)
    for it in range(3):
        e.iterate(it)
        r.iterate(it)
        se, sr = e.state(), r.state()
        np.testing.assert_array_equal(se["comp"], sr["comp"])
        np.testing.assert_allclose(se["beta"], sr["beta"], rtol=1e-11, atol=1e-15)
        np.testing.assert_allclose(se["eps"], sr["eps"], rtol=0, atol=1e-11)
