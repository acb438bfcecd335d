"""A second restatement of the reference sampler, in numpy, against the oracle.

The oracle (oracle/oracle.c) is the checker of every GPU kernel, so it is
itself checked here against an independent restatement written from the
reference sources: one sweep of BayesRBase::processColumn
(src/BayesRBase.cpp:287-392) over dense markers (DenseRKernel,
src/densebayesrkernel.cpp:10-20, on the columns of the DenseMarkerBuilder
standardisation) and over ragged markers (SparseBayesRKernel and
RaggedBayesRKernel, src/sparsebayesrkernel.cpp:10-34,
src/raggedbayesrkernel.cpp:10-35, statistics of src/sparsemarker.cpp:8-19 and
src/raggedsparsemarkerbuilder.cpp:45-55, running epsilon sum of
src/SparseBayesRRG.cpp:76-92) and over Eigen sparse markers
(src/eigenbayesrkernel.cpp:10-20, src/eigensparsemarkerbuilder.cpp:40-56), replayed marker by marker in the oracle's sweep
order with its draws u, z and its state before the sweep.  Checked:
P(component 0) of every marker, every component and beta, the residual and
the epsilon sum after the sweep, and the sweep statistics v (component counts
per group) and betasqnG.  A second test replays whole iterations of the
runGibbs loop body (updateMu, the sweep, the sigmaE, sigmaG and pi draws) from
the same stream variates.  Only the order of floating-point sums differs
between the two, so components must agree exactly and values to 1e-10.
"""
import numpy as np
import pytest

import oracle_lib as O
from bayesrrcmd_gb300 import plink

S2 = [[0.01, 0.001, 0.0001], [0.1, 0.01]]


def process_column(num, beta_old, u, z, sigmaE, sigmaG, pi, S, N):
    """The per-marker sampler of src/BayesRBase.cpp:306-364 for a given num:
    returns P(component 0), the component (None when the walk ends without
    one, which leaves beta unchanged) and the new beta."""
    K = len(S) + 1
    cva = np.asarray(S, np.float64)
    denom = (N - 1.0) + (sigmaE / sigmaG) * (1.0 / cva)
    muk = np.concatenate([[0.0], num / denom])
    scale = sigmaG / sigmaE * (N - 1.0)
    logL = np.log(np.asarray(pi[:K], np.float64))
    logL[1:] = logL[1:] - 0.5 * np.log(scale * cva + 1.0) + 0.5 * (muk[1:] * num) / sigmaE

    def prob(k):
        if np.any(np.abs(logL[1:] - logL[k]) > 700):
            return 0.0
        return 1.0 / np.exp(logL - logL[k]).sum()

    acum = prob(0)
    a0 = acum
    for k in range(K):
        if u <= acum:
            beta = 0.0 if k == 0 else z * np.sqrt(sigmaE / denom[k - 1]) + muk[k]
            return a0, k, beta
        if k + 1 < K:
            acum += prob(k + 1)
    return a0, None, beta_old


def ragged_statistics(g):
    """mean over all N (missing included), sd, Zsum of the ragged marker."""
    N = g.shape[1]
    val = np.where(g > 0, g, 0).astype(np.float64)
    zsum = val.sum(1)
    sqrdz = (val * val).sum(1)
    mean = zsum / N
    sd = np.sqrt((sqrdz - 2.0 * mean * zsum + N * mean * mean) / (N - 1.0))
    return mean, sd, zsum


def eigen_statistics(g):
    """The Eigen sparse marker (src/eigensparsemarkerbuilder.cpp:40-56): Zg with
    missing genotypes imputed at mean = (sum over non-missing) / N; sqrdZ,
    Zsum and sd include the imputed values."""
    N = g.shape[1]
    val = np.where(g > 0, g, 0).astype(np.float64)
    mean = val.sum(1) / N
    zg = np.where(g < 0, mean[:, None], val)
    zsum = zg.sum(1)
    sqrdz = (zg * zg).sum(1)
    sd = np.sqrt((sqrdz - 2.0 * mean * zsum + N * mean * mean) / (N - 1.0))
    return zg, mean, sd, zsum


def sweep_once(kind, N, M, miss, seed, strong=False):
    g, _ = plink.synth_genotypes(N, M, seed=seed, missing=miss)
    bed = plink.encode_bed(g)
    if strong:
        # one marker carries almost all of the variance: sigmaE becomes small,
        # its num large, and the 700 guards of the log-likelihoods fire
        x0 = plink.standardize_dense(g[:1])[0]
        y = (3.0 * x0 + np.random.default_rng(seed).normal(0.0, 0.05, N)).astype(np.float32)
    else:
        y, _, _ = plink.synth_phenotype(g, seed, max(2, M // 8), 0.6)
    group = (np.arange(M) % 2).astype(np.int32)
    oc = O.OracleChain(bed, N, y, S2, kind=kind, group=group, seed=seed)
    # the strong marker's guards fire while sigmaE is small, in the first iterations
    for it in range(1 if strong else 3):
        oc.iterate(it)
    s0 = oc.state()
    order = O.permutation(seed, 0, 77, M)
    u, z = O.marker_draws(seed, 0, 77, M)
    oc.sweep(order, u, z)
    return g, group, s0, order, u, z, oc.state()


def replay(kind, g, group, s0, order, u, z, S=S2, async_batch=0):
    """One sweep.  async_batch T > 0 replays the asyncppbayes schedule: the
    markers of each batch of T consecutive positions all read the residual and
    its running sum before any of them writes (processColumnAsync then
    updateGlobal, src/BayesRBase.cpp:394-524, src/SparseBayesRRG.cpp:94-102),
    and acum is left as it was (processColumnAsync never writes m_acum)."""
    M, N = g.shape
    beta, comp, acum = s0["beta"].copy(), s0["comp"].copy(), s0["acum"].copy()
    eps, eps_sum = s0["eps"].copy(), s0["epsSum"]
    v = np.zeros((len(S), 4))
    bsq = np.zeros(len(S))
    if kind == 0:
        x = plink.standardize_dense(g)
    elif kind == 1:
        mean, sd, zsum = ragged_statistics(g)
        ones, twos, missing = g == 1, g == 2, g < 0
    else:
        zg, mean, sd, zsum = eigen_statistics(g)

    def pick(j):
        gr = group[j]
        b_old = beta[j]
        if kind == 0:
            num = x[j] @ eps + b_old * (N - 1.0)
        elif kind == 1:
            num = b_old * (N - 1.0) - mean[j] * eps_sum / sd[j] + (eps[ones[j]].sum() + 2.0 * eps[twos[j]].sum()) / sd[j]
        else:
            num = b_old * (N - 1.0) - mean[j] * eps_sum / sd[j] + zg[j] @ eps / sd[j]
        a0, k, b_new = process_column(num, b_old, u[j], z[j], s0["sigmaE"], s0["sigmaG"][gr], s0["pi"][gr], S[gr], N)
        if async_batch <= 0:
            acum[j] = a0
        if k is not None:
            beta[j] = b_new
            comp[j] = k
            v[gr, k] += 1.0
            if k > 0:
                bsq[gr] += b_new * b_new
        return b_old, beta[j]

    def update(j, b_old, b_new):
        nonlocal eps, eps_sum
        if b_old == 0.0 and b_new == 0.0:
            return
        d = b_old - b_new
        if kind == 0:
            eps += d * x[j]
        elif kind == 2:
            eps_sum += d * zsum[j] / sd[j] - d * mean[j] * N / sd[j]
            eps += d * zg[j] / sd[j] - d * mean[j] / sd[j]
        else:
            eps_sum += d * zsum[j] / sd[j] - d * mean[j] * N / sd[j]
            adj = d * mean[j] / sd[j]
            delta = np.full(N, -adj)
            delta[ones[j]] += d / sd[j]
            delta[twos[j]] += 2.0 * d / sd[j]
            delta[missing[j]] += adj
            eps += delta

    if async_batch <= 0:
        for j in order:
            update(j, *pick(j))
    else:
        for q0 in range(0, len(order), async_batch):
            batch = order[q0:q0 + async_batch]
            picks = [pick(j) for j in batch]
            for j, (b_old, b_new) in zip(batch, picks):
                update(j, b_old, b_new)
    return dict(beta=beta, comp=comp, acum=acum, eps=eps, epsSum=eps_sum, v=v, betasqnG=bsq)


@pytest.mark.parametrize("kind,N,M,miss,seed,strong", [
    (0, 640, 160, 0.0, 21, False),
    (0, 333, 120, 0.02, 22, False),
    (1, 640, 160, 0.0, 23, False),
    (1, 501, 140, 0.03, 24, False),
    (0, 640, 60, 0.0, 25, True),
    (1, 640, 60, 0.02, 26, True),
    (2, 501, 140, 0.03, 27, False),
    (2, 640, 60, 0.02, 28, True),
])
def test_oracle_sweep_equals_numpy_restatement(kind, N, M, miss, seed, strong):
    g, group, s0, order, u, z, s1 = sweep_once(kind, N, M, miss, seed, strong)
    r = replay(kind, g, group, s0, order, u, z)
    np.testing.assert_array_equal(s1["comp"], r["comp"])
    np.testing.assert_array_equal(s1["beta"] != 0, r["beta"] != 0)
    np.testing.assert_allclose(s1["beta"], r["beta"], rtol=1e-10, atol=1e-14)
    np.testing.assert_allclose(s1["acum"], r["acum"], rtol=1e-10, atol=1e-15)
    np.testing.assert_allclose(s1["eps"], r["eps"], rtol=0, atol=1e-10)
    np.testing.assert_array_equal(s1["v"][:, :4], r["v"])
    np.testing.assert_allclose(s1["betasqnG"], r["betasqnG"], rtol=1e-10)
    if kind != 0:
        np.testing.assert_allclose(s1["epsSum"], r["epsSum"], rtol=0, atol=1e-9)
    # the sweep moved the chain: some markers changed component
    assert np.count_nonzero(s1["comp"] != s0["comp"]) > 0
    if strong:
        # the guards fired: P(component 0) is exactly zero for the strong marker
        assert s1["acum"][0] == 0.0


@pytest.mark.parametrize("kind,miss,T,seed", [
    (0, 0.0, 20, 31), (0, 0.02, 7, 32), (1, 0.03, 20, 33), (1, 0.0, 64, 34), (2, 0.03, 13, 35),
])
def test_oracle_async_sweep_equals_numpy_restatement(kind, miss, T, seed):
    """The asyncppbayes schedule (batches of T markers in flight) of the oracle
    against the numpy restatement, over a chain that has run two asynchronous
    iterations first."""
    N, M = 540, 150
    g, _ = plink.synth_genotypes(N, M, seed=seed, missing=miss)
    bed = plink.encode_bed(g)
    y, _, _ = plink.synth_phenotype(g, seed, M // 8, 0.6)
    group = (np.arange(M) % 2).astype(np.int32)
    oc = O.OracleChain(bed, N, y, S2, kind=kind, group=group, seed=seed, async_batch=T)
    for it in range(2):
        oc.iterate(it)
    s0 = oc.state()
    order = O.permutation(seed, 0, 77, M)
    u, z = O.marker_draws(seed, 0, 77, M)
    oc.sweep(order, u, z)
    s1 = oc.state()
    r = replay(kind, g, group, s0, order, u, z, async_batch=T)
    np.testing.assert_array_equal(s1["comp"], r["comp"])
    np.testing.assert_allclose(s1["beta"], r["beta"], rtol=1e-10, atol=1e-14)
    np.testing.assert_array_equal(s1["acum"], s0["acum"])
    np.testing.assert_allclose(s1["eps"], r["eps"], rtol=0, atol=1e-10)
    np.testing.assert_array_equal(s1["v"][:, :4], r["v"])
    np.testing.assert_allclose(s1["betasqnG"], r["betasqnG"], rtol=1e-10)
    if kind != 0:
        np.testing.assert_allclose(s1["epsSum"], r["epsSum"], rtol=0, atol=1e-9)
    assert np.count_nonzero(s1["comp"] != s0["comp"]) > 0
    # the schedule differs from the synchronous sweep
    sync = replay(kind, g, group, s0, order, u, z)
    assert not np.allclose(sync["eps"], r["eps"], rtol=0, atol=1e-12)


def test_oracle_async_batch_of_one_is_the_synchronous_chain():
    """One marker in flight is the sequential chain (acum aside, which the
    asynchronous path never writes)."""
    N, M = 400, 90
    g, _ = plink.synth_genotypes(N, M, seed=5, missing=0.01)
    bed = plink.encode_bed(g)
    y, _, _ = plink.synth_phenotype(g, 5, 10, 0.5)
    for kind in (0, 1, 2):
        a = O.OracleChain(bed, N, y, S2, kind=kind, group=(np.arange(M) % 2).astype(np.int32), seed=3)
        b = O.OracleChain(bed, N, y, S2, kind=kind, group=(np.arange(M) % 2).astype(np.int32), seed=3,
                          async_batch=1)
        for it in range(3):
            a.iterate(it)
            b.iterate(it)
            sa, sb = a.state(), b.state()
            for k in ("beta", "comp", "eps", "sigmaG"):
                np.testing.assert_array_equal(sa[k], sb[k])
            assert sa["sigmaE"] == sb["sigmaE"] and sa["mu"] == sb["mu"]
        assert (sb["acum"] == 0).all() and (sa["acum"] != 0).any()


# Two groups with the same number of components, as the reference's K x groups
# matrices of mixture variances and counts require (src/BayesRBase.cpp:200).
S_EQ = [[0.01, 0.001, 0.0001], [0.1, 0.01, 0.001]]
PRIOR = 1e-4   # v0E = s02E = v0G = s02G, the reference's defaults (src/options.hpp:86-89)
P_MU, P_SIGMAE, P_SIGMAG, P_PI = 2, 5, 6, 7   # stream purposes of the scalar draws


def u53(a, b):
    return ((a >> 5) * 67108864.0 + (b >> 6) + 0.5) / 9007199254740992.0


def std_gamma(seed, chain, it, purpose, sub, shape):
    rc, x = O.gamma(seed, chain, it, purpose, sub, shape)
    assert rc == 0
    return x


def inv_scaled_chisq(seed, chain, it, purpose, sub, dof, scale):
    """src/distributions_boost.cpp:45-60: 1 / Gamma(dof/2, scale 1/(dof*scale/2))."""
    return 1.0 / (std_gamma(seed, chain, it, purpose, sub, 0.5 * dof) / (0.5 * dof * scale))


def iterate_numpy(kind, g, group, s, seed, chain, it):
    """One pass of the runGibbs loop body (src/BayesRBase.cpp:186-247):
    updateMu (dense src/DenseBayesRRmz.cpp:36-42, sparse
    src/SparseBayesRRG.cpp:106-113), the sweep, sigmaE, then per group sigmaG
    and the Dirichlet draw of pi."""
    M, N = g.shape
    eps = s["eps"] + s["mu"]
    eps_sum = s["epsSum"]
    if kind == 0:
        mean = eps.sum() / N
    else:
        eps_sum = eps_sum + s["mu"] * N
        mean = eps_sum / N
    b = O.philox([0, it, P_MU, 0], [seed, chain])
    zmu = np.sqrt(-2.0 * np.log(u53(b[0], b[1]))) * np.cos(2.0 * np.pi * u53(b[2], b[3]))
    mu = mean + np.sqrt(s["sigmaE"] / N) * zmu
    eps = eps - mu
    if kind != 0:
        eps_sum -= mu * N
    order = O.permutation(seed, chain, it, M)
    u, z = O.marker_draws(seed, chain, it, M)
    r = replay(kind, g, group, dict(s, eps=eps, epsSum=eps_sum, mu=mu), order, u, z, S_EQ)
    dof = PRIOR + N
    sigmaE = inv_scaled_chisq(seed, chain, it, P_SIGMAE, 0, dof, ((r["eps"] ** 2).sum() + PRIOR * PRIOR) / dof)
    sigmaG = np.zeros(len(S_EQ))
    pi = np.zeros((len(S_EQ), 4))
    for gr in range(len(S_EQ)):
        v = r["v"][gr]
        m0 = v.sum() - v[0]
        sigmaG[gr] = inv_scaled_chisq(seed, chain, it, P_SIGMAG, gr, PRIOR + m0,
                                      (r["betasqnG"][gr] * m0 + PRIOR * PRIOR) / (PRIOR + m0))
        d = np.array([std_gamma(seed, chain, it, P_PI, gr * 256 + k, v[k] + 1.0) for k in range(4)])
        pi[gr] = d / d.sum()
    return dict(r, mu=mu, sigmaE=sigmaE, sigmaG=sigmaG, pi=pi)


@pytest.mark.parametrize("kind,miss,seed", [(0, 0.0, 31), (0, 0.02, 32), (1, 0.0, 33), (1, 0.03, 34), (2, 0.03, 35)])
def test_oracle_iteration_equals_numpy_restatement(kind, miss, seed):
    N, M = 480, 140
    g, _ = plink.synth_genotypes(N, M, seed=seed, missing=miss)
    bed = plink.encode_bed(g)
    y, _, _ = plink.synth_phenotype(g, seed, 12, 0.5)
    group = (np.arange(M) % 2).astype(np.int32)
    oc = O.OracleChain(bed, N, y, S_EQ, kind=kind, group=group, seed=seed, chain=3)
    for it in range(2):
        oc.iterate(it)
    for it in range(2, 5):
        s = oc.state()
        r = iterate_numpy(kind, g, group, s, seed, 3, it)
        oc.iterate(it)
        o = oc.state()
        np.testing.assert_array_equal(o["comp"], r["comp"], err_msg=f"iteration {it}")
        np.testing.assert_allclose(o["beta"], r["beta"], rtol=1e-10, atol=1e-14)
        np.testing.assert_allclose(o["eps"], r["eps"], rtol=0, atol=1e-10)
        np.testing.assert_allclose(o["mu"], r["mu"], rtol=1e-10, atol=1e-13)
        np.testing.assert_allclose(o["sigmaE"], r["sigmaE"], rtol=1e-10)
        np.testing.assert_allclose(o["sigmaG"], r["sigmaG"], rtol=1e-10)
        np.testing.assert_allclose(o["pi"][:, :4], r["pi"], rtol=1e-10)
        if kind != 0:
            np.testing.assert_allclose(o["epsSum"], r["epsSum"], rtol=0, atol=1e-9)
