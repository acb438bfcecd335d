"""Posterior summaries of the chosen forms against the FP64 oracle.

The accuracy bar of the chosen forms is stated on what a user of the chain
keeps: the posterior means after burn-in of beta, sigmaG and sigmaE, and the
posterior frequency of each mixture component.  Bar: 1e-6 relative for the
means (absolute floor 1e-13 for betas that are almost always zero) and 1e-6
absolute for the component frequencies, which with a few hundred markers
means the components agree in every kept iteration.  Forms: the Gram-blocked
FP32C dense sweep (two groups), the FP32C restart sweep over ragged markers
with missing genotypes and an FP64 residual refresh every 5 sweeps, and the
batched tensor-core chains.
"""
import numpy as np
import pytest

import oracle_lib as O
from bayesrrcmd_gb300 import gpu, plink

pytestmark = pytest.mark.gpu
RTOL = 1e-6
S1 = [[0.01, 0.001, 0.0001]]
S2 = [[0.01, 0.001, 0.0001], [0.1, 0.01]]
KMAX = 4


class Posterior:
    """Running sums of the kept iterations of one chain."""

    def __init__(self, M, G):
        self.n = 0
        self.beta = np.zeros(M)
        self.sigmaG = np.zeros(G)
        self.sigmaE = 0.0
        self.freq = np.zeros(KMAX)

    def add(self, s):
        self.n += 1
        self.beta += s["beta"]
        self.sigmaG += s["sigmaG"]
        self.sigmaE += s["sigmaE"]
        self.freq += np.bincount(s["comp"], minlength=KMAX)[:KMAX] / len(s["comp"])

    def means(self):
        return dict(beta=self.beta / self.n, sigmaG=self.sigmaG / self.n, sigmaE=self.sigmaE / self.n,
                    freq=self.freq / self.n)


def assert_posteriors_agree(p, q, what):
    a, b = p.means(), q.means()
    assert p.n == q.n > 0
    np.testing.assert_allclose(a["beta"], b["beta"], rtol=RTOL, atol=1e-13, err_msg=f"{what}: beta")
    np.testing.assert_allclose(a["sigmaG"], b["sigmaG"], rtol=RTOL, err_msg=f"{what}: sigmaG")
    np.testing.assert_allclose(a["sigmaE"], b["sigmaE"], rtol=RTOL, err_msg=f"{what}: sigmaE")
    np.testing.assert_allclose(a["freq"], b["freq"], rtol=0, atol=1e-6, err_msg=f"{what}: component frequencies")
    assert np.count_nonzero(b["beta"]) > 0


def dataset(N, M, seed, miss=0.0, p_lo=0.05):
    g, _ = plink.synth_genotypes(N, M, seed, missing=miss, p_lo=p_lo)
    bed = plink.encode_bed(g)
    y, _, _ = plink.synth_phenotype(g, seed, max(1, M // 50), 0.5)
    return g, bed, y


@pytest.mark.parametrize("kind,miss,refresh,gram,pair_rounds", [
    (gpu.KIND_DENSE, 0.0, 50, 1, 0),      # Gram-blocked FP32C dense sweep
    (gpu.KIND_RAGGED, 0.01, 5, -1, -1),   # FP32C restart rounds, ragged markers, refresh every 5 sweeps
    (gpu.KIND_RAGGED, 0.01, 5, -1, 1),    # FP32C pair-resolved rounds, ragged markers
    (gpu.KIND_DENSE, 0.01, 5, -1, 1),     # FP32C pair-resolved rounds, dense markers
])
def test_fp32c_posterior_means_match_fp64_oracle(gpu_lib, kind, miss, refresh, gram, pair_rounds):
    N, M, iters, burn = 3000, 700, 40, 10
    _, bed, y = dataset(N, M, seed=131, miss=miss, p_lo=0.01)
    group = (np.arange(M) % 2).astype(np.int32)
    ch = gpu.Chain(gpu.ChainConfig(N=N, M=M, kind=kind, form=gpu.FORM_FP32C, S=S2, seed=17,
                                   refresh_every=refresh, gram=gram, pair_rounds=pair_rounds))
    ch.pack_bed(bed)
    ch.set_groups(group)
    ch.set_phenotype(y)
    ch.init()
    assert ch.gram_info()["blocked"] == (gram == 1)
    assert ch.round_info()["pair_rounds"] == (pair_rounds == 1)
    oc = O.OracleChain(bed, N, y, S2, kind=kind, group=group, seed=17)
    pg, po = Posterior(M, 2), Posterior(M, 2)
    for it in range(iters):
        ch.iterate(1)
        oc.iterate(it)
        if it >= burn:
            pg.add(ch.state())
            po.add(oc.state())
    ch.close()
    assert_posteriors_agree(pg, po, f"kind {kind}")


def test_batched_posterior_means_match_fp64_oracle(gpu_lib):
    N, M, C, iters, burn = 2000, 300, 32, 24, 4
    g, bed, _ = dataset(N, M, seed=141)
    ys = np.stack([plink.synth_phenotype(g, 141 * 100 + c, max(1, M // 40), 0.2 + 0.5 * c / C)[0]
                   for c in range(C)]).astype(np.float32)
    b = gpu.Batch(gpu.ChainConfig(N=N, M=M, S=S1, seed=23, chain=0), C)
    b.pack_bed(bed)
    b.set_phenotypes(ys)
    b.init()
    checked = (0, 13, 31)
    oracles = {c: O.OracleChain(bed, N, ys[c], S1, seed=23, chain=c, perm_chain=0) for c in checked}
    pg = {c: Posterior(M, 1) for c in checked}
    po = {c: Posterior(M, 1) for c in checked}
    for it in range(iters):
        b.iterate(1)
        for c, oc in oracles.items():
            oc.iterate(it)
            if it >= burn:
                pg[c].add(b.state(c))
                po[c].add(oc.state())
    b.close()
    for c in checked:
        assert_posteriors_agree(pg[c], po[c], f"chain {c}")
