"""The pair-term corrections of the pair-resolved rounds, checked on the CPU.

For two markers p and t of a round, the kernels apply p's residual update and
move num_t by a formula in integer pair terms instead of recomputing x_t . eps.
This test replays the update exactly as the sweep applies it (ragged:
the listed residuals, the missing genotypes' compensation, the pending shift
and the running sum as in src/raggedbayesrkernel.cpp:10-35; dense: every
individual by its code's delta and the residual total) and compares the change
of num_t, formed as the sweep forms it, with the formula, in FP64 on random
data with and without missing genotypes.
"""
import numpy as np
import pytest

MISSING = -1


def genotypes(rng, n, miss):
    p = rng.uniform(0.05, 0.5)
    g = (rng.random(n) < p).astype(int) + (rng.random(n) < p).astype(int)
    g[rng.random(n) < miss] = MISSING
    if (g[g >= 0] == g[g >= 0][0]).all():
        g[0], g[1] = 0, 1
    return g


@pytest.mark.parametrize("miss", [0.0, 0.03])
@pytest.mark.parametrize("seed", range(5))
def test_ragged_pair_correction(seed, miss):
    rng = np.random.default_rng(seed)
    N = 300
    gp, gt = genotypes(rng, N, miss), genotypes(rng, N, miss)

    def stats(g):
        obs = g[g >= 0]
        mean = obs.mean()
        sd = np.sqrt(((obs - mean) ** 2).sum() / (obs.size - 1))
        return mean, 1.0 / sd, float(obs.sum())

    mp, ip, Zp = stats(gp)
    mt, it_, Zt = stats(gt)
    eps_s = rng.normal(size=N)          # stored residual
    shift = rng.normal() * 0.1          # pending uniform shift of the residual
    eps_sum = rng.normal() * 3.0        # running residual sum
    beta_t = rng.normal() * 0.01

    def num_t(eps_s, shift, eps_sum):
        t12 = (np.where(gt >= 0, np.maximum(gt, 0), 0) * eps_s).sum()
        return beta_t * (N - 1) - mt * eps_sum * it_ + (t12 + shift * Zt) * it_

    before = num_t(eps_s, shift, eps_sum)
    dbeta = rng.normal() * 0.05
    # p's update as the sweep applies it
    e2 = eps_s.copy()
    listed = gp > 0
    e2[listed] += dbeta * ip * gp[listed]
    e2[gp == MISSING] += dbeta * mp * ip
    shift2 = shift - dbeta * mp * ip
    sum2 = eps_sum + dbeta * ip * (Zp - mp * N)
    after = num_t(e2, shift2, sum2)
    # the pair terms and the formula
    gt0 = np.where(gt > 0, gt, 0)
    A = float((np.where(gp > 0, gp, 0) * gt0).sum())
    Bm = float(gt0[gp == MISSING].sum())
    corr = dbeta * ip * it_ * (A + mp * Bm - mt * (Zp - mp * N) - mp * Zt)
    np.testing.assert_allclose(after - before, corr, rtol=1e-9, atol=1e-12)


@pytest.mark.parametrize("miss", [0.0, 0.03])
@pytest.mark.parametrize("seed", range(5))
def test_dense_pair_correction(seed, miss):
    rng = np.random.default_rng(100 + seed)
    N = 300
    gp, gt = genotypes(rng, N, miss), genotypes(rng, N, miss)

    def consts(g):
        obs = g[g >= 0]
        cm = obs.mean()
        sigma = 1.0 / np.sqrt(((obs - cm) ** 2).sum() / (obs.size - 1))
        xm = rng.normal() * 1e-3          # value of a missing genotype (near zero)
        x = np.where(g >= 0, sigma * (np.maximum(g, 0) - cm), xm)
        return sigma, cm, xm, x

    sp, cp, xp, x_p = consts(gp)
    st, ct, xt, _ = consts(gt)
    eps = rng.normal(size=N)
    beta_t = rng.normal() * 0.01

    def num_t(eps):
        tot = (np.where(gt >= 0, np.maximum(gt, 0), 0) * eps).sum()
        sm = eps[gt == MISSING].sum()
        return (st * (tot - ct * (eps.sum() - sm)) + xt * sm) + beta_t * (N - 1)

    before = num_t(eps)
    dbeta = rng.normal() * 0.05
    after = num_t(eps + dbeta * x_p)
    g_p = np.where(gp > 0, gp, 0).astype(float)
    g_t = np.where(gt > 0, gt, 0).astype(float)
    mp_, mt_ = gp == MISSING, gt == MISSING
    P = (g_p * g_t).sum()
    MM = float((mp_ & mt_).sum())
    Gmp = g_t[mp_].sum()                # g_t over the individuals missing at p
    Gmt = g_p[mt_].sum()                # g_p over the individuals missing at t
    S_t, nmiss_t = g_t.sum(), float(mt_.sum())
    colsum_p = x_p.sum()
    dT = sp * (P - cp * (S_t - Gmp)) + xp * Gmp
    dSm = sp * (Gmt - cp * (nmiss_t - MM)) + xp * MM
    corr = dbeta * (st * dT - st * ct * colsum_p + (st * ct + xt) * dSm)
    np.testing.assert_allclose(after - before, corr, rtol=1e-9, atol=1e-12)
