"""Batched chains (tensor-core form) vs the oracle, chain by chain.

Every chain c of a batch is the oracle's chain with seed `seed`, chain id
cfg.chain + c, its own phenotype, and the sweep order of chain cfg.chain's
stream (the batch shares one order per iteration).  The batched residual is
exact fixed point (eps * 2^40): the chains differ from the FP64 oracle by the
rounding of the fixed-point update coefficients, so beta (with an absolute
floor of 1e-13 for betas near zero), sigmaE and sigmaG are compared at 1e-9
relative, components exactly, the residual at 1e-10 absolute, acum
(P(component 0), evaluated with FP32 exponentials) at 2e-6 relative.  The constant
part of each update is rounded once and applied to every individual, which
moves the residual mean coherently by up to 2^-41 per update: mu, a mean
plus a draw, gets an absolute bar of 1e-10.
"""
import numpy as np
import pytest

import oracle_lib as O
from bayesrrcmd_gb300 import gpu, plink

pytestmark = pytest.mark.gpu
RTOL = 1e-9
S1 = [[0.01, 0.001, 0.0001]]
S2 = [[0.01, 0.001, 0.0001], [0.1, 0.01]]


def problem(N, M, C, seed):
    g, _ = plink.synth_genotypes(N, M, seed, missing=0.0, p_lo=0.05)
    bed = plink.encode_bed(g)
    ys = np.stack([plink.synth_phenotype(g, seed * 100 + c, max(1, M // 40), 0.3 + 0.4 * (c % 5) / 4)[0]
                   for c in range(C)]).astype(np.float32)
    return bed, ys


def make_batch(bed, N, ys, S, C, seed, chain0=0, group=None, **kw):
    b = gpu.Batch(gpu.ChainConfig(N=N, M=bed.shape[0], S=S, seed=seed, chain=chain0, **kw), C)
    b.pack_bed(bed)
    if group is not None:
        b.set_groups(group)
    b.set_phenotypes(ys)
    b.init()
    return b


def compare(s, o, what):
    np.testing.assert_array_equal(s["comp"], o["comp"], err_msg=what)
    nz = o["beta"] != 0
    np.testing.assert_array_equal(s["beta"] != 0, nz, err_msg=what)
    np.testing.assert_allclose(s["beta"][nz], o["beta"][nz], rtol=RTOL, atol=1e-13, err_msg=what)
    np.testing.assert_allclose(s["acum"], o["acum"], rtol=2e-6, atol=1e-12, err_msg=what)
    np.testing.assert_allclose(s["sigmaE"], o["sigmaE"], rtol=RTOL, err_msg=what)
    np.testing.assert_allclose(s["sigmaG"], o["sigmaG"], rtol=RTOL, err_msg=what)
    np.testing.assert_allclose(s["mu"], o["mu"], rtol=RTOL, atol=1e-10, err_msg=what)
    np.testing.assert_allclose(s["eps"], o["eps"], rtol=0, atol=1e-10, err_msg=what)


@pytest.mark.parametrize("N,M,C,chains_checked", [
    (2000, 300, 32, range(32)),        # 125 slices of 16 individuals
    (600, 157, 64, range(0, 64, 3)),   # fewer CTAs than chains; last block partial
    (5003, 96, 64, [0, 1, 17, 63]),    # 152 slices, ragged last slice
])
def test_batch_matches_oracle_each_iteration(gpu_lib, N, M, C, chains_checked):
    bed, ys = problem(N, M, C, seed=N % 97 + M)
    b = make_batch(bed, N, ys, S1, C, seed=5, chain0=10)
    oracles = {c: O.OracleChain(bed, N, ys[c], S1, seed=5, chain=10 + c, perm_chain=10) for c in chains_checked}
    for it in range(3):
        b.iterate(1)
        for c, oc in oracles.items():
            oc.iterate(it)
            compare(b.state(c), oc.state(), f"iteration {it} chain {c}")


@pytest.mark.parametrize("N,C,grid,chains_checked", [
    (3200, 32, 8, [0, 5, 31]),     # 400 individuals per slice: four update tiles in one TMEM pass
    (4800, 64, 16, [0, 33, 63]),   # 300 per slice: three tiles, the last split by chains
])
def test_batch_update_tiles_of_large_slices(gpu_lib, N, C, grid, chains_checked):
    M = 96
    bed, ys = problem(N, M, C, seed=N % 89 + C)
    b = make_batch(bed, N, ys, S1, C, seed=7, chain0=3, grid=grid)
    oracles = {c: O.OracleChain(bed, N, ys[c], S1, seed=7, chain=3 + c, perm_chain=3) for c in chains_checked}
    for it in range(3):
        b.iterate(1)
        for c, oc in oracles.items():
            oc.iterate(it)
            compare(b.state(c), oc.state(), f"iteration {it} chain {c}")


def test_batch_two_groups(gpu_lib):
    N, M, C = 1500, 200, 32
    bed, ys = problem(N, M, C, seed=3)
    group = (np.arange(M) % 2).astype(np.int32)
    b = make_batch(bed, N, ys, S2, C, seed=8, group=group)
    oracles = {c: O.OracleChain(bed, N, ys[c], S2, seed=8, chain=c, group=group, perm_chain=0) for c in (0, 5, 31)}
    for it in range(3):
        b.iterate(1)
        for c, oc in oracles.items():
            oc.iterate(it)
            s, o = b.state(c), oc.state()
            compare(s, o, f"iteration {it} chain {c}")
            np.testing.assert_allclose(s["pi"][:, :4], o["pi"][:, :4], rtol=RTOL)


def test_batch_iterations_in_one_call_equal_single_calls(gpu_lib):
    N, M, C = 800, 120, 32
    bed, ys = problem(N, M, C, seed=11)
    one = make_batch(bed, N, ys, S1, C, seed=2)
    one.iterate(4)
    step = make_batch(bed, N, ys, S1, C, seed=2)
    for _ in range(4):
        step.iterate(1)
    for c in (0, 9, 31):
        a, b = one.state(c), step.state(c)
        np.testing.assert_array_equal(a["beta"], b["beta"])
        np.testing.assert_array_equal(a["eps"], b["eps"])


def test_batch_missing_genotypes_rejected(gpu_lib):
    g, _ = plink.synth_genotypes(300, 40, 1, missing=0.01)
    b = gpu.Batch(gpu.ChainConfig(N=300, M=40), 32)
    with pytest.raises(gpu.BrrError) as e:
        b.pack_bed(plink.encode_bed(g))
    assert "missing" in str(e.value)
    b.close()


def test_batch_too_many_individuals_for_64_chains(gpu_lib):
    with pytest.raises(gpu.BrrError) as e:
        gpu.Batch(gpu.ChainConfig(N=200000, M=10), 64)
    assert "does not fit" in str(e.value)


def test_batch_phase_counting_variant_changes_no_result(gpu_lib):
    """The phase-counting variant of the batched sweep computes the same chains
    bit for bit; with counting off the cycles read zero."""
    N, M, C = 1500, 200, 32
    bed, ys = problem(N, M, C, 17)
    plain = make_batch(bed, N, ys, S1, C, 5)
    counted = make_batch(bed, N, ys, S1, C, 5)
    counted.set_profiling(True)
    plain.iterate(2)
    counted.iterate(2)
    for c in (0, 13, C - 1):
        a, b = plain.state(c), counted.state(c)
        for k in ("beta", "comp", "eps"):
            np.testing.assert_array_equal(a[k], b[k])
    assert (plain.timing()[2] == 0).all()
    assert (counted.timing()[2] > 0).any()
    plain.close()
    counted.close()


def test_batch_wait_limit_returns_timeout_and_batch_recovers(gpu_lib):
    """The barrier before the resolve waits for a phantom CTA: every wait runs
    out after its short limit (the CTAs leave and free their TMEM), the call
    returns BRR_ERR_TIMEOUT, and the batch, re-initialised, follows the
    oracle's chains."""
    N, M, C = 1000, 96, 32
    bed, ys = problem(N, M, C, seed=12)
    b = make_batch(bed, N, ys, S1, C, seed=4, chain0=3)
    b.set_wait_limit(50_000_000, 1)
    for _ in range(2):
        with pytest.raises(gpu.BrrError) as e:
            b.iterate(1)
        assert e.value.code == -4
    b.set_wait_limit(2_000_000_000, 0)
    b.init()
    b.iterate(2)
    for c in (0, 31):
        oc = O.OracleChain(bed, N, ys[c], S1, seed=4, chain=3 + c, perm_chain=3)
        oc.iterate(0)
        oc.iterate(1)
        compare(b.state(c), oc.state(), f"chain {c}")
    b.close()
