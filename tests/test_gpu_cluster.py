"""The restart sweep as one thread-block cluster against the CPU oracle,
through the C ABI.

With `cluster` = C the sweep runs on C CTAs of one cluster: each holds its
slice of the residual in shared memory and stores its partial dot products
into every CTA's shared memory, where the round's mbarrier collects them.
Only the summation order of the partial sums differs from the grid-wide
sweep, so the bars are those of the grid-wide tests: FP64 form, per-iteration
beta, sigmaG, sigmaE and mu within 1e-10 relative of the oracle, components
identical; FP32C form, components identical, beta within 1e-7 relative.
"""
import numpy as np
import pytest

import oracle_lib as O
from bayesrrcmd_gb300 import gpu, plink

pytestmark = pytest.mark.gpu
RTOL = 1e-10
S1 = [[0.01, 0.001, 0.0001]]
S2 = [[0.01, 0.001, 0.0001], [0.1, 0.01]]


def problem(N, M, seed, miss=0.0, n_causal=None, h2=0.5, p_lo=0.05):
    g, _ = plink.synth_genotypes(N, M, seed, missing=miss, p_lo=p_lo)
    bed = plink.encode_bed(g)
    y, _, _ = plink.synth_phenotype(g, seed, n_causal or max(1, M // 50), h2)
    return bed, y


def make_gpu(bed, N, y, S, kind, group=None, seed=1, **kw):
    M = bed.shape[0]
    ch = gpu.Chain(gpu.ChainConfig(N=N, M=M, kind=kind, S=S, seed=seed, **kw))
    ch.pack_bed(bed)
    if group is not None:
        ch.set_groups(group)
    ch.set_phenotype(y)
    ch.init()
    return ch


def assert_close(s, o, rtol=RTOL, what=""):
    np.testing.assert_array_equal(s["comp"], o["comp"], err_msg=what)
    nz = o["beta"] != 0
    np.testing.assert_array_equal(s["beta"] != 0, nz, err_msg=what)
    np.testing.assert_allclose(s["beta"][nz], o["beta"][nz], rtol=rtol, atol=1e-15, err_msg=what)
    np.testing.assert_allclose(s["sigmaE"], o["sigmaE"], rtol=rtol, err_msg=what)
    np.testing.assert_allclose(s["sigmaG"], o["sigmaG"], rtol=rtol, err_msg=what)
    np.testing.assert_allclose(s["mu"], o["mu"], rtol=rtol, atol=1e-14, err_msg=what)


@pytest.mark.parametrize("kind", [gpu.KIND_DENSE, gpu.KIND_RAGGED, gpu.KIND_EIGEN])
@pytest.mark.parametrize("cluster", [16, 8, 2])
@pytest.mark.parametrize("N,M,miss", [(2000, 600, 0.01), (1203, 400, 0.0)])
def test_cluster_fp64_chain_matches_oracle_each_iteration(gpu_lib, kind, cluster, N, M, miss):
    bed, y = problem(N, M, seed=N + M + kind + cluster, miss=miss)
    ch = make_gpu(bed, N, y, S1, kind, seed=3, cluster=cluster)
    oc = O.OracleChain(bed, N, y, S1, kind=kind, seed=3)
    for it in range(5):
        ch.iterate(1)
        oc.iterate(it)
        assert_close(ch.state(), oc.state(), what=f"iteration {it}")
    np.testing.assert_allclose(ch.state()["eps"], oc.state()["eps"], rtol=0, atol=1e-11)


@pytest.mark.parametrize("kind", [gpu.KIND_DENSE, gpu.KIND_RAGGED, gpu.KIND_EIGEN])
def test_cluster_two_groups_and_fewer_slices_than_requested(gpu_lib, kind):
    """N = 203 has four 64-individual chunks: a cluster of 16 is cut to 4 CTAs."""
    N, M = 203, 300
    bed, y = problem(N, M, seed=5, miss=0.02)
    group = (np.arange(M) % 2).astype(np.int32)
    ch = make_gpu(bed, N, y, S2, kind, group=group, seed=4, cluster=16)
    oc = O.OracleChain(bed, N, y, S2, kind=kind, group=group, seed=4)
    for it in range(4):
        ch.iterate(1)
        oc.iterate(it)
        assert_close(ch.state(), oc.state(), rtol=1e-9, what=f"iteration {it}")


@pytest.mark.parametrize("kind", [gpu.KIND_DENSE, gpu.KIND_RAGGED, gpu.KIND_EIGEN])
def test_cluster_fp32c_tracks_fp64_oracle(gpu_lib, kind):
    N, M = 4000, 800
    bed, y = problem(N, M, seed=23, miss=0.01)
    ch = make_gpu(bed, N, y, S1, kind, form=gpu.FORM_FP32C, seed=6, refresh_every=2, cluster=16)
    assert not ch.gram_info()["blocked"]
    oc = O.OracleChain(bed, N, y, S1, kind=kind, seed=6)
    for it in range(4):
        ch.iterate(1)
        oc.iterate(it)
        s, o = ch.state(), oc.state()
        np.testing.assert_array_equal(s["comp"], o["comp"])
        nz = o["beta"] != 0
        np.testing.assert_allclose(s["beta"][nz], o["beta"][nz], rtol=1e-7, atol=1e-12)
        np.testing.assert_allclose(s["eps"], o["eps"], rtol=0, atol=1e-9)
        np.testing.assert_allclose(s["sigmaE"], o["sigmaE"], rtol=1e-8)


def test_cluster_and_grid_sweeps_differ_only_by_rounding(gpu_lib):
    N, M = 5000, 500
    bed, y = problem(N, M, seed=19, miss=0.01)
    for kind in (0, 1, 2):
        a = make_gpu(bed, N, y, S1, kind, seed=8)
        b = make_gpu(bed, N, y, S1, kind, seed=8, cluster=16)
        a.iterate(3)
        b.iterate(3)
        sa, sb = a.state(), b.state()
        assert_close(sb, sa)
        np.testing.assert_allclose(sb["eps"], sa["eps"], rtol=0, atol=1e-12)
        assert a.timing()[2] == b.timing()[2]   # the same rounds
        a.close()
        b.close()


@pytest.mark.parametrize("kind", [gpu.KIND_DENSE, gpu.KIND_RAGGED])
def test_cluster_async_schedule_matches_oracle(gpu_lib, kind):
    N, M, T = 1501, 400, 20
    bed, y = problem(N, M, seed=61, miss=0.01, n_causal=12)
    ch = make_gpu(bed, N, y, S1, kind, seed=9, async_batch=T, cluster=8)
    oc = O.OracleChain(bed, N, y, S1, kind=kind, seed=9, async_batch=T)
    for it in range(4):
        ch.iterate(1)
        oc.iterate(it)
        assert_close(ch.state(), oc.state(), what=f"iteration {it}")
        np.testing.assert_array_equal(ch.state()["acum"], 0.0)


def test_cluster_wait_limit_returns_timeout_status_and_context_recovers(gpu_lib):
    """Every CTA's round mbarrier is told to expect a record that no CTA
    stores; each wait runs out after the short limit, the CTAs meet at the
    closing cluster barrier, the call returns BRR_ERR_TIMEOUT and the same
    context, re-initialised, follows the oracle's chain."""
    N, M = 1000, 100
    bed, y = problem(N, M, seed=2)
    ch = make_gpu(bed, N, y, S1, 0, seed=2, cluster=8)
    ch.set_wait_limit(50_000_000, 1)
    for _ in range(2):
        with pytest.raises(gpu.BrrError) as e:
            ch.iterate(1)
        assert e.value.code == -4
    ch.set_wait_limit(2_000_000_000, 0)
    ch.init()
    ch.iterate(2)
    oc = O.OracleChain(bed, N, y, S1, kind=0, seed=2)
    oc.iterate(0)
    oc.iterate(1)
    assert_close(ch.state(), oc.state())
