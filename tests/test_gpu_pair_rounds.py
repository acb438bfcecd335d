"""Pair-resolved rounds of the FP32C ragged sweep against the FP64 oracle and
against the FP32C restart sweep, through the C ABI.

A round resolves all its markers: after a change at marker p the later
markers' num move by the exact linear change of x_t . eps that p's residual
update makes, built from integer pair terms summed over the slices.  With
pair_rounds = 1 every sweep takes pair-resolved rounds, with pair_rounds = 0
(the default) the first sweep and those that follow one with more than M/40
non-zero effects.  Only
rounding separates the result from the restart sweep, which samples every
marker against the residual itself, so the bars are the FP32C form's:
components identical, beta within 1e-7 relative of the FP64 oracle, the
residual within 1e-9.
"""
import numpy as np
import pytest

import oracle_lib as O
from bayesrrcmd_gb300 import gpu, plink

pytestmark = pytest.mark.gpu
S1 = [[0.01, 0.001, 0.0001]]
S2 = [[0.01, 0.001, 0.0001], [0.1, 0.01]]


def problem(N, M, seed, miss, p_lo=0.01, p_hi=0.5, n_causal=None):
    g, _ = plink.synth_genotypes(N, M, seed, missing=miss, p_lo=p_lo, p_hi=p_hi)
    bed = plink.encode_bed(g)
    y, _, _ = plink.synth_phenotype(g, seed, n_causal or max(1, M // 20), 0.6)
    return bed, y


def make(bed, N, y, S, group=None, seed=1, pair_rounds=1, **kw):
    M = bed.shape[0]
    ch = gpu.Chain(gpu.ChainConfig(N=N, M=M, kind=gpu.KIND_RAGGED, form=gpu.FORM_FP32C, S=S, seed=seed,
                                   refresh_every=4, pair_rounds=pair_rounds, **kw))
    ch.pack_bed(bed)
    if group is not None:
        ch.set_groups(group)
    ch.set_phenotype(y)
    ch.init()
    return ch


def close_to_oracle(s, o, what):
    np.testing.assert_array_equal(s["comp"], o["comp"], err_msg=what)
    nz = o["beta"] != 0
    np.testing.assert_array_equal(s["beta"] != 0, nz, err_msg=what)
    np.testing.assert_allclose(s["beta"][nz], o["beta"][nz], rtol=1e-7, atol=1e-12, err_msg=what)
    np.testing.assert_allclose(s["eps"], o["eps"], rtol=0, atol=1e-9, err_msg=what)
    np.testing.assert_allclose(s["sigmaE"], o["sigmaE"], rtol=1e-8, err_msg=what)
    np.testing.assert_allclose(s["sigmaG"], o["sigmaG"], rtol=1e-7, err_msg=what)
    np.testing.assert_allclose(s["epsSum"], o["epsSum"], rtol=1e-8, atol=1e-8, err_msg=what)


@pytest.mark.parametrize("N,M,miss,p_lo,p_hi", [
    (4000, 800, 0.01, 0.01, 0.5),       # common and rare markers, missing genotypes
    (20_000, 1000, 0.01, 0.001, 0.05),  # rare markers: many rounds with few shared individuals
    (1203, 333, 0.02, 0.05, 0.5),       # a last round of 13 markers, few individuals per slice
    (150, 70, 0.0, 0.1, 0.5),           # three 64-individual slices
])
def test_pair_rounds_match_oracle_each_iteration(gpu_lib, N, M, miss, p_lo, p_hi):
    bed, y = problem(N, M, seed=N + M, miss=miss, p_lo=p_lo, p_hi=p_hi)
    ch = make(bed, N, y, S1, seed=6)
    assert ch.round_info()["pair_rounds"]
    oc = O.OracleChain(bed, N, y, S1, kind=gpu.KIND_RAGGED, seed=6)
    changed = 0
    for it in range(5):
        ch.iterate(1)
        oc.iterate(it)
        s, o = ch.state(), oc.state()
        close_to_oracle(s, o, f"iteration {it}")
        changed += int(np.count_nonzero(o["beta"]))
    assert changed > 10
    # one round per 32 markers
    assert ch.timing()[2] == -(-M // 32)


def test_pair_rounds_two_groups(gpu_lib):
    N, M = 3001, 640
    bed, y = problem(N, M, seed=77, miss=0.01)
    group = (np.arange(M) % 2).astype(np.int32)
    ch = make(bed, N, y, S2, group=group, seed=3)
    oc = O.OracleChain(bed, N, y, S2, kind=gpu.KIND_RAGGED, group=group, seed=3)
    for it in range(4):
        ch.iterate(1)
        oc.iterate(it)
        close_to_oracle(ch.state(), oc.state(), f"iteration {it}")


def test_pair_rounds_and_restart_rounds_agree(gpu_lib):
    N, M = 6000, 900
    bed, y = problem(N, M, seed=5, miss=0.01)
    a = make(bed, N, y, S1, seed=11)
    b = make(bed, N, y, S1, seed=11, pair_rounds=-1)
    assert a.round_info()["pair_rounds"] and not b.round_info()["pair_rounds"]
    for _ in range(6):
        a.iterate(1)
        b.iterate(1)
        sa, sb = a.state(), b.state()
        np.testing.assert_array_equal(sa["comp"], sb["comp"])
        nz = sb["beta"] != 0
        np.testing.assert_allclose(sa["beta"][nz], sb["beta"][nz], rtol=1e-9, atol=1e-13)
        np.testing.assert_allclose(sa["eps"], sb["eps"], rtol=0, atol=1e-10)
    # far fewer grid rounds than the restart sweep's one per change
    assert a.timing()[2] * 2 < b.timing()[2]


def test_automatic_choice_follows_the_number_of_effects(gpu_lib):
    """pair_rounds = 0: pair-resolved rounds in the first sweep and after any sweep
    that leaves more than M/40 non-zero effects, restart rounds otherwise; both
    give the chain of the restart rounds up to rounding."""
    N, M = 4000, 1200
    bed, y = problem(N, M, seed=31, miss=0.01, n_causal=6)
    auto = make(bed, N, y, S1, seed=4, pair_rounds=0)
    restart = make(bed, N, y, S1, seed=4, pair_rounds=-1)
    modes = []
    for it in range(8):
        auto.iterate(1)
        restart.iterate(1)
        sa, sb = auto.state(), restart.state()
        np.testing.assert_array_equal(sa["comp"], sb["comp"])
        nz = sb["beta"] != 0
        np.testing.assert_allclose(sa["beta"][nz], sb["beta"][nz], rtol=1e-9, atol=1e-13)
        modes.append((auto.timing()[2], restart.timing()[2], int(np.count_nonzero(sb["beta"]))))
    assert modes[0][0] == -(-M // 32)
    for k in range(1, len(modes)):
        prev_nnz = modes[k - 1][2]
        if prev_nnz * 40 > M:
            assert modes[k][0] == -(-M // 32), modes
        else:
            assert modes[k][0] == modes[k][1], modes


def test_pair_rounds_are_not_used_where_they_do_not_apply(gpu_lib):
    N, M = 1000, 100
    bed, y = problem(N, M, seed=9, miss=0.01)
    for kw in (dict(kind=gpu.KIND_EIGEN), dict(spec_width=64), dict(cluster=8)):
        kind = kw.pop("kind", gpu.KIND_RAGGED)
        ch = gpu.Chain(gpu.ChainConfig(N=N, M=M, kind=kind, form=gpu.FORM_FP32C, S=S1, seed=1, **kw))
        ch.pack_bed(bed)
        ch.set_phenotype(y)
        ch.init()
        assert not ch.round_info()["pair_rounds"], kw
        ch.close()
        # and cannot be required there
        if "cluster" not in kw:
            ch = gpu.Chain(gpu.ChainConfig(N=N, M=M, kind=kind, form=gpu.FORM_FP32C, S=S1, seed=1, pair_rounds=1, **kw))
            ch.pack_bed(bed)
            ch.set_phenotype(y)
            with pytest.raises(gpu.BrrError):
                ch.init()
            ch.close()


def test_pair_rounds_wait_limit_returns_timeout_and_context_recovers(gpu_lib):
    N, M = 2000, 200
    bed, y = problem(N, M, seed=2, miss=0.01)
    ch = make(bed, N, y, S1, seed=2)
    ch.set_wait_limit(50_000_000, 1)
    with pytest.raises(gpu.BrrError) as e:
        ch.iterate(1)
    assert e.value.code == -4
    ch.set_wait_limit(2_000_000_000, 0)
    ch.init()
    ch.iterate(2)
    oc = O.OracleChain(bed, N, y, S1, kind=gpu.KIND_RAGGED, seed=2)
    oc.iterate(0)
    oc.iterate(1)
    close_to_oracle(ch.state(), oc.state(), "after recovery")


def make_dense(bed, N, y, S, group=None, seed=1, pair_rounds=1, **kw):
    M = bed.shape[0]
    ch = gpu.Chain(gpu.ChainConfig(N=N, M=M, kind=gpu.KIND_DENSE, form=gpu.FORM_FP32C, S=S, seed=seed, gram=-1,
                                   refresh_every=4, pair_rounds=pair_rounds, **kw))
    ch.pack_bed(bed)
    if group is not None:
        ch.set_groups(group)
    ch.set_phenotype(y)
    ch.init()
    return ch


def close_dense(s, o, what):
    np.testing.assert_array_equal(s["comp"], o["comp"], err_msg=what)
    nz = o["beta"] != 0
    np.testing.assert_array_equal(s["beta"] != 0, nz, err_msg=what)
    np.testing.assert_allclose(s["beta"][nz], o["beta"][nz], rtol=1e-7, atol=1e-12, err_msg=what)
    np.testing.assert_allclose(s["eps"], o["eps"], rtol=0, atol=1e-9, err_msg=what)
    np.testing.assert_allclose(s["sigmaE"], o["sigmaE"], rtol=1e-8, err_msg=what)
    np.testing.assert_allclose(s["sigmaG"], o["sigmaG"], rtol=1e-7, err_msg=what)


@pytest.mark.parametrize("N,M,miss", [
    (4000, 800, 0.01),     # missing genotypes: all four pair terms
    (3000, 500, 0.0),      # the genotype products alone
    (1203, 333, 0.02),     # a last round of 13 markers, a partial last code word
    (150, 70, 0.0),        # three 64-individual slices
])
def test_dense_pair_rounds_match_oracle_each_iteration(gpu_lib, N, M, miss):
    """Dense markers: the pair terms come from the 2-bit code words (genotype
    sum, products, individuals missing at either marker); num_t moves by
    dBeta_p times the change of sigma_t (sum g_t eps - colmean_t (total -
    missing sum)) + xm_t (missing sum) that p's update makes."""
    bed, y = problem(N, M, seed=N + 2 * M, miss=miss, p_lo=0.05, p_hi=0.5)
    ch = make_dense(bed, N, y, S1, seed=6)
    assert ch.round_info()["pair_rounds"] and not ch.gram_info()["blocked"]
    oc = O.OracleChain(bed, N, y, S1, kind=gpu.KIND_DENSE, seed=6)
    changed = 0
    for it in range(5):
        ch.iterate(1)
        oc.iterate(it)
        s, o = ch.state(), oc.state()
        close_dense(s, o, f"iteration {it}")
        changed += int(np.count_nonzero(o["beta"]))
    assert changed > 10
    assert ch.timing()[2] == -(-M // 32)
    assert ch.round_info()["last_sweep_pair_rounds"]


def test_dense_pair_rounds_two_groups(gpu_lib):
    N, M = 3001, 640
    bed, y = problem(N, M, seed=78, miss=0.01, p_lo=0.05)
    group = (np.arange(M) % 2).astype(np.int32)
    ch = make_dense(bed, N, y, S2, group=group, seed=3)
    oc = O.OracleChain(bed, N, y, S2, kind=gpu.KIND_DENSE, group=group, seed=3)
    for it in range(4):
        ch.iterate(1)
        oc.iterate(it)
        close_dense(ch.state(), oc.state(), f"iteration {it}")


@pytest.mark.parametrize("miss", [0.0, 0.01])
def test_dense_pair_rounds_and_restart_rounds_agree(gpu_lib, miss):
    N, M = 6000, 900
    bed, y = problem(N, M, seed=15, miss=miss, p_lo=0.05)
    a = make_dense(bed, N, y, S1, seed=11)
    b = make_dense(bed, N, y, S1, seed=11, pair_rounds=-1)
    assert not b.round_info()["pair_rounds"]
    for _ in range(6):
        a.iterate(1)
        b.iterate(1)
        sa, sb = a.state(), b.state()
        np.testing.assert_array_equal(sa["comp"], sb["comp"])
        nz = sb["beta"] != 0
        np.testing.assert_allclose(sa["beta"][nz], sb["beta"][nz], rtol=1e-9, atol=1e-13)
        np.testing.assert_allclose(sa["eps"], sb["eps"], rtol=0, atol=1e-10)
    assert a.timing()[2] < b.timing()[2]


def test_dense_pair_rounds_wait_limit_returns_timeout_and_context_recovers(gpu_lib):
    N, M = 2000, 200
    bed, y = problem(N, M, seed=4, miss=0.01, p_lo=0.05)
    ch = make_dense(bed, N, y, S1, seed=2)
    ch.set_wait_limit(50_000_000, 1)
    with pytest.raises(gpu.BrrError) as e:
        ch.iterate(1)
    assert e.value.code == -4
    ch.set_wait_limit(2_000_000_000, 0)
    ch.init()
    ch.iterate(2)
    oc = O.OracleChain(bed, N, y, S1, kind=gpu.KIND_DENSE, seed=2)
    oc.iterate(0)
    oc.iterate(1)
    close_dense(ch.state(), oc.state(), "after recovery")


def test_pair_rounds_and_the_gram_blocked_sweep_exclude_each_other(gpu_lib):
    N, M = 1000, 100
    bed, y = problem(N, M, seed=9, miss=0.0, p_lo=0.05)
    ch = gpu.Chain(gpu.ChainConfig(N=N, M=M, kind=gpu.KIND_DENSE, form=gpu.FORM_FP32C, S=S1, seed=1, gram=1,
                                   pair_rounds=1))
    ch.pack_bed(bed)
    ch.set_phenotype(y)
    with pytest.raises(gpu.BrrError):
        ch.init()
    ch.close()
    # with the Gram-blocked sweep the chain takes no pair-resolved rounds
    ch = gpu.Chain(gpu.ChainConfig(N=N, M=M, kind=gpu.KIND_DENSE, form=gpu.FORM_FP32C, S=S1, seed=1, gram=1))
    ch.pack_bed(bed)
    ch.set_phenotype(y)
    ch.init()
    ch.iterate(1)
    assert ch.gram_info()["blocked"] and not ch.round_info()["pair_rounds"]
    assert not ch.round_info()["last_sweep_pair_rounds"]
