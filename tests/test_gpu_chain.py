"""GPU Gibbs chain vs the CPU oracle, through the C ABI.

Tolerances (FP64 plain form, the drop-in): per-iteration beta, sigmaG, sigmaE
and mu within 1e-10 relative of the oracle, components identical.  The
replayed stream makes the chains comparable draw for draw; only the
summation order of dot products differs.
"""
from pathlib import Path

import numpy as np
import pytest

import oracle_lib as O
from bayesrrcmd_gb300 import gpu, plink

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"
RTOL = 1e-10
S1 = [[0.01, 0.001, 0.0001]]
S2 = [[0.01, 0.001, 0.0001], [0.1, 0.01]]


def problem(N, M, seed, miss=0.0, n_causal=None, h2=0.5, p_lo=0.05):
    g, _ = plink.synth_genotypes(N, M, seed, missing=miss, p_lo=p_lo)
    bed = plink.encode_bed(g)
    y, _, _ = plink.synth_phenotype(g, seed, n_causal or max(1, M // 50), h2)
    return bed, y


def make_gpu(bed, N, y, S, kind, form=gpu.FORM_FP64, group=None, seed=1, **kw):
    M = bed.shape[0]
    ch = gpu.Chain(gpu.ChainConfig(N=N, M=M, kind=kind, form=form, S=S, seed=seed, **kw))
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
    np.testing.assert_allclose(s["beta"][nz], o["beta"][nz], rtol=rtol, err_msg=what)
    np.testing.assert_allclose(s["sigmaE"], o["sigmaE"], rtol=rtol, err_msg=what)
    np.testing.assert_allclose(s["sigmaG"], o["sigmaG"], rtol=rtol, err_msg=what)
    np.testing.assert_allclose(s["mu"], o["mu"], rtol=rtol, atol=1e-14, err_msg=what)


@pytest.mark.parametrize("kind", [gpu.KIND_DENSE, gpu.KIND_RAGGED, gpu.KIND_EIGEN])
@pytest.mark.parametrize("N,M,miss", [(2000, 600, 0.0), (1203, 400, 0.01), (60, 50, 0.02)])
def test_fp64_chain_matches_oracle_each_iteration(gpu_lib, kind, N, M, miss):
    bed, y = problem(N, M, seed=N + M + kind, miss=miss)
    ch = make_gpu(bed, N, y, S1, kind, seed=3)
    oc = O.OracleChain(bed, N, y, S1, kind=kind, seed=3)
    for it in range(5):
        ch.iterate(1)
        oc.iterate(it)
        assert_close(ch.state(), oc.state(), what=f"iteration {it}")
    np.testing.assert_allclose(ch.state()["eps"], oc.state()["eps"], rtol=0, atol=1e-11)


GOLDEN_NAMES = {0: "synth_dense.npz", 1: "synth_ragged.npz", 2: "synth_eigen.npz"}


@pytest.mark.parametrize("kind", [0, 1, 2])
def test_fp64_chain_matches_committed_golden_trace(gpu_lib, kind):
    """Two groups with 4 and 3 components, missing genotypes, N = 203."""
    d = dict(np.load(GOLDEN / GOLDEN_NAMES[kind]))
    N = int(d["N"])
    ch = make_gpu(d["bed"], N, d["y"], S2, kind, group=d["group"], seed=int(d["seed"]))
    for it in range(d["trace_beta"].shape[0]):
        ch.iterate(1)
        s = ch.state()
        o = {k: d[f"trace_{k}"][it] for k in ("beta", "comp", "sigmaE", "sigmaG", "mu")}
        assert_close(s, o, what=f"iteration {it}")
    np.testing.assert_allclose(ch.state()["eps"], d["eps_final"], rtol=0, atol=1e-11)


def test_fp64_two_groups_different_component_counts(gpu_lib):
    N, M = 1500, 900
    bed, y = problem(N, M, seed=17)
    group = (np.arange(M) % 2).astype(np.int32)
    ch = make_gpu(bed, N, y, S2, 0, group=group, seed=9)
    oc = O.OracleChain(bed, N, y, S2, kind=0, group=group, seed=9)
    for it in range(4):
        ch.iterate(1)
        oc.iterate(it)
        s, o = ch.state(), oc.state()
        assert_close(s, o, what=f"iteration {it}")
        np.testing.assert_allclose(s["pi"][:, :4], o["pi"][:, :4], rtol=RTOL)
        assert (s["comp"][group == 1] < 3).all()


@pytest.mark.parametrize("kind", [0, 1, 2])
def test_sweep_boundary_resynchronised_from_oracle_state(gpu_lib, kind):
    """brr_set_state + brr_sweep with the oracle's own order and draws, for
    several iterations of a running chain: one sweep at a time, re-synchronised."""
    N, M = 900, 300
    bed, y = problem(N, M, seed=41, miss=0.01)
    oc = O.OracleChain(bed, N, y, S1, kind=kind, seed=5)
    ch = make_gpu(bed, N, y, S1, kind, seed=5)
    for it in range(4):
        oc.iterate(it)
        st = oc.state()
        ch.set_state(st)
        order = O.permutation(5, 0, 100 + it, M)
        u, z = O.marker_draws(5, 0, 100 + it, M)
        out = ch.sweep(order, u, z)
        oc.sweep(order, u, z)
        s, o = ch.state(), oc.state()
        np.testing.assert_array_equal(s["comp"], o["comp"])
        nz = o["beta"] != 0
        np.testing.assert_allclose(s["beta"][nz], o["beta"][nz], rtol=RTOL)
        np.testing.assert_allclose(s["acum"], o["acum"], rtol=1e-9, atol=1e-14)
        np.testing.assert_allclose(s["eps"], o["eps"], rtol=0, atol=1e-11)
        np.testing.assert_allclose(np.array(out.v[:4]), o["v"][0, :4])
        np.testing.assert_allclose(out.betasqnG[0], o["betasqnG"][0], rtol=RTOL)
        np.testing.assert_allclose(out.eps_sqnorm, (o["eps"] ** 2).sum(), rtol=1e-12)
        if kind != 0:
            np.testing.assert_allclose(s["epsSum"], o["epsSum"], rtol=1e-9, atol=1e-9)


@pytest.mark.parametrize("kind", [0, 1, 2])
def test_speculation_width_does_not_change_results(gpu_lib, kind):
    """Markers are accepted only while the residual is unchanged, so the width
    of the speculative round changes the chain only through the rounding of
    the partial dot products (the lanes per marker follow the width)."""
    N, M = 1000, 400
    bed, y = problem(N, M, seed=8, miss=0.01)
    ref = None
    for w in (8, 16, 32, 64):
        ch = make_gpu(bed, N, y, S1, kind, seed=2, spec_width=w)
        ch.iterate(3)
        s = ch.state()
        ch.close()
        if ref is None:
            ref = s
        else:
            assert_close(s, ref, rtol=1e-12)
            np.testing.assert_allclose(s["eps"], ref["eps"], rtol=0, atol=1e-13)


def test_grid_size_changes_only_rounding(gpu_lib):
    N, M = 3000, 200
    bed, y = problem(N, M, seed=12)
    states = []
    for grid in (1, 7, 0):
        ch = make_gpu(bed, N, y, S1, 0, seed=4, grid=grid)
        ch.iterate(2)
        states.append(ch.state())
        ch.close()
    for s in states[1:]:
        assert_close(s, states[0])


def test_tiny_problems(gpu_lib):
    for N, M in ((2, 1), (3, 2), (9, 70)):
        g = np.tile(np.array([0, 1, 2], np.int8), (M, N))[:, :N]
        g[:, 0] = 0
        g[:, 1] = 1
        bed = plink.encode_bed(g)
        y = np.linspace(-1, 1, N).astype(np.float32)
        for kind in (0, 1, 2):
            ch = make_gpu(bed, N, y, S1, kind, seed=1)
            oc = O.OracleChain(bed, N, y, S1, kind=kind, seed=1)
            for it in range(3):
                ch.iterate(1)
                oc.iterate(it)
                assert_close(ch.state(), oc.state(), rtol=1e-9)


def test_fp32c_tracks_fp64_oracle(gpu_lib):
    """FP32-compensated form: same components as the FP64 oracle over a short
    chain and beta within 1e-7 relative; the residual stays within 1e-9."""
    N, M = 4000, 800
    bed, y = problem(N, M, seed=23, miss=0.01)
    for kind in (0, 1, 2):
        ch = make_gpu(bed, N, y, S1, kind, form=gpu.FORM_FP32C, seed=6, refresh_every=2)
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


def test_refresh_reproduces_residual(gpu_lib):
    N, M = 1500, 300
    bed, y = problem(N, M, seed=31, miss=0.02)
    for kind in (0, 1, 2):
        ch = make_gpu(bed, N, y, S1, kind, seed=7)
        ch.iterate(3)
        before = ch.state()["eps"]
        ch.refresh()
        np.testing.assert_allclose(ch.state()["eps"], before, rtol=0, atol=1e-11)


def test_wait_limit_returns_timeout_status_and_context_recovers(gpu_lib):
    """The grid barrier is told to wait for arrivals that never come; every
    wait runs out after its short limit, the call returns BRR_ERR_TIMEOUT and
    the same context runs normally afterwards."""
    N, M = 1000, 100
    bed, y = problem(N, M, seed=2)
    ch = make_gpu(bed, N, y, S1, 0, seed=2)
    ch.set_wait_limit(50_000_000, 1)
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


@pytest.mark.parametrize("miss", [0.0, 0.02])
def test_blocked_sweep_wait_limit_returns_timeout_and_context_recovers(gpu_lib, miss):
    """The Gram-blocked FP32C sweep: its grid barrier waits for a phantom CTA;
    the barrier wait and the role signals run out after the short limit, the
    bulk Gram copies in flight are waited for, the call returns BRR_ERR_TIMEOUT
    and the same context, re-initialised, follows the oracle's chain."""
    N, M = 1500, 300
    bed, y = problem(N, M, seed=3, miss=miss)
    ch = make_gpu(bed, N, y, S1, 0, form=gpu.FORM_FP32C, seed=2, gram=1, refresh_every=3)
    assert ch.gram_info()["blocked"]
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
    s, o = ch.state(), oc.state()
    np.testing.assert_array_equal(s["comp"], o["comp"])
    nz = o["beta"] != 0
    np.testing.assert_allclose(s["beta"][nz], o["beta"][nz], rtol=1e-9, atol=1e-13)
    np.testing.assert_allclose(s["eps"], o["eps"], rtol=0, atol=1e-10)


def test_call_order_errors(gpu_lib):
    ch = gpu.Chain(gpu.ChainConfig(N=100, M=3))
    with pytest.raises(gpu.BrrError):
        ch.iterate(1)
    g, _ = plink.synth_genotypes(100, 3, 1)
    ch.pack_bed(plink.encode_bed(g))
    with pytest.raises(gpu.BrrError):
        ch.set_groups(np.array([0, 1, 0], np.int32))
    with pytest.raises(gpu.BrrError):
        ch.set_phenotype(np.full(100, np.nan, np.float32))


@pytest.mark.parametrize("miss", [0.0, 0.02])
def test_gram_blocked_fp32c_matches_restart_fp32c_and_oracle(gpu_lib, miss):
    """The blocked FP32C sweep (exact Gram corrections, fixed rounds of B
    markers) follows the same chain as the restart sweep and the FP64 oracle:
    identical components, beta within 1e-9 relative."""
    N, M = 3000, 700
    bed, y = problem(N, M, seed=51, miss=miss)
    group = (np.arange(M) % 2).astype(np.int32)
    blocked = make_gpu(bed, N, y, S2, 0, form=gpu.FORM_FP32C, group=group, seed=8, refresh_every=3, gram=1)
    assert blocked.gram_info()["blocked"]
    restart = make_gpu(bed, N, y, S2, 0, form=gpu.FORM_FP32C, group=group, seed=8, refresh_every=3, gram=-1)
    assert not restart.gram_info()["blocked"]
    oc = O.OracleChain(bed, N, y, S2, kind=0, group=group, seed=8)
    for it in range(4):
        blocked.iterate(1)
        restart.iterate(1)
        oc.iterate(it)
        b, r, o = blocked.state(), restart.state(), oc.state()
        for s in (b, r):
            np.testing.assert_array_equal(s["comp"], o["comp"])
            nz = o["beta"] != 0
            np.testing.assert_allclose(s["beta"][nz], o["beta"][nz], rtol=1e-9, atol=1e-13)
            np.testing.assert_allclose(s["eps"], o["eps"], rtol=0, atol=1e-10)
            np.testing.assert_allclose(s["sigmaG"], o["sigmaG"], rtol=1e-9)
    sw, tot, rounds = blocked.timing()
    assert rounds == -(-M // 64)


@pytest.mark.parametrize("width", [16, 32])
def test_gram_blocked_other_widths(gpu_lib, width):
    N, M = 1500, 333
    bed, y = problem(N, M, seed=61)
    ch = make_gpu(bed, N, y, S1, 0, form=gpu.FORM_FP32C, seed=4, gram=1, spec_width=width)
    oc = O.OracleChain(bed, N, y, S1, kind=0, seed=4)
    for it in range(3):
        ch.iterate(1)
        oc.iterate(it)
        s, o = ch.state(), oc.state()
        np.testing.assert_array_equal(s["comp"], o["comp"])
        nz = o["beta"] != 0
        np.testing.assert_allclose(s["beta"][nz], o["beta"][nz], rtol=1e-9, atol=1e-13)


@pytest.mark.parametrize("gram,form", [(1, gpu.FORM_FP32C), (-1, gpu.FORM_FP32C), (-1, gpu.FORM_FP64)])
def test_phase_counting_variant_changes_no_result(gpu_lib, gram, form):
    """The phase-counting kernel variants (brr_set_profiling) compute the same
    chain bit for bit; with counting off the counters read zero."""
    N, M = 2500, 450
    bed, y = problem(N, M, seed=71)
    plain = make_gpu(bed, N, y, S1, 0, form=form, seed=6, gram=gram)
    counted = make_gpu(bed, N, y, S1, 0, form=form, seed=6, gram=gram)
    counted.set_profiling(True)
    for _ in range(2):
        plain.iterate(1)
        counted.iterate(1)
        a, b = plain.state(), counted.state()
        for k in ("beta", "comp", "eps", "sigmaG"):
            np.testing.assert_array_equal(a[k], b[k])
        assert a["sigmaE"] == b["sigmaE"] and a["mu"] == b["mu"]
    assert (plain.phase_cycles() == 0).all()
    ph = counted.phase_cycles()
    rounds = counted.timing()[2]
    assert ph[5] == rounds > 0 and ph[3] > 0
    plain.close()
    counted.close()
