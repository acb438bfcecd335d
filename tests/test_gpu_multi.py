"""Uneven batch (independent regressions of different sizes in one launch) vs
the oracle, instance by instance.

Every instance is a chain with its own genotypes, phenotype, seed, chain id
and marker kind; the autotuner's iterations are real iterations, so the
oracle chains run them too.  The plain FP64 form matches at the single-chain
bars (1e-10 relative, components identical); the FP32C form at its bars.
"""
import numpy as np
import pytest

import oracle_lib as O
from bayesrrcmd_gb300 import gpu, plink

pytestmark = pytest.mark.gpu
S1 = [[0.01, 0.001, 0.0001]]
S2 = [[0.01, 0.001, 0.0001], [0.1, 0.01]]

SHAPES = [  # N, M, kind, missing
    (300, 200, gpu.KIND_DENSE, 0.0),
    (1203, 150, gpu.KIND_RAGGED, 0.01),
    (2500, 300, gpu.KIND_DENSE, 0.01),
    (5000, 100, gpu.KIND_EIGEN, 0.02),
    (700, 250, gpu.KIND_RAGGED, 0.0),
]


def problems(shapes, seed0):
    out = []
    for k, (N, M, kind, miss) in enumerate(shapes):
        g, _ = plink.synth_genotypes(N, M, seed0 + k, missing=miss, p_lo=0.02)
        bed = plink.encode_bed(g)
        y, _, _ = plink.synth_phenotype(g, seed0 + k, max(1, M // 30), 0.5)
        out.append((N, M, kind, bed, y))
    return out


def make(probs, form, S, seed=3):
    cfgs = [gpu.ChainConfig(N=N, M=M, kind=kind, form=form, S=S, seed=seed, chain=10 + k,
                            refresh_every=2 if form == gpu.FORM_FP32C else 0)
            for k, (N, M, kind, _, _) in enumerate(probs)]
    m = gpu.Multi(cfgs)
    for k, (N, M, kind, bed, y) in enumerate(probs):
        m.pack_bed(k, bed)
        if len(S) > 1:
            m.set_groups(k, (np.arange(M) % 2).astype(np.int32))
        m.set_phenotype(k, y)
    m.init()
    return m


def oracles(probs, S, seed=3):
    return [O.OracleChain(bed, N, y, S, kind=kind, seed=seed, chain=10 + k,
                          group=(np.arange(M) % 2).astype(np.int32) if len(S) > 1 else None)
            for k, (N, M, kind, bed, y) in enumerate(probs)]


def test_multi_fp64_matches_oracle_through_tuning(gpu_lib):
    probs = problems(SHAPES, 40)
    m = make(probs, gpu.FORM_FP64, S2)
    ocs = oracles(probs, S2)
    it = 0
    m.tune(1)                       # 3 round widths + 1 rebalancing = 4 iterations
    for _ in range(4):
        for oc in ocs:
            oc.iterate(it)
        it += 1
    for step in range(2):
        m.iterate(1)
        for oc in ocs:
            oc.iterate(it)
        it += 1
        for k, oc in enumerate(ocs):
            s, o = m.state(k), oc.state()
            what = f"instance {k} iteration {it - 1}"
            np.testing.assert_array_equal(s["comp"], o["comp"], err_msg=what)
            nz = o["beta"] != 0
            np.testing.assert_allclose(s["beta"][nz], o["beta"][nz], rtol=1e-10, err_msg=what)
            np.testing.assert_allclose(s["sigmaE"], o["sigmaE"], rtol=1e-10, err_msg=what)
            # sigmaG is drawn from the sum of the group's squared betas over six
            # iterations of drift: 1e-9
            np.testing.assert_allclose(s["sigmaG"], o["sigmaG"], rtol=1e-9, err_msg=what)
            np.testing.assert_allclose(s["mu"], o["mu"], rtol=1e-10, atol=1e-14, err_msg=what)
            np.testing.assert_allclose(s["eps"], o["eps"], rtol=0, atol=1e-11, err_msg=what)
    t = m.timing()
    assert t["ctas"].sum() <= 152 and (t["ctas"] >= 1).all()
    assert set(t["width"].tolist()) <= {8, 16, 32}
    assert (t["inst_ms"] > 0).all()
    m.close()


def test_multi_fp32c_tracks_fp64_oracle(gpu_lib):
    probs = problems(SHAPES[:4], 60)
    m = make(probs, gpu.FORM_FP32C, S1)
    ocs = oracles(probs, S1)
    for it in range(3):
        m.iterate(1)
        for k, oc in enumerate(ocs):
            oc.iterate(it)
            s, o = m.state(k), oc.state()
            what = f"instance {k} iteration {it}"
            np.testing.assert_array_equal(s["comp"], o["comp"], err_msg=what)
            nz = o["beta"] != 0
            np.testing.assert_allclose(s["beta"][nz], o["beta"][nz], rtol=1e-7, atol=1e-12, err_msg=what)
            np.testing.assert_allclose(s["eps"], o["eps"], rtol=0, atol=1e-9, err_msg=what)
    m.close()


def test_multi_single_instance_equals_single_chain(gpu_lib):
    """One instance in the multi-instance launch is the single-chain sweep."""
    N, M = 3000, 400
    g, _ = plink.synth_genotypes(N, M, 7, missing=0.01)
    bed = plink.encode_bed(g)
    y, _, _ = plink.synth_phenotype(g, 7, 10, 0.5)
    cfg = gpu.ChainConfig(N=N, M=M, S=S1, seed=9, grid=8)
    m = gpu.Multi([cfg])
    m.pack_bed(0, bed)
    m.set_phenotype(0, y)
    m.init()
    m.iterate(3)
    ch = gpu.Chain(gpu.ChainConfig(N=N, M=M, S=S1, seed=9, grid=int(m.timing()["ctas"][0])))
    ch.pack_bed(bed)
    ch.set_phenotype(y)
    ch.init()
    ch.iterate(3)
    a, b = m.state(0), ch.state()
    np.testing.assert_array_equal(a["beta"], b["beta"])
    np.testing.assert_array_equal(a["eps"], b["eps"])
    m.close()
    ch.close()


def test_multi_wait_limit_returns_timeout_and_instances_recover(gpu_lib):
    """One instance's grid barrier waits for a phantom CTA: its waits run out
    after the short limit, the iteration returns BRR_ERR_TIMEOUT while the
    other instances finish, and after brr_multi_init every instance follows
    its oracle chain again."""
    probs = problems(SHAPES[:3], 80)
    m = make(probs, gpu.FORM_FP64, S1)
    m.set_wait_limit(50_000_000, 1, instance=1)
    with pytest.raises(gpu.BrrError) as e:
        m.iterate(1)
    assert e.value.code == -4
    m.set_wait_limit(2_000_000_000, 0)
    m.init()
    m.iterate(2)
    ocs = oracles(probs, S1)
    for k, oc in enumerate(ocs):
        oc.iterate(0)
        oc.iterate(1)
        s, o = m.state(k), oc.state()
        np.testing.assert_array_equal(s["comp"], o["comp"], err_msg=f"instance {k}")
        nz = o["beta"] != 0
        np.testing.assert_allclose(s["beta"][nz], o["beta"][nz], rtol=1e-10, err_msg=f"instance {k}")
        np.testing.assert_allclose(s["eps"], o["eps"], rtol=0, atol=1e-11, err_msg=f"instance {k}")
    m.close()
