"""Parity at the sizes the throughput figures are quoted on.

C3 size: N = 100,000 individuals (the benchmark's N) x M = 10,000 markers,
p ~ U(0.01, 0.5), two marker groups with separate mixtures (S1 =
0.01,0.001,0.0001 on the first half of the markers, S2 = 0.1,0.01 on the
second), 100 causal markers, h2 = 0.4; five iterations.  The plain FP64 chain
matches the FP64 oracle at the drop-in's bar (1e-10 relative per iteration,
components identical) and the Gram-blocked FP32C chain (the chosen form) at
its bars (components identical, beta 1e-9 relative, residual 1e-10
absolute, sigmaG 1e-9).

C4 size: 64 batched chains on N = 50,000 x M = 200,000 shared genotypes,
p ~ U(0.01, 0.5), each chain its own phenotype (h2 ~ U(0.1, 0.7), 1,000 causal
markers); chains 0, 31 and 63 against their oracle chains for two
iterations, at the batched form's bars for this size (c4_compare: the
fixed-point rounding of 40,000 updates per sweep gives betas an absolute
error of a few 1e-13).

The oracle keeps dense markers as four standardised values per marker and
reads the codes from the BED payload (the columns would take 8 GB and 80 GB);
its results are those of the stored columns bit for bit.  Oracle chains run
on host threads (the oracle's calls release the interpreter lock).
"""
import concurrent.futures as cf

import numpy as np
import pytest

import oracle_lib as O
from bayesrrcmd_gb300 import gpu

pytestmark = pytest.mark.gpu
S_C3 = [[0.01, 0.001, 0.0001], [0.1, 0.01]]
S1 = [[0.01, 0.001, 0.0001]]


def device_bed(torch, N, M, seed, lo, hi):
    d = torch.empty(M * ((N + 3) // 4), dtype=torch.uint8, device="cuda:0")
    gpu.synth_bed_device(d.data_ptr(), N, M, seed, lo, hi, 0.0)
    return d


def phenotypes(d_bed, N, M, specs, seed):
    """One phenotype per (n_causal, h2) spec: standardised causal columns
    times N(0, h2/n_causal) effects plus N(0, 1-h2) noise."""
    rng = np.random.default_rng(seed)
    probe = gpu.Chain(gpu.ChainConfig(N=N, M=M, S=S1))
    probe.pack_bed_device(d_bed.data_ptr(), d_bed.numel())
    ys = []
    for n_causal, h2 in specs:
        causal = np.sort(rng.choice(M, n_causal, replace=False)).astype(np.uint32)
        b = rng.normal(0.0, np.sqrt(h2 / n_causal), n_causal)
        ys.append((probe.xbeta(causal, b) + rng.normal(0.0, np.sqrt(1.0 - h2), N)).astype(np.float32))
    probe.close()
    return np.stack(ys)


def chain(d_bed, N, M, y, group, form, seed, **kw):
    ch = gpu.Chain(gpu.ChainConfig(N=N, M=M, S=S_C3, form=form, seed=seed,
                                   refresh_every=50 if form == gpu.FORM_FP32C else 0, **kw))
    ch.pack_bed_device(d_bed.data_ptr(), d_bed.numel())
    ch.set_groups(group)
    ch.set_phenotype(y)
    ch.init()
    return ch


def test_c3_size_plain_and_blocked_chains_match_oracle(gpu_lib):
    import torch
    N, M = 100_000, 10_000
    d_bed = device_bed(torch, N, M, 303, 0.01, 0.5)
    y = phenotypes(d_bed, N, M, [(100, 0.4)], 303)[0]
    group = (np.arange(M) >= M // 2).astype(np.int32)
    plain = chain(d_bed, N, M, y, group, gpu.FORM_FP64, 11)
    blocked = chain(d_bed, N, M, y, group, gpu.FORM_FP32C, 11, gram=1)
    assert blocked.gram_info()["blocked"]
    bed = d_bed.cpu().numpy().reshape(M, -1)
    del d_bed
    oc = O.OracleChain(bed, N, y, S_C3, kind=0, group=group, seed=11, dense_lut=True)
    for it in range(5):
        plain.iterate(1)
        blocked.iterate(1)
        oc.iterate(it)
        o = oc.state()
        nz = o["beta"] != 0
        assert nz.sum() > 50
        what = f"iteration {it}"
        s = plain.state()
        np.testing.assert_array_equal(s["comp"], o["comp"], err_msg=what)
        np.testing.assert_array_equal(s["beta"] != 0, nz, err_msg=what)
        np.testing.assert_allclose(s["beta"][nz], o["beta"][nz], rtol=1e-10, atol=1e-15, err_msg=what)
        np.testing.assert_allclose(s["sigmaE"], o["sigmaE"], rtol=1e-10, err_msg=what)
        np.testing.assert_allclose(s["sigmaG"], o["sigmaG"], rtol=1e-10, err_msg=what)
        np.testing.assert_allclose(s["mu"], o["mu"], rtol=1e-10, atol=1e-14, err_msg=what)
        np.testing.assert_allclose(s["eps"], o["eps"], rtol=0, atol=1e-10, err_msg=what)
        b = blocked.state()
        np.testing.assert_array_equal(b["comp"], o["comp"], err_msg=what)
        np.testing.assert_allclose(b["beta"][nz], o["beta"][nz], rtol=1e-9, atol=1e-13, err_msg=what)
        np.testing.assert_allclose(b["eps"], o["eps"], rtol=0, atol=1e-10, err_msg=what)
        np.testing.assert_allclose(b["sigmaG"], o["sigmaG"], rtol=1e-9, err_msg=what)
        np.testing.assert_allclose(b["sigmaE"], o["sigmaE"], rtol=1e-9, err_msg=what)
    plain.close()
    blocked.close()


def c4_compare(s, o, what):
    """Bars of the batched form at C4 size.  The residual is fixed point
    eps * 2^40 and every update coefficient is rounded to that grid, so each
    update leaves an error of up to 2^-41 per individual, coherent over the
    changed marker's genotype pattern; over the ~40,000 updates of a sweep at
    M = 200,000 the dot products move by up to ~2e-8, so betas carry an
    absolute error of a few 1e-13 (relative 1e-7 on the smallest non-zero
    betas, within the 1e-6 posterior-mean target).  Components identical,
    beta within 1e-9 relative or 1e-12 absolute, residual within 1e-9
    absolute, sigmaE and sigmaG within 1e-9 relative, acum within 2e-6
    relative (FP32 exponentials), mu within 1e-9 absolute (the constant part
    of every update is rounded once and moves the residual mean coherently by
    up to 2^-41: about 1e-10 after the sweeps' 40,000 updates)."""
    np.testing.assert_array_equal(s["comp"], o["comp"], err_msg=what)
    nz = o["beta"] != 0
    np.testing.assert_array_equal(s["beta"] != 0, nz, err_msg=what)
    d = {
        "beta": np.abs(s["beta"][nz] - o["beta"][nz]) - 1e-9 * np.abs(o["beta"][nz]) - 1e-12,
        "eps": np.abs(s["eps"] - o["eps"]) - 1e-9,
        "sigmaE": np.abs(s["sigmaE"] / o["sigmaE"] - 1) - 1e-9,
        "sigmaG": np.abs(np.asarray(s["sigmaG"]) / np.asarray(o["sigmaG"]) - 1) - 1e-9,
        "acum": np.abs(s["acum"] - o["acum"]) - 2e-6 * np.abs(o["acum"]) - 1e-12,
        "mu": np.abs(s["mu"] - o["mu"]) - 1e-9,
    }
    seen = {"beta_abs": float(np.abs(s["beta"][nz] - o["beta"][nz]).max()),
            "eps_abs": float(np.abs(s["eps"] - o["eps"]).max()),
            "sigmaE_rel": float(abs(s["sigmaE"] / o["sigmaE"] - 1)),
            "acum_abs": float(np.abs(s["acum"] - o["acum"]).max()), "mu_abs": float(abs(s["mu"] - o["mu"]))}
    bad = [k for k, v in d.items() if np.max(v) > 0]
    assert not bad, f"{what}: {bad} beyond the bars; observed {seen}"


def test_c4_size_batched_chains_match_oracle(gpu_lib):
    import torch
    N, M, C = 50_000, 200_000, 64
    seed = 404
    d_bed = device_bed(torch, N, M, seed, 0.01, 0.5)
    rng = np.random.default_rng(seed)
    ys = phenotypes(d_bed, N, M, [(1000, rng.uniform(0.1, 0.7)) for _ in range(C)], seed + 1)
    bt = gpu.Batch(gpu.ChainConfig(N=N, M=M, S=S1, seed=seed, chain=0), C)
    bt.pack_bed_device(d_bed.data_ptr(), d_bed.numel())
    bt.set_phenotypes(ys)
    bt.init()
    bed = d_bed.cpu().numpy().reshape(M, -1)
    del d_bed
    checked = (0, 31, 63)
    ocs = {c: O.OracleChain(bed, N, ys[c], S1, seed=seed, chain=c, perm_chain=0, dense_lut=True) for c in checked}
    with cf.ThreadPoolExecutor(len(checked)) as ex:
        for it in range(2):
            futs = [ex.submit(oc.iterate, it) for oc in ocs.values()]
            bt.iterate(1)
            for f in futs:
                f.result()
            for c, oc in ocs.items():
                o = oc.state()
                assert (o["beta"] != 0).sum() > 100
                c4_compare(bt.state(c), o, f"iteration {it} chain {c}")
    bt.close()
