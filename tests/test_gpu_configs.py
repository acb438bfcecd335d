"""The reference-sized configurations as parity cases (GPU chains vs the oracle).

C1: plain dense BayesR, N = 2,000 x M = 5,000, p ~ U(0.05, 0.5), 100 causal
markers, S = 0.01,0.001,0.0001, a chain of 10 iterations, FP64 form.
C2: ragged sparse, N = 20,000 x M = 50,000, 70 % of the markers rare
(p ~ U(0.001, 0.05)), the rest p ~ U(0.05, 0.5), 1 % missing, 500 causal,
h2 = 0.5; the plain FP64 form and the FP32C form (FP64 refresh every 50
sweeps) against the oracle for the first iterations of the chain.
Genotypes are generated on the device (seeded); the phenotype from the
standardised causal columns.  Betas are compared at 1e-10 relative with an
absolute floor of 1e-15: among thousands of non-zero betas a few lie near 0
(beta = z sd + num / denom nearly cancelling), where a relative bar measures
the cancellation, not the chain.
"""
import numpy as np
import pytest

import oracle_lib as O
from bayesrrcmd_gb300 import gpu

pytestmark = pytest.mark.gpu
S1 = [[0.01, 0.001, 0.0001]]


def device_bed(torch, N, parts, seed, missing):
    """Concatenated synthetic BED payloads, one per (markers, p_lo, p_hi) part."""
    cb = (N + 3) // 4
    out = []
    for k, (m, lo, hi) in enumerate(parts):
        d = torch.empty(m * cb, dtype=torch.uint8, device="cuda:0")
        gpu.synth_bed_device(d.data_ptr(), N, m, seed + k, lo, hi, missing)
        out.append(d)
    return torch.cat(out)


def phenotype(d_bed, N, M, n_causal, h2, seed):
    rng = np.random.default_rng(seed)
    probe = gpu.Chain(gpu.ChainConfig(N=N, M=M, S=S1))
    probe.pack_bed_device(d_bed.data_ptr(), d_bed.numel())
    causal = np.sort(rng.choice(M, n_causal, replace=False)).astype(np.uint32)
    b = rng.normal(0.0, np.sqrt(h2 / n_causal), n_causal)
    gv = probe.xbeta(causal, b)
    probe.close()
    return (gv + rng.normal(0.0, np.sqrt(1.0 - h2), N)).astype(np.float32)


def chain(bed, N, M, y, kind, form, seed):
    ch = gpu.Chain(gpu.ChainConfig(N=N, M=M, kind=kind, form=form, S=S1, seed=seed,
                                   refresh_every=50 if form == gpu.FORM_FP32C else 0))
    ch.pack_bed(bed)
    ch.set_phenotype(y)
    ch.init()
    return ch


def test_c1_dense_fp64_chain_of_ten(gpu_lib):
    import torch
    N, M = 2000, 5000
    d_bed = device_bed(torch, N, [(M, 0.05, 0.5)], 101, 0.0)
    y = phenotype(d_bed, N, M, 100, 0.5, 101)
    bed = d_bed.cpu().numpy().reshape(M, -1)
    ch = chain(bed, N, M, y, gpu.KIND_DENSE, gpu.FORM_FP64, 5)
    oc = O.OracleChain(bed, N, y, S1, kind=0, seed=5)
    for it in range(10):
        ch.iterate(1)
        oc.iterate(it)
        s, o = ch.state(), oc.state()
        np.testing.assert_array_equal(s["comp"], o["comp"], err_msg=f"iteration {it}")
        nz = o["beta"] != 0
        np.testing.assert_allclose(s["beta"][nz], o["beta"][nz], rtol=1e-10, atol=1e-15, err_msg=f"iteration {it}")
        np.testing.assert_allclose([s["sigmaE"], s["sigmaG"][0]], [o["sigmaE"], o["sigmaG"][0]], rtol=1e-10)
    ch.close()


@pytest.mark.parametrize("form", [gpu.FORM_FP64, gpu.FORM_FP32C])
def test_c2_ragged_first_iterations(gpu_lib, form):
    import torch
    N, M = 20000, 50000
    rare = 35000
    d_bed = device_bed(torch, N, [(rare, 0.001, 0.05), (M - rare, 0.05, 0.5)], 202, 0.01)
    y = phenotype(d_bed, N, M, 500, 0.5, 202)
    bed = d_bed.cpu().numpy().reshape(M, -1)
    ch = chain(bed, N, M, y, gpu.KIND_RAGGED, form, 7)
    oc = O.OracleChain(bed, N, y, S1, kind=1, seed=7)
    for it in range(2):
        ch.iterate(1)
        oc.iterate(it)
        s, o = ch.state(), oc.state()
        np.testing.assert_array_equal(s["comp"], o["comp"], err_msg=f"iteration {it}")
        nz = o["beta"] != 0
        assert nz.sum() > 100
        if form == gpu.FORM_FP64:
            np.testing.assert_allclose(s["beta"][nz], o["beta"][nz], rtol=1e-10, atol=1e-15,
                                       err_msg=f"iteration {it}")
            np.testing.assert_allclose(s["eps"], o["eps"], rtol=0, atol=1e-11)
        else:
            np.testing.assert_allclose(s["beta"][nz], o["beta"][nz], rtol=1e-7, atol=1e-12, err_msg=f"iteration {it}")
            np.testing.assert_allclose(s["eps"], o["eps"], rtol=0, atol=1e-9)
        np.testing.assert_allclose(s["sigmaE"], o["sigmaE"], rtol=1e-8)
    ch.close()
