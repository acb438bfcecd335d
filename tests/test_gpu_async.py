"""asyncppbayes on the GPU: the asynchronous schedule of the reference's
ParallelGraph (src/parallelgraph.cpp:51-150, src/BayesRBase.cpp:394-524) with
T markers in flight, against the FP64 oracle's restatement of that schedule.

Every marker of a batch of T consecutive sweep positions reads the residual
(and, for sparse markers, its running sum) before any of them writes; the
changes are then applied in sweep order and acum (P(component 0)) is left as
it was, as processColumnAsync never writes it.  The GPU sweep resolves each
batch in one grid round.  Bars of the drop-in: per iteration beta, sigmaG,
sigmaE and mu within 1e-10 relative, components identical, residual within
1e-11 absolute.
"""
import subprocess

import numpy as np
import pytest

import oracle_lib as O
from bayesrrcmd_gb300 import gpu, plink

pytestmark = pytest.mark.gpu
S2 = [[0.01, 0.001, 0.0001], [0.1, 0.01]]


@pytest.mark.parametrize("kind", [gpu.KIND_DENSE, gpu.KIND_RAGGED, gpu.KIND_EIGEN])
@pytest.mark.parametrize("T", [20, 7, 64])
def test_async_chain_matches_oracle_schedule(gpu_lib, kind, T):
    N, M = 1501, 400
    g, _ = plink.synth_genotypes(N, M, seed=61 + T, missing=0.01, p_lo=0.05)
    bed = plink.encode_bed(g)
    y, _, _ = plink.synth_phenotype(g, 61 + T, 12, 0.5)
    group = (np.arange(M) % 2).astype(np.int32)
    ch = gpu.Chain(gpu.ChainConfig(N=N, M=M, kind=kind, S=S2, seed=9, async_batch=T))
    ch.pack_bed(bed)
    ch.set_groups(group)
    ch.set_phenotype(y)
    ch.init()
    oc = O.OracleChain(bed, N, y, S2, kind=kind, group=group, seed=9, async_batch=T)
    for it in range(5):
        ch.iterate(1)
        oc.iterate(it)
        s, o = ch.state(), oc.state()
        what = f"iteration {it}"
        np.testing.assert_array_equal(s["comp"], o["comp"], err_msg=what)
        nz = o["beta"] != 0
        assert nz.sum() > 5
        np.testing.assert_array_equal(s["beta"] != 0, nz, err_msg=what)
        np.testing.assert_allclose(s["beta"][nz], o["beta"][nz], rtol=1e-10, atol=1e-15, err_msg=what)
        np.testing.assert_allclose(s["sigmaE"], o["sigmaE"], rtol=1e-10, err_msg=what)
        np.testing.assert_allclose(s["sigmaG"], o["sigmaG"], rtol=1e-10, err_msg=what)
        np.testing.assert_allclose(s["mu"], o["mu"], rtol=1e-10, atol=1e-14, err_msg=what)
        np.testing.assert_allclose(s["eps"], o["eps"], rtol=0, atol=1e-11, err_msg=what)
        np.testing.assert_array_equal(s["acum"], 0.0)
    assert ch.timing()[2] == -(-M // T)
    ch.close()


def test_async_configuration_is_checked(gpu_lib):
    for kw in (dict(async_batch=65), dict(async_batch=-1), dict(async_batch=8, form=gpu.FORM_FP32C)):
        with pytest.raises(gpu.BrrError) as e:
            gpu.Chain(gpu.ChainConfig(N=100, M=10, **kw))
        assert e.value.code == -1


def test_brr_asyncppbayes_end_to_end(gpu_lib, tmp_path):
    """brr --analysis-type asyncppbayes --analysis-tokens 9: the sample rows
    are the oracle's asynchronous chain (values as printed, 6 digits)."""
    from bayesrrcmd_gb300.build import build_cli
    brr = str(build_cli())
    N, M = 509, 120
    g, _ = plink.synth_genotypes(N, M, seed=4, missing=0.01)
    payload = plink.encode_bed(g)
    prefix = tmp_path / "toy"
    plink.write_plink(prefix, payload, N)
    y, _, _ = plink.synth_phenotype(g, 4, 6, 0.5)
    plink.write_phen(tmp_path / "toy.phen", y)
    out = tmp_path / "async.csv"
    r = subprocess.run([brr, "--analysis-type", "asyncppbayes", "--analysis-tokens", "9", "--bfile", str(prefix),
                        "--pheno", str(tmp_path / "toy.phen"), "--S", "0.01,0.001,0.0001", "--chain-length", "4",
                        "--burn-in", "0", "--thin", "1", "--seed", "11", "--mcmc-samples", str(out)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    yr = plink.read_phen(tmp_path / "toy.phen", plink.read_fam(prefix.with_suffix(".fam")))
    oc = O.OracleChain(payload, N, yr, [[0.01, 0.001, 0.0001]], kind=0, seed=11, async_batch=9)
    lines = out.read_text().splitlines()
    assert len(lines) == 1 + 4
    for it, line in enumerate(lines[1:]):
        oc.iterate(it)
        s = oc.state()
        v = np.array([float(t) for t in line.split(", ")])
        np.testing.assert_allclose(v[2:2 + M], s["beta"], rtol=1e-5, atol=1e-9)
        np.testing.assert_array_equal(v[4 + M:4 + 2 * M], s["comp"])
