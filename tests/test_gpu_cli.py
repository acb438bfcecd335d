"""`brr` end to end on the GPU: preprocess files and a ppbayes run.

The ppbayes sample file has 1 + ceil(chain/thin) lines (the reference's
smoke invariant, test/ppbayestest.cpp:138-149) and its rows hold the same
chain as the oracle (values as printed with 6 significant digits).
"""
import subprocess
from pathlib import Path

import numpy as np
import pytest

import oracle_lib as O
from bayesrrcmd_gb300 import plink
from bayesrrcmd_gb300.build import build_cli

pytestmark = pytest.mark.gpu
S2 = [[0.01, 0.001, 0.0001], [0.1, 0.01]]


@pytest.fixture(scope="module")
def brr(gpu_lib):
    return str(build_cli())


@pytest.fixture
def dataset(tmp_path):
    N, M = 509, 120
    g, _ = plink.synth_genotypes(N, M, seed=4, missing=0.01)
    payload = plink.encode_bed(g)
    prefix = tmp_path / "toy"
    plink.write_plink(prefix, payload, N)
    y, _, _ = plink.synth_phenotype(g, 4, 6, 0.5)
    plink.write_phen(tmp_path / "toy.phen", y)
    group = (np.arange(M) % 2).astype(np.int32)
    plink.write_groups(tmp_path / "toy.group", group)
    return dict(N=N, M=M, g=g, payload=payload, prefix=prefix, y=plink.read_phen(tmp_path / "toy.phen",
                plink.read_fam(prefix.with_suffix(".fam"))), group=group, dir=tmp_path)


def run(brr, *args):
    r = subprocess.run([brr, *args], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    return r.stdout


@pytest.mark.parametrize("sparse", [None, "ragged", "eigen"])
def test_preprocess_writes_reference_formats(brr, dataset, sparse):
    d = dataset
    args = ["--preprocess", "--bfile", str(d["prefix"]), "--pheno", str(d["dir"] / "toy.phen")]
    if sparse:
        args += ["--sparse-data", sparse]
    run(brr, *args)
    N, M = d["N"], d["M"]
    if sparse is None:
        data = np.fromfile(d["dir"] / "toy.ppbed", np.float64).reshape(M, N)
        idx = np.fromfile(d["dir"] / "toy.ppbedindex", np.uint64).reshape(M, 3)
        np.testing.assert_array_equal(data, O.dense_columns(d["payload"], N))
        np.testing.assert_array_equal(idx[:, 0], np.arange(M) * N * 8)
        np.testing.assert_array_equal(idx[:, 1], N * 8)
    elif sparse == "eigen":
        import test_cli_preprocessed as P
        got = (d["dir"] / "toy.eigen.sparsebed").read_bytes()
        got_idx = (d["dir"] / "toy.eigen.sparsebedindex").read_bytes()
        ref = d["dir"] / "ref"
        P.write_eigen(ref, d["payload"], N)
        assert got == (d["dir"] / "ref.eigen.sparsebed").read_bytes()
        assert got_idx == (d["dir"] / "ref.eigen.sparsebedindex").read_bytes()
    else:
        raw = (d["dir"] / "toy.ragged.sparsebed").read_bytes()
        idx = np.fromfile(d["dir"] / "toy.ragged.sparsebedindex", np.uint64).reshape(M, 3)
        rc, st = O.ragged_stats(d["payload"], N)
        lists = O.ragged_lists(d["payload"], N)
        for j in range(M):
            pos = int(idx[j, 0])
            stats = np.frombuffer(raw, np.float64, 4, pos)
            np.testing.assert_array_equal(stats, st[j])
            pos += 32
            for off, ix in lists:
                n = int(np.frombuffer(raw, np.uint64, 1, pos)[0])
                pos += 8
                got = np.frombuffer(raw, np.int32, n, pos)
                pos += 4 * n
                np.testing.assert_array_equal(got, ix[off[j]:off[j + 1]])
            assert pos == int(idx[j, 0] + idx[j, 1])


@pytest.mark.parametrize("chain,thin,burn", [(10, 1, 0), (7, 3, 0), (6, 2, 2)])
def test_ppbayes_sample_file(brr, dataset, chain, thin, burn):
    d = dataset
    out = d["dir"] / "samples.csv"
    run(brr, "--analysis-type", "ppbayes", "--bfile", str(d["prefix"]), "--pheno", str(d["dir"] / "toy.phen"),
        "--group", str(d["dir"] / "toy.group"), "--S", "0.01,0.001,0.0001;0.1,0.01",
        "--chain-length", str(chain), "--burn-in", str(burn), "--thin", str(thin), "--seed", "11",
        "--mcmc-samples", str(out))
    lines = out.read_text().splitlines()
    kept = [it for it in range(chain) if it >= burn and it % thin == 0]
    assert len(lines) == 1 + len(kept)
    if burn == 0:
        assert len(lines) == 1 + int(np.ceil(chain / thin))
    M, N = d["M"], d["N"]
    header = lines[0].split(",")
    assert header[:3] == ["iteration", "mu", "beta[1]"] and header[-1] == f"epsilon[{N}]"
    assert len(header) == 2 + M + 1 + 2 + M + M + N
    oc = O.OracleChain(d["payload"], N, d["y"], S2, kind=0, group=d["group"], seed=11)
    rows = {}
    for it in range(chain):
        oc.iterate(it)
        if it in kept:
            rows[it] = oc.state()
    for line in lines[1:]:
        v = np.array([float(t) for t in line.split(", ")])
        it = int(v[0])
        s = rows[it]
        np.testing.assert_allclose(v[1], s["mu"], rtol=1e-5, atol=1e-6)
        np.testing.assert_allclose(v[2:2 + M], s["beta"], rtol=1e-5, atol=1e-9)
        np.testing.assert_allclose(v[2 + M], s["sigmaE"], rtol=1e-5)
        np.testing.assert_array_equal(v[5 + M:5 + 2 * M], s["comp"])


def test_ppbayes_missing_phenotypes_are_an_error(brr, dataset):
    d = dataset
    phen = d["dir"] / "toy.phen"
    lines = phen.read_text().splitlines()
    t = lines[3].split()
    lines[3] = f"{t[0]} {t[1]} NA"
    phen.write_text("\n".join(lines) + "\n")
    r = subprocess.run([brr, "--analysis-type", "ppbayes", "--bfile", str(d["prefix"]), "--pheno", str(phen),
                        "--chain-length", "2", "--mcmc-samples", str(d["dir"] / "x.csv")],
                       capture_output=True, text=True)
    assert r.returncode == 1 and "phenotype" in r.stderr


@pytest.mark.parametrize("sparse", [None, "ragged", "eigen"])
def test_ppbayes_reads_reference_preprocessed_files(brr, dataset, sparse):
    """With <prefix>.ppbed / .ragged.sparsebed / .eigen.sparsebed and its index present, ppbayes
    reads them as the reference does (src/analysisrunner.cpp:186-196): files
    written in the reference's layout from the oracle's builders give the
    oracle's chain."""
    import test_cli_preprocessed as P
    d = dataset
    if sparse is None:
        P.write_dense(d["prefix"], d["payload"], d["N"])
        extra = []
    elif sparse == "eigen":
        P.write_eigen(d["prefix"], d["payload"], d["N"])
        extra = ["--sparse-data", "eigen"]
    else:
        P.write_ragged(d["prefix"], d["payload"], d["N"])
        extra = ["--sparse-data", "ragged"]
    out = d["dir"] / "samples_pp.csv"
    log = run(brr, "--analysis-type", "ppbayes", "--bfile", str(d["prefix"]), "--pheno", str(d["dir"] / "toy.phen"),
              "--group", str(d["dir"] / "toy.group"), "--S", "0.01,0.001,0.0001;0.1,0.01",
              "--chain-length", "4", "--burn-in", "0", "--thin", "1", "--seed", "11",
              "--mcmc-samples", str(out), *extra)
    assert "Start reading preprocessed bed file" in log
    M, N = d["M"], d["N"]
    kind = {None: 0, "ragged": 1, "eigen": 2}[sparse]
    oc = O.OracleChain(d["payload"], N, d["y"], S2, kind=kind, group=d["group"], seed=11)
    lines = out.read_text().splitlines()
    for it, line in enumerate(lines[1:]):
        oc.iterate(it)
        s = oc.state()
        v = np.array([float(t) for t in line.split(", ")])
        np.testing.assert_allclose(v[2:2 + M], s["beta"], rtol=1e-5, atol=1e-9)
        np.testing.assert_array_equal(v[5 + M:5 + 2 * M], s["comp"])


def test_ppbayes_eigen_marker_with_mean_one(brr, dataset):
    """A marker whose genotype sum is N stores its missing genotypes as 1.0,
    like heterozygotes; the chain read from the Eigen file is the oracle's
    chain on the original genotypes."""
    import test_cli_preprocessed as P
    d = dataset
    N, M = d["N"], d["M"]
    g = d["g"].copy()
    row = np.zeros(N, np.int8)
    perm = np.random.default_rng(7).permutation(N)
    row[perm[:200]] = 2
    row[perm[200:309]] = 1            # 2*200 + 109 = 509 = N
    row[perm[309:319]] = -1
    g[7] = row
    payload = plink.encode_bed(g)
    plink.write_plink(d["prefix"], payload, N)
    stats = P.write_eigen(d["prefix"], payload, N)
    assert stats[7, 0] == 1.0
    out = d["dir"] / "samples_mean1.csv"
    run(brr, "--analysis-type", "ppbayes", "--bfile", str(d["prefix"]), "--pheno", str(d["dir"] / "toy.phen"),
        "--group", str(d["dir"] / "toy.group"), "--S", "0.01,0.001,0.0001;0.1,0.01",
        "--chain-length", "4", "--burn-in", "0", "--thin", "1", "--seed", "11",
        "--mcmc-samples", str(out), "--sparse-data", "eigen")
    oc = O.OracleChain(payload, N, d["y"], S2, kind=2, group=d["group"], seed=11)
    for it, line in enumerate(out.read_text().splitlines()[1:]):
        oc.iterate(it)
        s = oc.state()
        v = np.array([float(t) for t in line.split(", ")])
        np.testing.assert_allclose(v[2:2 + M], s["beta"], rtol=1e-5, atol=1e-9)
        np.testing.assert_array_equal(v[5 + M:5 + 2 * M], s["comp"])


def test_ppbayes_column_log(brr, dataset):
    """--colLog runs the phase-counting sweep variant and writes one row of its
    16 counters per iteration (the GPU counterpart of the reference's
    per-column timing log, src/BayesRBase.cpp:381-389); the chain, and so the
    sample file, is the same as without the log."""
    d = dataset
    chain = 4
    common = ["--analysis-type", "ppbayes", "--bfile", str(d["prefix"]), "--pheno", str(d["dir"] / "toy.phen"),
              "--chain-length", str(chain), "--burn-in", "0", "--thin", "1", "--seed", "3"]
    logged, plain, cols = d["dir"] / "logged.csv", d["dir"] / "plain.csv", d["dir"] / "cols.csv"
    run(brr, *common, "--mcmc-samples", str(logged), "--colLog", str(cols))
    run(brr, *common, "--mcmc-samples", str(plain))
    assert logged.read_text() == plain.read_text()
    rows = cols.read_text().splitlines()
    assert rows[0].split(",") == ["iter"] + [f"phase{k}" for k in range(16)]
    v = np.array([[int(t) for t in r.split(",")] for r in rows[1:]])
    assert v.shape == (chain, 17)
    np.testing.assert_array_equal(v[:, 0], np.arange(chain))
    assert (v[:, 1 + 5] > 0).all() and (v[:, 1 + 3] > 0).all()   # grid rounds, sampling cycles
