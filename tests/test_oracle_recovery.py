"""Statistical recovery of the reference's two-group simulation by the oracle.

The reference ships a simulated two-group data set with its truth
(test.groups/: phenotype, marker groups, mixture sizes `0.001,0.01;0.001,0.01`,
true genetic variances in true.var.txt = total, group 1, group 2, and the 100
causal markers with their effects in true.effects.txt) on the genotypes of its
uk10k fixture (test.zip:test/data/uk10k_chr1_1mb.bed, the same .bim).  Its own
group test never runs on these files (test/ppbayestest.cpp:229-238 instantiates
the ungrouped fixture), and its check script only prints sigmaG
(test.groups/check.output.R).  Here the FP64 oracle chain (the restatement the
GPU kernels are checked against) runs 400 iterations with 100 of burn-in and
must recover the truth: per-group posterior-mean sigmaG (scaled back by the
phenotype variance, since the chain standardises y) within 25 % and within 3
posterior standard deviations of the true variance, the total within 20 %,
causal markers included at least 5 times as often as the others, and the
posterior-mean effects of the causal markers correlated at least 0.6 with
the true effects.
"""
import zipfile
from pathlib import Path

import numpy as np
import pytest

import oracle_lib as O
from refdir import reference_dir

REF = reference_dir()
GROUPS = REF / "test.groups"


def _load():
    z = REF / "test.zip"
    if not z.exists() or not GROUPS.exists():
        pytest.skip("reference fixtures not mounted")
    raw = np.frombuffer(zipfile.ZipFile(z).read("test/data/uk10k_chr1_1mb.bed"), np.uint8)
    N, M = 3642, 6717
    bed = np.ascontiguousarray(raw[3:].reshape(M, (N + 3) // 4))
    bim = [ln.split()[1] for ln in (GROUPS / "uk10k_chr1_1mb.bim").read_text().splitlines()]
    assert bim == [ln.split()[1] for ln in (REF / "test/data/uk10k_chr1_1mb.bim").read_text().splitlines()]
    fam = [ln.split()[:2] for ln in (GROUPS / "uk10k_chr1_1mb.fam").read_text().splitlines()]
    phen = [ln.split() for ln in (GROUPS / "test.phen").read_text().splitlines()[1:] if ln.strip()]
    assert [p[:2] for p in phen] == fam
    y = np.array([float(p[2]) for p in phen], np.float32)
    grp = [ln.split() for ln in (GROUPS / "test.group").read_text().splitlines() if ln.strip()]
    assert [g[0] for g in grp] == bim
    group = np.array([int(g[1]) for g in grp], np.int32)
    S = [[float(v) for v in part.split(",")] for part in (GROUPS / "test.cva").read_text().strip().split(";")]
    true_var = np.loadtxt(GROUPS / "true.var.txt")
    eff = [ln.split() for ln in (GROUPS / "true.effects.txt").read_text().splitlines()[1:] if ln.strip()]
    where = {s: j for j, s in enumerate(bim)}
    causal = np.array([where[e[0]] for e in eff])
    effect = np.array([float(e[1]) for e in eff])
    return bed, N, M, y, group, S, true_var, causal, effect


def test_two_group_simulation_is_recovered():
    bed, N, M, y, group, S, true_var, causal, effect = _load()
    assert S == [[0.001, 0.01], [0.001, 0.01]]
    iters, burn = 400, 100
    oc = O.OracleChain(bed, N, y, S, kind=0, group=group, seed=1)
    sg, beta, incl = [], np.zeros(M), np.zeros(M)
    for it in range(iters):
        oc.iterate(it)
        if it >= burn:
            s = oc.state()
            sg.append(s["sigmaG"].copy())
            beta += s["beta"]
            incl += s["beta"] != 0
    kept = iters - burn
    vy = float(np.var(y.astype(np.float64), ddof=1))
    sg = np.array(sg) * vy
    mean, sd = sg.mean(0), sg.std(0)
    for g in range(2):
        truth = true_var[1 + g]
        assert abs(mean[g] - truth) <= 0.25 * truth, (g, mean[g], truth)
        assert abs(mean[g] - truth) <= 3.0 * sd[g], (g, mean[g], sd[g], truth)
    assert abs(mean.sum() - true_var[0]) <= 0.20 * true_var[0]
    pip = incl / kept
    others = np.delete(pip, causal)
    assert pip[causal].mean() >= 5.0 * others.mean()
    assert np.corrcoef(beta[causal] / kept, effect)[0, 1] >= 0.6
