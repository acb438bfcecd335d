"""Regenerate the committed golden fixtures of tests/golden/.

    python tests/golden/make_golden.py

1. uk10k_counts_digest.npz: per-marker genotype counts of the reference's
   uk10k fixture (test.zip:test/data/uk10k_chr1_1mb.bed, read from the
   reference checkout when it is mounted) decoded by the oracle; only column
   sums and the first 64 markers are stored.
2. synth_dense.npz / synth_ragged.npz / synth_eigen.npz: a small seeded
   synthetic problem (BED payload, phenotype, groups) with the oracle's packer
   outputs and the state after each of five Gibbs iterations.  All problems
   carry missing genotypes, N not a multiple of 4 or 64, and two groups with
   different component counts.
"""
from __future__ import annotations

import sys
import zipfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

import oracle_lib as O  # noqa: E402
from refdir import reference_dir  # noqa: E402
from bayesrrcmd_gb300 import plink  # noqa: E402

S2 = [[0.01, 0.001, 0.0001], [0.1, 0.01]]


def synth_problem(kind: int):
    N, M = 203, 61
    g, _ = plink.synth_genotypes(N, M, seed=20 + kind, missing=0.03, p_lo=0.02, p_hi=0.5)
    bed = plink.encode_bed(g)
    y, _, _ = plink.synth_phenotype(g, 20 + kind, 8, 0.5)
    group = (np.arange(M) % 3 == 0).astype(np.int32)
    return N, M, bed, y, group


def make_synth(kind: int, iters: int = 5):
    N, M, bed, y, group = synth_problem(kind)
    out = dict(N=N, M=M, bed=bed, y=y, group=group, counts=O.counts(bed, N), seed=77)
    if kind == 0:
        rc, t = O.marker_table_dense(bed, N)
    else:
        rc, t = O.ragged_stats(bed, N) if kind == 1 else O.eigen_stats(bed, N)
        for name, (off, idx) in zip(("ones", "twos", "miss"), O.ragged_lists(bed, N)):
            out[f"off_{name}"], out[f"idx_{name}"] = off, idx
    assert rc == 0
    out["table"] = t
    ch = O.OracleChain(bed, N, y, S2, kind=kind, group=group, seed=77)
    keys = ("beta", "comp", "acum", "sigmaE", "sigmaG", "mu", "pi")
    hist = {k: [] for k in keys}
    for it in range(iters):
        ch.iterate(it)
        s = ch.state()
        for k in keys:
            hist[k].append(s[k])
    for k in keys:
        out[f"trace_{k}"] = np.array(hist[k])
    out["eps_final"] = ch.state()["eps"]
    return out


def main():
    z = reference_dir() / "test.zip"
    if z.exists():
        raw = np.frombuffer(zipfile.ZipFile(z).read("test/data/uk10k_chr1_1mb.bed"), np.uint8)
        N, M = 3642, 6717
        c = O.counts(raw[3:].reshape(M, (N + 3) // 4), N)
        np.savez_compressed(HERE / "uk10k_counts_digest.npz", col_sums=c.sum(0), head=c[:64])
    np.savez_compressed(HERE / "synth_dense.npz", **make_synth(0))
    np.savez_compressed(HERE / "synth_ragged.npz", **make_synth(1))
    np.savez_compressed(HERE / "synth_eigen.npz", **make_synth(2))


if __name__ == "__main__":
    main()
