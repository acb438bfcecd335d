"""The oracle reproduces the committed golden fixtures bit for bit (CPU)."""
from pathlib import Path

import numpy as np
import pytest

import oracle_lib as O

GOLDEN = Path(__file__).resolve().parent / "golden"
S2 = [[0.01, 0.001, 0.0001], [0.1, 0.01]]


NAMES = {0: "synth_dense.npz", 1: "synth_ragged.npz", 2: "synth_eigen.npz"}


def load(kind):
    return dict(np.load(GOLDEN / NAMES[kind]))


@pytest.mark.parametrize("kind", [0, 1, 2])
def test_oracle_reproduces_golden(kind):
    d = load(kind)
    N, bed = int(d["N"]), d["bed"]
    np.testing.assert_array_equal(O.counts(bed, N), d["counts"])
    if kind == 0:
        rc, t = O.marker_table_dense(bed, N)
    else:
        rc, t = O.ragged_stats(bed, N) if kind == 1 else O.eigen_stats(bed, N)
        for name, (off, idx) in zip(("ones", "twos", "miss"), O.ragged_lists(bed, N)):
            np.testing.assert_array_equal(off, d[f"off_{name}"])
            np.testing.assert_array_equal(idx, d[f"idx_{name}"])
    assert rc == 0
    assert np.array_equal(t.view(np.uint64), d["table"].view(np.uint64))
    ch = O.OracleChain(bed, N, d["y"], S2, kind=kind, group=d["group"], seed=int(d["seed"]))
    for it in range(d["trace_beta"].shape[0]):
        ch.iterate(it)
        s = ch.state()
        np.testing.assert_array_equal(s["beta"], d["trace_beta"][it])
        np.testing.assert_array_equal(s["comp"], d["trace_comp"][it])
        assert s["sigmaE"] == d["trace_sigmaE"][it]
        np.testing.assert_array_equal(s["sigmaG"], d["trace_sigmaG"][it])
        assert s["mu"] == d["trace_mu"][it]


def test_dense_lut_storage_equals_column_storage():
    """The compact dense storage (four values per marker, codes read from the
    BED payload) gives the same chain bit for bit as the stored columns."""
    d = dict(np.load(GOLDEN / "synth_dense.npz"))
    N = int(d["N"])
    S = [[0.01, 0.001, 0.0001], [0.1, 0.01]]
    a = O.OracleChain(d["bed"], N, d["y"], S, kind=0, group=d["group"], seed=int(d["seed"]))
    b = O.OracleChain(d["bed"], N, d["y"], S, kind=0, group=d["group"], seed=int(d["seed"]), dense_lut=True)
    for it in range(4):
        a.iterate(it)
        b.iterate(it)
        sa, sb = a.state(), b.state()
        for k in ("beta", "comp", "eps", "acum", "sigmaG"):
            np.testing.assert_array_equal(sa[k], sb[k])
        assert sa["sigmaE"] == sb["sigmaE"] and sa["mu"] == sb["mu"]
