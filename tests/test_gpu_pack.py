"""Device packer vs the oracle: bit-exact counts, tables and ragged indices."""
from pathlib import Path

import numpy as np
import pytest

import oracle_lib as O
from bayesrrcmd_gb300 import gpu, plink

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"

SHAPES = [
    (4, 3, 0.0),        # one byte per column
    (5, 2, 0.0),        # ragged last byte
    (63, 7, 0.05),      # just under one chunk
    (64, 9, 0.0),       # exactly one chunk
    (65, 11, 0.1),      # one chunk plus one individual
    (1003, 37, 0.01),
    (4099, 5, 0.02),    # many slices, few markers
]


def bits(a):
    return np.ascontiguousarray(a).view(np.uint64)


@pytest.mark.parametrize("N,M,miss", SHAPES)
@pytest.mark.parametrize("kind", [gpu.KIND_DENSE, gpu.KIND_RAGGED, gpu.KIND_EIGEN])
def test_pack_bit_exact(gpu_lib, N, M, miss, kind):
    g, _ = plink.synth_genotypes(N, M, seed=N * 7 + M, missing=miss, p_lo=0.01)
    bed = plink.encode_bed(g)
    with gpu.Chain(gpu.ChainConfig(N=N, M=M, kind=kind)) as ch:
        ch.pack_bed(bed)
        t, n = ch.marker_table()
        np.testing.assert_array_equal(n, O.counts(bed, N))
        if kind == gpu.KIND_DENSE:
            rc, ref = O.marker_table_dense(bed, N)
        else:
            rc, ref = O.ragged_stats(bed, N) if kind == gpu.KIND_RAGGED else O.eigen_stats(bed, N)
            for (go, gi), (oo, oi) in zip(ch.ragged_lists(n), O.ragged_lists(bed, N)):
                np.testing.assert_array_equal(go, oo)
                np.testing.assert_array_equal(gi, oi)
        assert rc == 0
        assert np.array_equal(bits(t), bits(ref))


NAMES = {0: "synth_dense.npz", 1: "synth_ragged.npz", 2: "synth_eigen.npz"}


@pytest.mark.parametrize("kind", [0, 1, 2])
def test_pack_matches_committed_golden(gpu_lib, kind):
    d = dict(np.load(GOLDEN / NAMES[kind]))
    N, M = int(d["N"]), int(d["M"])
    with gpu.Chain(gpu.ChainConfig(N=N, M=M, kind=kind)) as ch:
        ch.pack_bed(d["bed"])
        t, n = ch.marker_table()
        np.testing.assert_array_equal(n, d["counts"])
        assert np.array_equal(bits(t), bits(d["table"]))
        if kind != 0:
            for name, (go, gi) in zip(("ones", "twos", "miss"), ch.ragged_lists(n)):
                np.testing.assert_array_equal(go, d[f"off_{name}"])
                np.testing.assert_array_equal(gi, d[f"idx_{name}"])


@pytest.mark.parametrize("grid", [1, 3, 16])
def test_pack_independent_of_grid(gpu_lib, grid):
    N, M = 2000, 23
    g, _ = plink.synth_genotypes(N, M, seed=5, missing=0.02)
    bed = plink.encode_bed(g)
    with gpu.Chain(gpu.ChainConfig(N=N, M=M, kind=gpu.KIND_RAGGED, grid=grid)) as ch:
        ch.pack_bed(bed)
        t, n = ch.marker_table()
        for (go, gi), (oo, oi) in zip(ch.ragged_lists(n), O.ragged_lists(bed, N)):
            np.testing.assert_array_equal(gi, oi)


def test_monomorphic_marker_is_an_error(gpu_lib):
    g = np.zeros((3, 100), np.int8)
    g[0, :50] = 1
    g[2, 3] = 2
    bed = plink.encode_bed(g)
    for kind in (0, 1, 2):
        with gpu.Chain(gpu.ChainConfig(N=100, M=3, kind=kind)) as ch:
            with pytest.raises(gpu.BrrError) as e:
                ch.pack_bed(bed)
            assert e.value.code == -5 and "marker 1" in str(e.value)


def test_wrong_payload_size_is_an_error(gpu_lib):
    with gpu.Chain(gpu.ChainConfig(N=100, M=3)) as ch:
        with pytest.raises(gpu.BrrError) as e:
            ch.pack_bed(np.zeros(10, np.uint8))
        assert e.value.code == -1
