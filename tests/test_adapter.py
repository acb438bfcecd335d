"""The reference-interface adapter: GpuMarkerBuilder and GpuSweepGraph.

tests/adapter_harness.cpp stands in for the reference's BayesRBase: it keeps
the chain state in host vectors as the reference does, runs the runGibbs loop
body, and hands each sweep to GpuSweepGraph::exec through the
BayesRSweepAccess accessors; the markers reach the device through
GpuMarkerBuilder, fed with processAllele calls decoded from a PLINK .bed file
the way the reference's preprocess graph decodes it.  The chain it writes out
must be the FP64 oracle's chain: the drop-in forms at 1e-10 relative per
iteration with identical components, the Gram-blocked FP32C form at its bars.
"""
import subprocess
from pathlib import Path

import numpy as np
import pytest

import oracle_lib as O
from bayesrrcmd_gb300 import gpu, plink

ROOT = Path(__file__).resolve().parents[1]
HARNESS = ROOT / "bayesrrcmd_gb300" / "_build" / "adapter_harness"
S2 = [[0.01, 0.001, 0.0001], [0.1, 0.01]]


def build_harness() -> Path:
    from bayesrrcmd_gb300.build import LIBDIR, build_adapter
    build_adapter()
    src = ROOT / "tests" / "adapter_harness.cpp"
    deps = [src, *(ROOT / "bayesrrcmd_gb300" / "adapter").glob("*"), ROOT / "include" / "brr_gpu.h",
            ROOT / "bayesrrcmd_gb300" / "csrc" / "brr_stream.h"]
    if not HARNESS.exists() or any(d.stat().st_mtime > HARNESS.stat().st_mtime for d in deps):
        HARNESS.parent.mkdir(exist_ok=True)
        r = subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-o", str(HARNESS), str(src),
                            f"-I{ROOT / 'include'}", f"-L{LIBDIR}", "-lbrr_adapter", "-lbrr_gpu",
                            f"-Wl,-rpath,{LIBDIR}"], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
    return HARNESS


def test_adapter_builds_against_the_c_abi():
    """The adapter library and a reference-style driver compile and link
    against libbrr_gpu.so; the driver starts and checks its arguments."""
    h = build_harness()
    r = subprocess.run([str(h)], capture_output=True, text=True)
    assert r.returncode == 64 and "usage" in r.stderr


def run_harness(tmp_path, g, y, group, kind, form, gram, iters, seed):
    N = g.shape[1]
    M = g.shape[0]
    bed = tmp_path / "x.bed"
    bed.write_bytes(bytes([0x6C, 0x1B, 0x01]) + plink.encode_bed(g).tobytes())
    (tmp_path / "y.f32").write_bytes(np.ascontiguousarray(y, np.float32).tobytes())
    (tmp_path / "g.i32").write_bytes(np.ascontiguousarray(group, np.int32).tobytes())
    out = tmp_path / "trace.bin"
    spec = ";".join(",".join(repr(v) for v in row) for row in S2)
    r = subprocess.run([str(build_harness()), str(bed), str(tmp_path / "y.f32"), str(tmp_path / "g.i32"), str(N),
                        str(M), str(kind), str(form), str(gram), spec, str(seed), str(iters), str(out)],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    t = np.fromfile(out, np.float64)
    row = 2 * M + 1 + len(S2) + 1
    assert t.size == iters * row
    t = t.reshape(iters, row)
    return [dict(beta=t[i, :M], comp=t[i, M:2 * M].astype(np.int32), sigmaE=t[i, 2 * M],
                 sigmaG=t[i, 2 * M + 1:2 * M + 1 + len(S2)], mu=t[i, -1]) for i in range(iters)]


@pytest.mark.gpu
@pytest.mark.parametrize("kind,form,gram,rtol", [
    (gpu.KIND_DENSE, gpu.FORM_FP64, -1, 1e-10),
    (gpu.KIND_RAGGED, gpu.FORM_FP64, -1, 1e-10),
    (gpu.KIND_EIGEN, gpu.FORM_FP64, -1, 1e-10),
    (gpu.KIND_DENSE, gpu.FORM_FP32C, 1, 1e-9),
])
def test_adapter_chain_matches_oracle(gpu_lib, tmp_path, kind, form, gram, rtol):
    N, M, iters, seed = 1500, 400, 5, 13
    g, _ = plink.synth_genotypes(N, M, 77, missing=0.01, p_lo=0.05)
    y, _, _ = plink.synth_phenotype(g, 77, 12, 0.5)
    group = (np.arange(M) % 2).astype(np.int32)
    trace = run_harness(tmp_path, g, y, group, kind, form, gram, iters, seed)
    oc = O.OracleChain(plink.encode_bed(g), N, y, S2, kind=kind, group=group, seed=seed)
    for it in range(iters):
        oc.iterate(it)
        o, s = oc.state(), trace[it]
        what = f"iteration {it}"
        np.testing.assert_array_equal(s["comp"], o["comp"], err_msg=what)
        nz = o["beta"] != 0
        assert nz.sum() > 5
        np.testing.assert_array_equal(s["beta"] != 0, nz, err_msg=what)
        np.testing.assert_allclose(s["beta"][nz], o["beta"][nz], rtol=rtol, atol=1e-13, err_msg=what)
        np.testing.assert_allclose(s["sigmaE"], o["sigmaE"], rtol=rtol, err_msg=what)
        np.testing.assert_allclose(s["sigmaG"], o["sigmaG"], rtol=rtol, err_msg=what)
        np.testing.assert_allclose(s["mu"], o["mu"], rtol=rtol, atol=1e-14, err_msg=what)
