"""The C-ABI library loads, exports every declared entry point, and its
structures have the layout the ctypes binding assumes (no GPU needed)."""
import ctypes as C
import re
import subprocess
from pathlib import Path

import pytest

from bayesrrcmd_gb300 import gpu
from bayesrrcmd_gb300.build import build_gpu

ROOT = Path(__file__).resolve().parents[1]
HEADERS = sorted((ROOT / "include").glob("*.h"))


def declared_functions():
    names = []
    for h in HEADERS:
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(brr_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_library_builds_and_exports_all_declared_symbols():
    lib_path = build_gpu()
    lib = C.CDLL(str(lib_path))
    names = declared_functions()
    assert len(names) >= 16
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert set(gpu.EXPORTS) <= set(names)


def test_struct_layout_matches_header(tmp_path):
    src = tmp_path / "layout.c"
    src.write_text(
        '#include <stdio.h>\n#include <stddef.h>\n#include "brr_gpu.h"\n'
        "int main(void){printf(\"%zu %zu %zu %zu %zu %zu %zu\\n\", sizeof(brr_config), offsetof(brr_config, S),"
        " offsetof(brr_config, seed), offsetof(brr_config, device), sizeof(brr_state), offsetof(brr_state, iteration),"
        " sizeof(brr_sweep_out)); return 0;}\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", str(ROOT / "include"), "-o", str(exe), str(src)], check=True)
    vals = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    assert vals == [C.sizeof(gpu.BrrConfig), gpu.BrrConfig.S.offset, gpu.BrrConfig.seed.offset,
                    gpu.BrrConfig.device.offset, C.sizeof(gpu.BrrState), gpu.BrrState.iteration.offset,
                    C.sizeof(gpu.BrrSweepOut)]


def test_errors_without_gpu_are_reported_not_crashing():
    """On a host without an sm_103 device, context creation fails with a status."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    lib = gpu.load_library()
    cfg = gpu.ChainConfig(N=10, M=5).to_c()
    h = C.c_void_p()
    rc = lib.brr_ctx_create(C.byref(cfg), C.byref(h))
    assert rc == -8 and lib.brr_last_error()


def test_invalid_config_rejected():
    lib = gpu.load_library()
    h = C.c_void_p()
    bad = gpu.ChainConfig(N=1, M=5).to_c()
    assert lib.brr_ctx_create(C.byref(bad), C.byref(h)) == -1
    bad = gpu.ChainConfig(N=10, M=5, S=[[0.1, -1.0]]).to_c()
    assert lib.brr_ctx_create(C.byref(bad), C.byref(h)) == -1
    bad = gpu.ChainConfig(N=10, M=5, spec_width=12).to_c()
    assert lib.brr_ctx_create(C.byref(bad), C.byref(h)) == -1
    # the cluster sweep: 2..16 CTAs, and it is the restart sweep
    for kw in (dict(cluster=1), dict(cluster=17), dict(cluster=-2), dict(cluster=8, gram=1)):
        bad = gpu.ChainConfig(N=10, M=5, **kw).to_c()
        assert lib.brr_ctx_create(C.byref(bad), C.byref(h)) == -1, kw
        assert b"cluster" in lib.brr_last_error()


def test_batch_config_rejected_before_the_device():
    """The batched form checks its arguments before it looks for a GPU."""
    lib = gpu.load_library()
    h = C.c_void_p()
    cfg = gpu.ChainConfig(N=100, M=5).to_c()
    assert lib.brr_batch_create(C.byref(cfg), 48, C.byref(h)) == -1          # 32 or 64 chains
    assert b"32 or 64" in lib.brr_last_error()
    rag = gpu.ChainConfig(N=100, M=5, kind=gpu.KIND_RAGGED).to_c()
    assert lib.brr_batch_create(C.byref(rag), 64, C.byref(h)) == -1          # dense markers only
    bad = gpu.ChainConfig(N=100, M=5, S=[[0.1, 0.0]]).to_c()
    assert lib.brr_batch_create(C.byref(bad), 64, C.byref(h)) == -1


def test_batch_without_gpu_is_a_device_error():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    lib = gpu.load_library()
    h = C.c_void_p()
    cfg = gpu.ChainConfig(N=100, M=5).to_c()
    assert lib.brr_batch_create(C.byref(cfg), 64, C.byref(h)) == -8


def test_multi_config_rejected_before_the_device():
    lib = gpu.load_library()
    h = C.c_void_p()
    one = (gpu.BrrConfig * 1)(gpu.ChainConfig(N=100, M=5).to_c())
    assert lib.brr_multi_create(one, 0, C.byref(h)) == -1
    assert lib.brr_multi_create(one, 33, C.byref(h)) == -1
    mixed = (gpu.BrrConfig * 2)(gpu.ChainConfig(N=100, M=5).to_c(),
                                gpu.ChainConfig(N=100, M=5, form=gpu.FORM_FP32C).to_c())
    assert lib.brr_multi_create(mixed, 2, C.byref(h)) == -1
    assert b"sweep form" in lib.brr_last_error()
