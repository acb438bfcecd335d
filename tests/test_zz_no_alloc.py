"""brr_xbeta_noalloc, the allocation-free genetic-value entry point, against
brr_xbeta.

It exists for callers that cannot allocate device memory when they need the
values (a runtime that owns the GPU through its own pool, a serving loop that
must not block on the allocator): the term list is staged in a fixed static
device array and the result goes to a buffer the caller owns.  The test owns
the output buffer (allocated with torch), calls the entry point twice in a
row with different term lists through the C ABI and compares each result with
brr_xbeta on the same context; further tests check that repeated calls leave
the device's free memory unchanged, that an output buffer the kernel could not
write in full is refused before any launch, and (on the CPU) that the
entry point's source names no allocating call.  This file is collected last.
"""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from bayesrrcmd_gb300 import gpu, plink

RTOL = 1e-12
CSRC = Path(__file__).resolve().parents[1] / "bayesrrcmd_gb300" / "csrc"


def _ptr(a, ct):
    return a.ctypes.data_as(C.POINTER(ct))


def _call(lib, ch, idx, b, d_out):
    return lib.brr_xbeta_noalloc(ch.h, _ptr(idx, C.c_uint32), _ptr(b, C.c_double), len(idx), C.c_void_p(d_out))


@pytest.mark.gpu
@pytest.mark.parametrize("kind", [gpu.KIND_DENSE, gpu.KIND_RAGGED, gpu.KIND_EIGEN])
def test_noalloc_matches_allocating_entry_point_on_two_calls(gpu_lib, kind):
    import torch
    N, M = 3001, 257
    g, _ = plink.synth_genotypes(N, M, seed=99, missing=0.02)
    lib = gpu_lib
    with gpu.Chain(gpu.ChainConfig(N=N, M=M, kind=kind, device=0), lib=lib) as ch:
        ch.pack_bed(plink.encode_bed(g))
        out = torch.full((N,), float("nan"), dtype=torch.float64, device="cuda:0")
        rng = np.random.default_rng(kind)
        for call, n in enumerate((37, 200)):
            idx = np.ascontiguousarray(rng.choice(M, n, replace=False), np.uint32)
            b = np.ascontiguousarray(rng.normal(0.0, 0.1, n), np.float64)
            ref = ch.xbeta(idx, b)
            rc = _call(lib, ch, idx, b, out.data_ptr())
            assert rc == 0, lib.brr_last_error().decode()
            torch.cuda.synchronize()
            np.testing.assert_allclose(out.cpu().numpy(), ref, rtol=RTOL, atol=1e-15,
                                       err_msg=f"call {call}")


@pytest.mark.gpu
def test_noalloc_calls_leave_free_device_memory_unchanged(gpu_lib):
    import torch
    N, M = 5000, 300
    g, _ = plink.synth_genotypes(N, M, seed=5)
    lib = gpu_lib
    with gpu.Chain(gpu.ChainConfig(N=N, M=M, device=0), lib=lib) as ch:
        ch.pack_bed(plink.encode_bed(g))
        out = torch.zeros(N, dtype=torch.float64, device="cuda:0")
        rng = np.random.default_rng(11)
        idx = np.ascontiguousarray(rng.choice(M, 120, replace=False), np.uint32)
        b = np.ascontiguousarray(rng.normal(0.0, 0.1, 120), np.float64)
        assert _call(lib, ch, idx, b, out.data_ptr()) == 0, lib.brr_last_error().decode()
        torch.cuda.synchronize()
        free0, _ = torch.cuda.mem_get_info()
        for _ in range(20):
            assert _call(lib, ch, idx, b, out.data_ptr()) == 0, lib.brr_last_error().decode()
        torch.cuda.synchronize()
        free1, _ = torch.cuda.mem_get_info()
        assert free1 == free0


@pytest.mark.gpu
def test_noalloc_refuses_output_it_cannot_write_in_full(gpu_lib):
    """Host memory, and a device pointer with fewer than N doubles to the end
    of its allocation, are refused with BRR_ERR_ARG and nothing is launched
    (the buffer's bytes past the pointer are left as they were)."""
    import torch
    N, M = 1000, 20
    g, _ = plink.synth_genotypes(N, M, seed=8)
    lib = gpu_lib
    idx = np.arange(5, dtype=np.uint32)
    b = np.full(5, 0.3)
    with gpu.Chain(gpu.ChainConfig(N=N, M=M, device=0), lib=lib) as ch:
        ch.pack_bed(plink.encode_bed(g))
        host = np.zeros(N, np.float64)
        assert _call(lib, ch, idx, b, host.ctypes.data) == -1
        assert "device or managed" in lib.brr_last_error().decode()
        assert _call(lib, ch, idx, b, 8) == -1
        buf = torch.full((4 * N,), 7.0, dtype=torch.float64, device="cuda:0")
        torch.cuda.synchronize()
        cuda = C.CDLL("libcuda.so.1")
        base, size = C.c_uint64(), C.c_size_t()
        assert cuda.cuMemGetAddressRange_v2(C.byref(base), C.byref(size), C.c_uint64(buf.data_ptr())) == 0
        end = base.value + size.value
        short = end - 8 * (N - 1)
        assert short >= buf.data_ptr()
        assert _call(lib, ch, idx, b, short) == -1
        assert "bytes to the end of its allocation" in lib.brr_last_error().decode()
        assert _call(lib, ch, idx, b, buf.data_ptr() + 4) == -1
        torch.cuda.synchronize()
        assert bool((buf == 7.0).all())
        assert _call(lib, ch, idx, b, buf.data_ptr()) == 0, lib.brr_last_error().decode()


@pytest.mark.gpu
def test_noalloc_rejects_more_terms_than_its_static_array(gpu_lib):
    import torch
    N, M = 200, 5
    g, _ = plink.synth_genotypes(N, M, seed=3)
    lib = gpu_lib
    with gpu.Chain(gpu.ChainConfig(N=N, M=M, device=0), lib=lib) as ch:
        ch.pack_bed(plink.encode_bed(g))
        out = torch.zeros(N, dtype=torch.float64, device="cuda:0")
        n = 65537
        idx = np.zeros(n, np.uint32)
        b = np.zeros(n, np.float64)
        rc = _call(lib, ch, idx, b, out.data_ptr())
        assert rc == -1
        assert "65536" in lib.brr_last_error().decode()


def _strip_comments(src):
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return re.sub(r"//[^\n]*", "", src)


def _function_body(src, name):
    i = src.index(name + "(")
    j = src.index("{", i)
    depth, k = 0, j
    while True:
        depth += {"{": 1, "}": -1}.get(src[k], 0)
        if depth == 0:
            return src[j:k + 1]
        k += 1


def test_noalloc_source_names_no_allocating_call():
    """The allocation-free path (its translation unit and the C-ABI function
    body) names no device-allocating call, torch's included."""
    banned = re.compile(r"cudaMalloc\w*|cudaFree\w*|cuMemAlloc\w*|cuMemFree\w*|cuMemCreate|dalloc|torch|at::")
    unit = _strip_comments((CSRC / "brr_noalloc.cu").read_text())
    assert not banned.search(unit), banned.search(unit)
    api = _strip_comments((CSRC / "brr_api.cu").read_text())
    body = _function_body(api, "int brr_xbeta_noalloc")
    assert "noalloc_xbeta" in body and "noalloc_check_output" in body
    assert not banned.search(body), body
