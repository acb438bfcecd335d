"""brr_xbeta_noalloc, the allocation-free genetic-value entry point, against
brr_xbeta.

It exists for callers that cannot allocate device memory when they need the
values (a runtime that owns the GPU through its own pool, a serving loop that
must not block on the allocator): the term list is staged in a fixed static
device array and the result goes to a buffer the caller owns.  The test owns
the output buffer (allocated with torch), calls the entry point twice in a
row with different term lists through the C ABI and compares each result with
brr_xbeta on the same context.  This file is collected last.
"""
import ctypes as C

import numpy as np
import pytest

from bayesrrcmd_gb300 import gpu, plink

pytestmark = pytest.mark.gpu
RTOL = 1e-12


def _ptr(a, ct):
    return a.ctypes.data_as(C.POINTER(ct))


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
            rc = lib.brr_xbeta_noalloc(ch.h, _ptr(idx, C.c_uint32), _ptr(b, C.c_double), n,
                                       C.c_void_p(out.data_ptr()))
            assert rc == 0, lib.brr_last_error().decode()
            torch.cuda.synchronize()
            np.testing.assert_allclose(out.cpu().numpy(), ref, rtol=RTOL, atol=1e-15,
                                       err_msg=f"call {call}")


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
        rc = lib.brr_xbeta_noalloc(ch.h, _ptr(idx, C.c_uint32), _ptr(b, C.c_double), n, C.c_void_p(out.data_ptr()))
        assert rc == -1
        assert "65536" in lib.brr_last_error().decode()
