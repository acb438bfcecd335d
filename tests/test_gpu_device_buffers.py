"""Entry points that take a device pointer check it before any kernel reads or
writes it: host memory, and a device pointer with fewer bytes to the end of
its allocation than the call reads or writes, are refused with BRR_ERR_ARG and
nothing is launched.  Covers brr_synth_bed_device (writes M*ceil(N/4) bytes),
brr_pack_bed_device and brr_batch_pack_bed_device (read nbytes); the uneven
batch's brr_multi_pack_bed_device goes through brr_pack_bed_device.  The
reference reads BED files from disk only (src/data.cpp:52-75), so these checks
have no counterpart there; the refusal follows its status-return convention.
"""
import ctypes as C

import numpy as np
import pytest

from bayesrrcmd_gb300 import gpu, plink

pytestmark = pytest.mark.gpu


def _segment_end(ptr: int) -> int:
    cuda = C.CDLL("libcuda.so.1")
    base, size = C.c_uint64(), C.c_size_t()
    assert cuda.cuMemGetAddressRange_v2(C.byref(base), C.byref(size), C.c_uint64(ptr)) == 0
    return base.value + size.value


def test_device_entry_points_refuse_buffers_they_would_overrun(gpu_lib):
    import torch
    lib = gpu_lib
    N, M = 1000, 20
    nb = M * ((N + 3) // 4)
    host = np.zeros(nb, np.uint8)
    buf = torch.full((2 * nb,), 0x5A, dtype=torch.uint8, device="cuda:0")
    torch.cuda.synchronize()
    # a pointer inside the allocation with one byte too few to its end
    short = _segment_end(buf.data_ptr()) - (nb - 1)
    assert short >= buf.data_ptr()

    for ptr, words in ((host.ctypes.data, "device or managed"), (short, "bytes to the end of its allocation")):
        with pytest.raises(gpu.BrrError) as e:
            gpu.synth_bed_device(ptr, N, M, 3, 0.05, 0.5, 0.0, lib=lib)
        assert e.value.code == -1 and words in str(e.value)
        with pytest.raises(gpu.BrrError) as e:
            gpu.synth_bed_device_beta(ptr, N, M, 3, 0.5, 2.0, 0.01, 0.5, 0.0, lib=lib)
        assert e.value.code == -1 and words in str(e.value)
    torch.cuda.synchronize()
    assert bool((buf == 0x5A).all())

    # the exact size is accepted, and the payload packs like the same bytes from the host
    gpu.synth_bed_device(buf.data_ptr(), N, M, 3, 0.05, 0.5, 0.0, lib=lib)
    torch.cuda.synchronize()
    payload = buf[:nb].cpu().numpy()
    with gpu.Chain(gpu.ChainConfig(N=N, M=M, seed=1), lib=lib) as ch:
        for ptr, words in ((host.ctypes.data, "device or managed"), (short, "bytes to the end of its allocation")):
            with pytest.raises(gpu.BrrError) as e:
                ch.pack_bed_device(ptr, nb)
            assert e.value.code == -1 and words in str(e.value)
        ch.pack_bed_device(buf.data_ptr(), nb)
        t_dev, n_dev = ch.marker_table()
    with gpu.Chain(gpu.ChainConfig(N=N, M=M, seed=1), lib=lib) as ch:
        ch.pack_bed(payload)
        t_host, n_host = ch.marker_table()
    np.testing.assert_array_equal(t_dev, t_host)
    np.testing.assert_array_equal(n_dev, n_host)

    g, _ = plink.synth_genotypes(N, M, seed=5, missing=0.0)
    ok = torch.from_numpy(plink.encode_bed(g)).to("cuda:0")
    with gpu.Batch(gpu.ChainConfig(N=N, M=M, seed=1), chains=32, lib=lib) as bt:
        for ptr, words in ((host.ctypes.data, "device or managed"), (short, "bytes to the end of its allocation")):
            with pytest.raises(gpu.BrrError) as e:
                bt.pack_bed_device(ptr, nb)
            assert e.value.code == -1 and words in str(e.value)
        bt.pack_bed_device(ok.data_ptr(), nb)
