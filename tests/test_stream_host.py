"""The product's draw stream (bayesrrcmd_gb300/csrc/brr_stream.h) against the
oracle's, bit for bit, on the host (CPU only).

Both sides replace the reference's Boost mt19937 draws
(src/distributions_boost.cpp:16-65) by one counter-based stream; the GPU
kernels and the host driver compile brr_stream.h, the oracle has its own C
copy.  Here a small driver compiled from brr_stream.h with the library's host
flags (-ffp-contract=off) prints Philox blocks, per-marker (u, z) draws,
Gamma variates over shapes from 0.3 to 50,000 and inverse scaled chi-square
draws as exact hexadecimal doubles, and each must equal the oracle's value.
"""
import shutil
import subprocess

import numpy as np
import pytest

import oracle_lib as O
from bayesrrcmd_gb300.build import CSRC

DRIVER = r"""
#include <cstdio>
#include "brr_stream.h"
using namespace brr;
int main()
{
    const uint32_t seeds[3] = {1u, 20261203u, 0xFFFFFFFFu};
    const uint32_t chains[2] = {0u, 37u};
    for (uint32_t s : seeds)
        for (uint32_t ch : chains) {
            const StreamKey k{s, ch};
            for (uint32_t i = 0; i < 4; ++i) {
                const U4 b = stream_block(k, i * 977u, i * 13u, 1u + i, i * 5u);
                std::printf("P %u %u %u %u %u %u %u %u %u\n", s, ch, i, b.x, b.y, b.z, b.w, 0u, 0u);
            }
            for (uint32_t it = 0; it < 3; ++it)
                for (uint32_t j = 0; j < 50; ++j) {
                    double u, z;
                    marker_draws(k, it, j, &u, &z);
                    std::printf("M %u %u %u %u %a %a\n", s, ch, it, j, u, z);
                }
            const double shapes[7] = {0.3, 0.5, 1.0, 2.5, 17.0, 1000.5, 50000.0};
            for (uint32_t it = 0; it < 3; ++it)
                for (int q = 0; q < 7; ++q) {
                    double g = -1.0;
                    const bool ok = gamma_draw(k, it, 5u + (uint32_t)(q % 3), (uint32_t)q, shapes[q], &g);
                    std::printf("G %u %u %u %d %a %d %a\n", s, ch, it, q, shapes[q], ok ? 1 : 0, g);
                }
            double x = -1.0;
            const bool ok = inv_scaled_chisq(k, 4u, 5u, 0u, 100000.0001, 0.61, &x);
            std::printf("X %u %u %d %a\n", s, ch, ok ? 1 : 0, x);
        }
    return 0;
}
"""


@pytest.fixture(scope="module")
def stream_lines(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no C++ compiler")
    d = tmp_path_factory.mktemp("stream")
    src, exe = d / "driver.cpp", d / "driver"
    src.write_text(DRIVER)
    r = subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", f"-I{CSRC}", str(src), "-o", str(exe), "-lm"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    return [ln.split() for ln in out.splitlines()]


def test_philox_blocks_equal_oracle(stream_lines):
    rows = [t for t in stream_lines if t[0] == "P"]
    assert len(rows) == 24
    for t in rows:
        s, ch, i = int(t[1]), int(t[2]), int(t[3])
        want = O.philox([i * 977, i * 13, 1 + i, i * 5], [s, ch])
        assert [int(v) for v in t[4:8]] == want


def test_marker_draws_equal_oracle_bit_for_bit(stream_lines):
    rows = [t for t in stream_lines if t[0] == "M"]
    assert len(rows) == 3 * 2 * 3 * 50
    cache = {}
    for t in rows:
        s, ch, it, j = (int(v) for v in t[1:5])
        if (s, ch, it) not in cache:
            cache[(s, ch, it)] = O.marker_draws(s, ch, it, 50)
        u, z = cache[(s, ch, it)]
        assert float.fromhex(t[5]) == u[j] and float.fromhex(t[6]) == z[j]


def test_gamma_draws_equal_oracle_bit_for_bit(stream_lines):
    rows = [t for t in stream_lines if t[0] == "G"]
    assert len(rows) == 3 * 2 * 3 * 7
    for t in rows:
        s, ch, it, q = (int(v) for v in t[1:5])
        shape = float.fromhex(t[5])
        assert t[6] == "1"
        rc, g = O.gamma(s, ch, it, 5 + q % 3, q, shape)
        assert rc == 0 and float.fromhex(t[7]) == g
    # the variates have the moments of Gamma(shape, 1) roughly: mean near shape
    big = [float.fromhex(t[7]) / float.fromhex(t[5]) for t in rows if float.fromhex(t[5]) >= 1000]
    assert np.all(np.abs(np.array(big) - 1.0) < 0.2)


def test_inverse_scaled_chisq_matches_its_definition(stream_lines):
    """1 / Gamma(dof/2, scale 1/(dof*scale/2)) (src/distributions_boost.cpp:45-60)
    from the oracle's Gamma variate of the same stream position."""
    rows = [t for t in stream_lines if t[0] == "X"]
    assert len(rows) == 6
    dof, scale = 100000.0001, 0.61
    for t in rows:
        s, ch = int(t[1]), int(t[2])
        assert t[3] == "1"
        rc, g = O.gamma(s, ch, 4, 5, 0, 0.5 * dof)
        assert rc == 0
        want = 1.0 / ((1.0 / (0.5 * dof * scale)) * g)
        assert float.fromhex(t[4]) == want
        assert abs(float.fromhex(t[4]) / scale - 1.0) < 0.05
