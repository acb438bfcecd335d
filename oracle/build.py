"""Build recipe of the CPU oracle (test infrastructure only).

Compiles oracle.c into oracle/_build/liboracle.so with gcc, without fused
multiply-add contraction so that x86-64 and aarch64 hosts agree bit for bit.
That build is the checker.  A second build, liboracle_timing.so, uses the
reference's fast release flags (-O3 -ffast-math -funroll-loops,
CMakeLists.txt:48-50 of the reference; -march=native left out so the recipe
is the same on every host) and serves only as the timed CPU baseline: its
results may differ from the checker's in the last bits.
"""
from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_build" / "liboracle.so"
OUT_TIMING = HERE / "_build" / "liboracle_timing.so"
EXACT_FLAGS = ["-O2", "-ffp-contract=off"]
TIMING_FLAGS = ["-O3", "-ffast-math", "-funroll-loops"]


def _build(out: Path, flags) -> Path:
    src = [HERE / "oracle.c", HERE / "oracle.h", Path(__file__)]
    if out.exists() and all(s.stat().st_mtime <= out.stat().st_mtime for s in src):
        return out
    out.parent.mkdir(exist_ok=True)
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        raise RuntimeError("no C compiler for the oracle")
    cmd = [cc, *flags, "-std=c11", "-fPIC", "-shared", "-o", str(out), str(HERE / "oracle.c"), "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    return out


def build_oracle() -> Path:
    """The checker: exact IEEE arithmetic, no contraction."""
    return _build(OUT, EXACT_FLAGS)


def build_oracle_timing() -> Path:
    """The timed CPU baseline: the same source with the reference's fast flags."""
    return _build(OUT_TIMING, TIMING_FLAGS)


if __name__ == "__main__":
    print(build_oracle(), build_oracle_timing())
