"""Build recipe of the CPU oracle (test infrastructure only).

Compiles oracle.c into oracle/_build/liboracle.so with gcc, without fused
multiply-add contraction so that x86-64 and aarch64 hosts agree bit for bit.
"""
from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_build" / "liboracle.so"


def build_oracle() -> Path:
    src = [HERE / "oracle.c", HERE / "oracle.h"]
    if OUT.exists() and all(s.stat().st_mtime <= OUT.stat().st_mtime for s in src):
        return OUT
    OUT.parent.mkdir(exist_ok=True)
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        raise RuntimeError("no C compiler for the oracle")
    cmd = [cc, "-O2", "-std=c11", "-ffp-contract=off", "-fPIC", "-shared", "-o", str(OUT),
           str(HERE / "oracle.c"), "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    return OUT


if __name__ == "__main__":
    print(build_oracle())
