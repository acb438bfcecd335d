"""In-tree build of libbrr_gpu.so for sm_103a (nvcc, no cmake).

Each translation unit is compiled in parallel to an object file and the
objects are linked into ``bayesrrcmd_gb300/lib/libbrr_gpu.so``.  Host code is
compiled with ``-ffp-contract=off`` so that the scalar draws made on the host
are bit-identical on x86-64 and aarch64.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
LIBDIR = PKG / "lib"
BUILD = PKG / "_build"
LIB = LIBDIR / "libbrr_gpu.so"
SOURCES = ["brr_pack.cu", "brr_sweep.cu", "brr_block.cu", "brr_batch.cu", "brr_api.cu", "brr_batch_api.cu",
           "brr_multi_api.cu", "brr_noalloc.cu", "brr_gram.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libbrr_gpu.so")


def _stale(target: Path, deps) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def build_gpu(verbose: bool = False) -> Path:
    """Compile and link libbrr_gpu.so if any source is newer than it."""
    BUILD.mkdir(exist_ok=True)
    LIBDIR.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + [PKG.parent / "include" / "brr_gpu.h"]
    cc = nvcc()

    def compile_one(src: str) -> Path:
        obj = BUILD / (Path(src).stem + ".o")
        if _stale(obj, [CSRC / src] + headers):
            cmd = [cc, *ARCH, *NVFLAGS, "-c", str(CSRC / src), "-o", str(obj)]
            if verbose:
                print(" ".join(cmd), file=sys.stderr)
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    if _stale(LIB, objs):
        cmd = [cc, *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-lcudart", "-lcublas", "-lcublasLt"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link of libbrr_gpu.so failed:\n{r.stdout}\n{r.stderr}")
    return LIB


HOST = PKG / "host"
BINDIR = PKG / "bin"
CLI = BINDIR / "brr"


def zlib_flags(cxx: str) -> list:
    """-DBRR_WITH_ZLIB -lz when a program using zlib compiles and links here,
    else nothing: `brr` then reads only uncompressed preprocessed files and
    says so when it meets a compressed record."""
    BUILD.mkdir(exist_ok=True)
    probe = BUILD / "zlib_probe.cpp"
    probe.write_text("#include <zlib.h>\nint main() { return zlibVersion() == nullptr; }\n")
    r = subprocess.run([cxx, str(probe), "-o", str(BUILD / "zlib_probe"), "-lz"], capture_output=True, text=True)
    return ["-DBRR_WITH_ZLIB", "-lz"] if r.returncode == 0 else []


def build_cli(verbose: bool = False) -> Path:
    """Compile the `brr` command-line host (C++17) against libbrr_gpu.so."""
    lib = build_gpu(verbose)
    BINDIR.mkdir(exist_ok=True)
    srcs = sorted(HOST.glob("*.cpp"))
    deps = srcs + sorted(HOST.glob("*.h")) + [PKG.parent / "include" / "brr_gpu.h", lib]
    if _stale(CLI, deps):
        cxx = shutil.which("g++") or shutil.which("c++")
        if not cxx:
            raise RuntimeError("no C++ compiler for the brr host")
        z = zlib_flags(cxx)
        cmd = [cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-pthread", *z[:1], "-o", str(CLI), *map(str, srcs),
               f"-L{LIBDIR}", "-lbrr_gpu", *z[1:], "-Wl,-rpath,$ORIGIN/../lib"]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"build of brr failed:\n{r.stdout}\n{r.stderr}")
    return CLI


ADAPTER = PKG / "adapter"
ADAPTER_LIB = LIBDIR / "libbrr_adapter.so"


def build_adapter(verbose: bool = False) -> Path:
    """Compile the reference-interface adapter (GpuMarkerBuilder,
    GpuSweepGraph; C++17) into libbrr_adapter.so against libbrr_gpu.so."""
    lib = build_gpu(verbose)
    srcs = sorted(ADAPTER.glob("*.cpp"))
    deps = srcs + sorted(ADAPTER.glob("*.h")) + [PKG.parent / "include" / "brr_gpu.h", lib]
    if _stale(ADAPTER_LIB, deps):
        cxx = shutil.which("g++") or shutil.which("c++")
        if not cxx:
            raise RuntimeError("no C++ compiler for the adapter")
        cmd = [cxx, "-O2", "-std=c++17", "-fPIC", "-shared", "-Wall", "-o", str(ADAPTER_LIB), *map(str, srcs),
               f"-L{LIBDIR}", "-lbrr_gpu", "-Wl,-rpath,$ORIGIN"]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"build of libbrr_adapter.so failed:\n{r.stdout}\n{r.stderr}")
    return ADAPTER_LIB


def build_all(verbose: bool = False):
    return build_gpu(verbose), build_cli(verbose), build_adapter(verbose)


if __name__ == "__main__":
    print(build_all(verbose=True))
