"""In-tree build of the engine's shared library (libpcf.so) with nvcc.

Every CUDA translation unit is compiled for sm_103a only, in parallel, and
linked with the host C++ units into parcompfin_gb300/_lib/libpcf.so. The
library is loaded from the source tree (never installed), so the extension
that tests and benchmarks use is the one built here.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
OUT_DIR = os.path.join(PKG, "_lib")
BUILD_DIR = os.path.join(PKG, "_build")
LIB = os.path.join(OUT_DIR, "libpcf.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
           "-Xcompiler", "-fvisibility=hidden"]

# (source, extra flags). The binomial and lattice units must not contract
# a*b+c into FMA: they reproduce the reference's FP64 rounding term by term.
SOURCES = [
    ("mc_kernels.cu", []),
    ("lsm.cu", []),
    ("binom.cu", ["-fmad=false", "-Xcompiler", "-ffp-contract=off"]),
    ("lattice.cu", ["-fmad=false", "-Xcompiler", "-ffp-contract=off"]),
    ("pcf_api.cpp", []),
    ("pcf_batch.cpp", []),
    ("pcf_server.cpp", []),
    ("pcf_math.cpp", []),
    ("pcf_tune.cpp", []),
]


def _nvcc() -> str:
    for c in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libpcf")


def _sources():
    return [(s, f) for s, f in SOURCES if os.path.exists(os.path.join(CSRC, s))]


def _stale() -> bool:
    if not os.path.exists(LIB) or not os.path.exists(CLI):
        return True
    t = os.path.getmtime(LIB)
    for name in os.listdir(CSRC):
        if os.path.getmtime(os.path.join(CSRC, name)) > t:
            return True
    inc = os.path.join(os.path.dirname(PKG), "include", "pcf.h")
    return os.path.exists(inc) and os.path.getmtime(inc) > t


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile libpcf.so if any source is newer than it; return its path."""
    if not force and not _stale():
        return LIB
    nvcc = _nvcc()
    os.makedirs(OUT_DIR, exist_ok=True)
    os.makedirs(BUILD_DIR, exist_ok=True)

    def compile_one(item):
        src, extra = item
        obj = os.path.join(BUILD_DIR, src + ".o")
        cmd = [nvcc, *ARCH, *NVFLAGS, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
        if src.endswith(".cpp"):
            cmd = [nvcc, "-x", "cu", *ARCH, *NVFLAGS, *extra, "-c", os.path.join(CSRC, src),
                   "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
        if verbose:
            sys.stderr.write(r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=max(1, min(8, os.cpu_count() or 1))) as ex:
        objs = list(ex.map(compile_one, _sources()))
    tmp = LIB + ".tmp"
    cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    build_cli()
    return LIB


# The drop-in command-line programs: one executable (pcf_cli.cpp) linked
# against libpcf.so, reachable under every reference program name in _lib/bin.
CLI = os.path.join(OUT_DIR, "pcf_cli")
CLI_BIN = os.path.join(OUT_DIR, "bin")
CLI_NAMES = [m + v for m in ("mc_eur", "mc_eur_multi", "mc_asia", "mc_amer", "binom_embar")
             for v in ("", "_omp", "_mpi", "_hybrid")] + ["binom_vanilla_eur", "binom_vanilla_amer"]


def build_cli() -> str:
    src = os.path.join(CSRC, "pcf_cli.cpp")
    if not os.path.exists(src):
        return ""
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        raise RuntimeError("a C++ compiler is required to build pcf_cli")
    tmp = CLI + ".tmp"
    cmd = [cxx, "-O2", "-std=c++17", src, "-o", tmp, "-L" + OUT_DIR, "-lpcf",
           "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"pcf_cli build failed:\n{r.stderr}")
    os.replace(tmp, CLI)
    os.makedirs(CLI_BIN, exist_ok=True)
    for name in CLI_NAMES:
        link = os.path.join(CLI_BIN, name)
        if os.path.lexists(link):
            os.remove(link)
        os.symlink(os.path.join("..", "pcf_cli"), link)
    return CLI


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
