"""Build and load the oracle (TEST INFRASTRUCTURE ONLY).

liborc.so is the CPU restatement of the reference (pcf_oracle.cpp). It is the
checker for the CUDA engine: only tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py may load it. oracle/_ref/ holds the reference's
own sources compiled by build_ref.sh, where the reference is present.
"""
from __future__ import annotations

import ctypes as C
import glob
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liborc.so")
REF_DIR = os.path.join(HERE, "_ref")

_D, _I, _U32, _U64, _I64 = C.c_double, C.c_int, C.c_uint32, C.c_uint64, C.c_int64
_PD = C.POINTER(C.c_double)
_PU32 = C.POINTER(C.c_uint32)

SIGS = {
    "orc_philox4x32_10": (None, [_PU32, _PU32, _PU32]),
    "orc_normals4": (None, [_U64, _U32, _U32, _U64, _U32, _PD]),
    "orc_bs_price": (_D, [_D, _D, _D, _D, _D, _I]),
    "orc_geo_weighted_price": (_D, [_D, _D, _D, _D, _D, _I, _PD, _I, _PD]),
    "orc_asian_geo_weights": (None, [_I, _I, _PD]),
    "orc_geo_asian_price": (_D, [_D, _D, _D, _D, _D, _I, _I, _I, _PD]),
    "orc_geo_basket_price": (_D, [_I, _PD, _PD, _PD, _D, _D, _D, _D, _I, _PD]),
    "ref_mc_eur": (_D, [_D, _D, _D, _D, _D, _I, _D, _U32]),
    "ref_mc_eur_omp": (_D, [_D, _D, _D, _D, _D, _I, _D, _U32, _I]),
    "ref_mc_asia": (_D, [_D, _D, _D, _D, _D, _I, _I, _D, _U32]),
    "ref_mc_asia_omp": (_D, [_D, _D, _D, _D, _D, _I, _I, _D, _U32, _I]),
    "ref_mc_amer": (_D, [_D, _D, _D, _D, _D, _I, _I, _D, _U32]),
    "ref_mc_amer_omp": (_D, [_D, _D, _D, _D, _D, _I, _I, _D, _U32, _I]),
    "ref_mc_asia_omp_stats": (None, [_D, _D, _D, _D, _D, _I, _I, _D, _U32, _I, _PD]),
    "ref_binom_embar": (_D, [_D, _D, _D, _D, _D, _I, _D]),
    "ref_binom_embar_omp": (_D, [_D, _D, _D, _D, _D, _I, _D, _I]),
    "ref_binom_embar_window": (_D, [_D, _D, _D, _D, _D, _I, _D, _I, _I]),
    "ref_comb": (_D, [_I, _I]),
    "ref_lattice": (None, [_D, _D, _D, _I, _PD]),
    "ref_binom_vanilla_eur": (_D, [_D, _D, _D, _D, _D, _I, _D]),
    "ref_binom_vanilla_amer": (_D, [_D, _D, _D, _D, _D, _I, _D]),
    "twin_mc_eur": (None, [_D, _D, _D, _D, _D, _I64, _I, _U64, _U32, _PD]),
    "twin_mc_asia": (None, [_D, _D, _D, _D, _D, _I64, _I, _I, _I, _U64, _U32, _PD]),
    "twin_mc_basket": (None, [_I, _PD, _PD, _PD, _D, _D, _D, _D, _I64, _I, _U64, _U32, _PD]),
    "twin_mc_amer": (None, [_D, _D, _D, _D, _D, _I64, _I, _I, _I, _U64, _U32, _PD]),
    "orc_emulate_lsm_record": (None, [_D, _D, _D, _D, _D, _I64, _I, _I, _U64, _U32,
                                      C.POINTER(C.c_float), _PD, C.POINTER(C.c_uint16),
                                      C.POINTER(C.c_float), _PD]),
    "twin_mc_amer_audit": (None, [_D, _D, _D, _D, _D, _I64, _I, _I, _I, _U64, _U32,
                                  C.POINTER(C.c_float), _PD, C.POINTER(C.c_uint16),
                                  C.POINTER(C.c_float), _PD, _PD]),
}


def build(force: bool = False) -> str:
    src = os.path.join(HERE, "pcf_oracle.cpp")
    hdr = os.path.join(HERE, "philox_host.h")
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= max(os.path.getmtime(src), os.path.getmtime(hdr))):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    tmp = LIB + ".tmp"
    subprocess.run(["g++", "-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fPIC",
                    "-shared", "-o", tmp, src], check=True)
    os.replace(tmp, LIB)
    return LIB


def build_ref(reference_root: str | None = None) -> bool:
    """Compile the reference's own sources into _ref/ when they are present.

    The location is the argument, else the PCF_REFERENCE_ROOT environment
    variable; with neither, or no sources there, nothing is built."""
    reference_root = reference_root or os.environ.get("PCF_REFERENCE_ROOT", "")
    if not reference_root or not os.path.isdir(os.path.join(reference_root, "src")):
        return False
    subprocess.run(["sh", os.path.join(HERE, "build_ref.sh"), reference_root], check=True,
                   capture_output=True)
    return True


_orc = None


def load() -> C.CDLL:
    global _orc
    if _orc is None:
        build()
        lib = C.CDLL(LIB)
        for name, (res, args) in SIGS.items():
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _orc = lib
    return _orc


class RefLib:
    """One reference source compiled as a shared object (oracle/_ref)."""

    def __init__(self, path: str):
        self.lib = C.CDLL(path)
        self.lib.ref_call.restype = C.c_double
        self.lib.ref_call.argtypes = [_D, _D, _D, _D, _D, _I, _I, _D, _I]
        self.lib.ref_set_seed.argtypes = [C.c_longlong]
        self.lib.ref_set_threads.argtypes = [_I]

    def __call__(self, S0, E, r, sigma, T, N, M=0, payoff_fun=1.0, threads=0, seed=0):
        self.lib.ref_set_seed(int(seed))
        if threads:
            self.lib.ref_set_threads(int(threads))
        return self.lib.ref_call(S0, E, r, sigma, T, int(N), int(M), float(payoff_fun),
                                 int(threads))


def ref_available() -> list[str]:
    return sorted(os.path.basename(p)[4:-3] for p in glob.glob(os.path.join(REF_DIR, "ref_*.so")))


def load_ref(name: str) -> RefLib | None:
    p = os.path.join(REF_DIR, f"ref_{name}.so")
    if not os.path.exists(p):
        return None
    try:
        return RefLib(p)
    except OSError:
        return None
