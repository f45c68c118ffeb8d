"""The C-ABI library builds, loads and exports every symbol include/pcf.h
declares; host-side argument handling works without a GPU (CPU only: no
call here launches a kernel)."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = []
    for h in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if h.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", h)).read()
            names += re.findall(r"PCF_API\s+[\w\s\*]+?\b(pcf_\w+)\s*\(", txt)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = _declared()
    for n in ("pcf_mc_eur", "pcf_mc_asia", "pcf_mc_eur_multi", "pcf_ctx_create"):
        assert n in names


def test_library_exports_every_declared_symbol(pcf_lib):
    missing = [n for n in _declared() if not hasattr(pcf_lib, n)]
    assert not missing, missing


def test_binding_covers_header(pcf_lib):
    from parcompfin_gb300 import _lib
    missing = [n for n in _declared() if n not in _lib.SIGNATURES]
    assert not missing, missing


def test_version_and_strerror(pcf_lib):
    assert b"sm_103a" in pcf_lib.pcf_version()
    assert pcf_lib.pcf_strerror(-1) == b"invalid argument"
    assert pcf_lib.pcf_strerror(-3).startswith(b"singular")


def test_payoff_codes():
    from parcompfin_gb300 import payoff_code
    assert payoff_code("call") == 1 and payoff_code("put") == -1
    assert payoff_code(1.0) == 1 and payoff_code(-1) == -1
    for bad in ("Call", "straddle", 0, 2, 0.5):
        with pytest.raises(ValueError, match="Unknown payoff function"):
            payoff_code(bad)


def test_invalid_arguments_are_rejected_before_any_device_work(pcf_lib):
    from parcompfin_gb300 import _lib
    out = _lib.McResult()
    # payoff_fun 2 is rejected like the reference's invalid_argument.
    assert pcf_lib.pcf_mc_eur(None, 100, 100, .05, .2, 1, 1000, 2, 0, 0, C.byref(out)) == -1
    assert b"payoff" in pcf_lib.pcf_last_error()
    assert pcf_lib.pcf_mc_eur(None, 100, 100, .05, .2, 1, 0, 1, 0, 0, C.byref(out)) == -1
    assert pcf_lib.pcf_mc_eur(None, -1, 100, .05, .2, 1, 10, 1, 0, 0, C.byref(out)) == -1
    assert pcf_lib.pcf_mc_eur(None, 100, 100, .05, .2, float("nan"), 10, 1, 0, 0,
                              C.byref(out)) == -1
    assert pcf_lib.pcf_mc_asia(None, 100, 100, .05, .2, 1, 10, 0, 1, 0, 0, 0, C.byref(out)) == -1
    assert pcf_lib.pcf_mc_asia(None, 100, 100, .05, .2, 1, 10, 4, 1, 7, 0, 0, C.byref(out)) == -1
    assert pcf_lib.pcf_mc_eur_multi(None, 100, 100, .05, .2, 1, 10, 1, 65, .5, 0, 0,
                                    C.byref(out)) == -1
    assert pcf_lib.pcf_mc_eur_multi(None, 100, 100, .05, .2, 1, 10, 1, 4, 1.5, 0, 0,
                                     C.byref(out)) == -1


def test_non_finite_parameters_are_rejected(pcf_lib):
    """NaN or infinite parameters are PCF_EINVAL on every entry point, before
    any device work (the reference would price garbage)."""
    out = _lib_result()
    nan, inf = float("nan"), float("inf")
    price = C.c_double()
    for bad in ((nan, 100, .05, .3, 1.0), (100, nan, .05, .3, 1.0), (100, 100, nan, .3, 1.0),
                (100, 100, .05, nan, 1.0), (100, 100, .05, .3, inf)):
        assert pcf_lib.pcf_mc_amer(None, *bad, 4096, 10, -1, 0, 0, 0, C.byref(out)) == -1
        assert pcf_lib.pcf_mc_eur(None, *bad, 4096, 1, 0, 0, C.byref(out)) == -1
        assert pcf_lib.pcf_mc_asia(None, *bad, 4096, 12, 1, 0, 0, 0, C.byref(out)) == -1
        assert pcf_lib.pcf_binom_embar(None, *bad, 1000, 1, 0, C.byref(price)) == -1
        assert pcf_lib.pcf_binom_vanilla(None, *bad, 1000, 1, 1, C.byref(price)) == -1
        assert pcf_lib.pcf_mc_amer_audit(None, *bad, 4096, 10, -1, 0, 0, C.byref(out), None,
                                         None, None, None) == -1


def _lib_result():
    from parcompfin_gb300 import _lib
    return _lib.McResult()


def test_no_device_fails_loudly(pcf_lib):
    """Without a GPU the engine reports it and never falls back to the CPU."""
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    from parcompfin_gb300 import PcfError, mc_eur
    with pytest.raises(PcfError):
        mc_eur(100, 100, .05, .2, 1, 1000, "call")
