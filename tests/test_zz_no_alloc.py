"""pcf_mc_eur_noalloc, the European entry point that allocates nothing.

It exists for callers that cannot call cudaMalloc while pricing (a plugin in
a framework whose caching allocator holds the GPU's memory, a loop that
cannot afford the synchronisation an allocation may cause, code allowed to
allocate only at start-up). Its scratch is a fixed array inside the library,
so these tests check:
  * two calls in a row, through the C ABI, each against pcf_mc_eur (the
    allocating entry point) within the 1e-5 relative tolerance of the other
    Monte Carlo GPU tests (the second call runs on the array the first one
    left behind);
  * the size limit is rejected with a clear error.
This file is collected last so that a run stopping at the first failure has
run every other test; it also passes on its own in a fresh process.
"""
import ctypes as C

import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-5


def _noalloc(lib, torch, args, out, stream):
    S0, E, r, sig, T, N, pf, seed = args
    return lib.pcf_mc_eur_noalloc(S0, E, r, sig, T, N, pf, seed, C.c_void_p(out.data_ptr()),
                                  C.c_void_p(stream.cuda_stream))


def test_noalloc_matches_allocating_entry_point_two_calls():
    import torch
    from parcompfin_gb300 import _lib, mc_eur_result
    lib = _lib.load()
    out = torch.full((5,), -1.0, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()
    cases = [(100.0, 100.0, .05, .2, 1.0, 1_000_000, 1, 42),
             (100.0, 110.0, .02, .75, 1.0, 3_000_001, -1, 7)]
    for args in cases:
        st = _noalloc(lib, torch, args, out, stream)
        assert st == 0, lib.pcf_last_error()
        torch.cuda.synchronize()
        got = out.cpu().tolist()
        S0, E, r, sig, T, N, pf, seed = args
        ref = mc_eur_result(S0, E, r, sig, T, N, pf, seed=seed, use_cv=True)
        for k in range(5):
            assert abs(got[k] - ref.sums[k]) <= TOL * abs(ref.sums[k]), (k, got[k], ref.sums[k])


def test_noalloc_rejects_sizes_beyond_its_limit():
    import torch
    from parcompfin_gb300 import _lib
    lib = _lib.load()
    out = torch.zeros(5, dtype=torch.float64, device="cuda")
    st = _noalloc(lib, torch, (100.0, 100.0, .05, .2, 1.0, (1 << 30) + 4, 1, 1), out,
                  torch.cuda.current_stream())
    assert st == _lib.PCF_EINVAL
    assert b"no-allocation limit" in lib.pcf_last_error()
    assert lib.pcf_mc_eur_noalloc(100.0, 100.0, .05, .2, 1.0, 1000, 1, 1, None, None) == \
        _lib.PCF_EINVAL
