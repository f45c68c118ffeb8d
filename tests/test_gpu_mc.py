"""GPU parity of the Monte Carlo kernels (European, Asian, basket).

Three bars, each written in the test that uses it:
  * deterministic draws: the CUDA kernel (FP32 paths) against the oracle's
    FP64 twin fed the identical Philox draws, relative 1e-5 on the price;
  * closed forms: within 4 standard errors;
  * the reference's own algorithm (the oracle restatement, bit-identical to
    the reference, with std::mt19937 draws): within 3 combined standard errors.
"""
import ctypes as C
import math

import pytest

pytestmark = pytest.mark.gpu

DET_REL = 1e-5  # deterministic-draw tolerance, FP32 GPU vs FP64 twin


def twin_price(s, n, disc):
    m = s[0] / n
    return disc * m


def rel(a, b):
    return abs(a - b) / max(abs(b), 1e-300)


def _eur_twin(orc, S0, E, r, sigma, T, N, pf, seed):
    s = (C.c_double * 5)()
    orc.twin_mc_eur(S0, E, r, sigma, T, N, pf, seed, 0, s)
    return list(s)


@pytest.mark.parametrize("N", [1, 2, 3, 5, 1000, 4097, 65536, 1_000_000])
@pytest.mark.parametrize("pf", [1, -1])
def test_eur_matches_fp64_twin(orc, ctx, N, pf):
    from parcompfin_gb300 import mc_eur_result
    res = mc_eur_result(100, 100, .05, .2, 1, N, pf, seed=42, use_cv=True, ctx=ctx)
    s = _eur_twin(orc, 100, 100, .05, .2, 1, N, pf, 42)
    assert res.n_paths == N
    for k in range(5):
        if s[k] == 0:
            assert abs(res.sums[k]) < 1e-6
        else:
            assert rel(res.sums[k], s[k]) < DET_REL, (k, res.sums[k], s[k])
    assert rel(res.price_plain, math.exp(-.05) * s[0] / N) < DET_REL or s[0] == 0


def test_plain_and_cv_launches_share_the_payoff_sums(ctx):
    """The control-variate sums are compiled in only on request; the payoff
    sums are accumulated the same way either way."""
    from parcompfin_gb300 import mc_asia_result, mc_eur_result
    a = mc_eur_result(100, 95, .05, .2, 1, 123_457, 1, seed=3, ctx=ctx)
    b = mc_eur_result(100, 95, .05, .2, 1, 123_457, 1, seed=3, use_cv=True, ctx=ctx)
    assert list(a.sums[:2]) == list(b.sums[:2]) and list(a.sums[2:]) == [0.0, 0.0, 0.0]
    a = mc_asia_result(100, 95, .05, .2, 1, 5000, 12, -1, seed=3, ctx=ctx)
    b = mc_asia_result(100, 95, .05, .2, 1, 5000, 12, -1, seed=3, use_cv=True, ctx=ctx)
    assert list(a.sums[:2]) == list(b.sums[:2])


def test_eur_atm_call_against_black_scholes(ctx):
    from parcompfin_gb300 import mc_eur_result
    bs = 10.450583572185565
    res = mc_eur_result(100, 100, .05, .2, 1.0, 1_000_000, "call", seed=42, use_cv=True, ctx=ctx)
    assert abs(res.price_plain - bs) < 4 * res.std_error_plain
    assert abs(res.price_cv - bs) < 4 * res.std_error_cv
    assert res.std_error_cv < res.std_error_plain / 2


def test_eur_against_reference_algorithm(orc, ctx):
    """Reference mc_eur (mt19937 stream, oracle restatement) vs the GPU kernel."""
    from parcompfin_gb300 import mc_eur_result
    for (S0, E, r, sig, T, pf) in [(100, 110, .02, .75, 1.0, 1), (100, 90, .03, .3, .5, -1)]:
        N = 400_000
        ref = [orc.ref_mc_eur(S0, E, r, sig, T, N, float(pf), seed) for seed in (11, 12, 13, 14)]
        ref_mean = sum(ref) / len(ref)
        res = mc_eur_result(S0, E, r, sig, T, 4 * N, pf, seed=5, ctx=ctx)
        # Both estimate the same mean with the same per-path variance.
        se = res.std_error_plain * math.sqrt(2)
        assert abs(res.price_plain - ref_mean) < 3 * se, (res.price_plain, ref_mean, se)


def test_eur_deterministic_and_seed_dependent(ctx):
    from parcompfin_gb300 import mc_eur
    a = mc_eur(100, 100, .05, .2, 1, 100_000, 1, seed=7, ctx=ctx)
    b = mc_eur(100, 100, .05, .2, 1, 100_000, 1, seed=7, ctx=ctx)
    c = mc_eur(100, 100, .05, .2, 1, 100_000, 1, seed=8, ctx=ctx)
    assert a == b and a != c


def test_eur_zero_vol_is_forward_intrinsic(ctx):
    from parcompfin_gb300 import mc_eur
    v = mc_eur(100, 90, .05, 0.0, 1.0, 10_000, 1, ctx=ctx)
    assert v == pytest.approx((100 * math.exp(.05) - 90) * math.exp(-.05), rel=1e-6)


def test_eur_large_n(ctx):
    from parcompfin_gb300 import mc_eur_result
    res = mc_eur_result(100, 100, .05, .2, 1.0, 1 << 28, 1, seed=1, ctx=ctx)
    assert abs(res.price_plain - 10.450583572185565) < 4 * res.std_error_plain


def _asia_twin(orc, S0, E, r, sig, T, N, M, pf, mode, seed):
    s = (C.c_double * 5)()
    orc.twin_mc_asia(S0, E, r, sig, T, N, M, pf, mode, seed, 0, s)
    return list(s)


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("N,M", [(1, 1), (7, 3), (1000, 12), (4096, 13), (20000, 52),
                                 (3000, 252), (10001, 252), (257, 7)])
def test_asia_matches_fp64_twin(orc, ctx, mode, N, M):
    # Threads price their paths in pairs: odd N and odd paths per thread leave
    # a path without a partner at the end of an item.
    from parcompfin_gb300 import mc_asia_result
    for pf in (1, -1):
        res = mc_asia_result(100, 100, .04, .3, 1.0, N, M, pf, mode=mode, seed=13, use_cv=True,
                             ctx=ctx)
        s = _asia_twin(orc, 100, 100, .04, .3, 1.0, N, M, pf, mode, 13)
        for k in range(5):
            if s[k] == 0:
                assert abs(res.sums[k]) < 1e-6
            else:
                assert rel(res.sums[k], s[k]) < DET_REL, (k, res.sums[k], s[k])


def test_asia_against_reference_algorithm(orc, ctx):
    """Reference mc_asia running sum (mode 0) vs the GPU kernel, 3 combined SE."""
    from parcompfin_gb300 import mc_asia_result
    S0, E, r, sig, T, M = 100, 100, .05, .2, 1.0, 52
    N = 50_000
    ref = [orc.ref_mc_asia(S0, E, r, sig, T, N, M, 1.0, seed) for seed in range(1, 9)]
    ref_mean = sum(ref) / len(ref)
    res = mc_asia_result(S0, E, r, sig, T, 8 * N, M, 1, mode=0, seed=3, ctx=ctx)
    se = res.std_error_plain * math.sqrt(2)
    assert abs(res.price_plain - ref_mean) < 3 * se, (res.price_plain, ref_mean, se)


@pytest.mark.parametrize("mode", [0, 1])
def test_asia_control_variate(orc, ctx, mode):
    from parcompfin_gb300 import mc_asia_result
    res = mc_asia_result(100, 95, .04, .25, 1.5, 1 << 20, 52, 1, mode=mode, seed=2, use_cv=True,
                         ctx=ctx)
    # the geometric payoff's sample mean agrees with its closed form
    gbar = res.sums[2] / res.n_paths
    g2 = res.sums[3] / res.n_paths
    se_g = math.sqrt((g2 - gbar * gbar) / res.n_paths)
    assert abs(gbar - res.cv_mean) < 4 * se_g
    assert res.std_error_cv < res.std_error_plain / 5
    assert abs(res.price_cv - res.price_plain) < 4 * res.std_error_plain


def _chol(corr, d):
    L = [0.0] * (d * d)
    for i in range(d):
        for j in range(i + 1):
            v = corr[i * d + j] - sum(L[i * d + k] * L[j * d + k] for k in range(j))
            L[i * d + j] = math.sqrt(v) if i == j else v / L[j * d + j]
    return L


# From 24 assets the tensor-core kernel runs (3xTF32 products; 17 to 23 run
# the CUDA-core kernel for up to 32 assets): 17, 24 and 48 leave
# padded K and N, 32 and 64 fill them exactly.
@pytest.mark.parametrize("d", [1, 4, 7, 16, 17, 24, 32, 33, 48, 64])
def test_basket_matches_fp64_twin(orc, ctx, d):
    from parcompfin_gb300 import mc_basket_result
    import random
    rng = random.Random(d)
    S0 = [100.0 + rng.uniform(-5, 5) for _ in range(d)]
    sig = [rng.uniform(.15, .35) for _ in range(d)]
    corr = [1.0 if i == j else .3 for i in range(d) for j in range(d)]
    N = 20000
    res = mc_basket_result(S0, sig, corr, .03, 1.0, 100.0, N, 1, scale_by_sqrt_T=True, seed=11,
                           use_cv=True, ctx=ctx)
    s = (C.c_double * 5)()
    A = C.c_double * d
    orc.twin_mc_basket(d, A(*S0), A(*sig), (C.c_double * (d * d))(*_chol(corr, d)), .03, 1.0, 1.0,
                       100.0, N, 1, 11, 0, s)
    for k in range(5):
        assert rel(res.sums[k], s[k]) < DET_REL, (k, res.sums[k], s[k])


def test_basket_reference_article_values(ctx):
    """results/results_mc_eur_multi.csv:19 -- the reference prices the d=4,
    rho=.5 basket (S0=K=100, r=.1, sigma=.2, T=1) at 11.9205 with 1e8 paths."""
    from parcompfin_gb300 import mc_eur_multi_result
    res = mc_eur_multi_result(100, 100, .1, .2, 1.0, 1 << 24, 1, 4, .5, seed=4, use_cv=True,
                              ctx=ctx)
    ref_se = res.std_error_plain * math.sqrt((1 << 24) / 1e8)
    se = math.hypot(res.std_error_cv, ref_se)
    assert abs(res.price_cv - 11.9205) < 3 * se + 5e-5, (res.price_cv, se)


def test_wide_baskets_share_one_launch(orc, ctx):
    """Baskets of 20, 40 and 64 assets in one batch: the tensor-core kernel
    stages each contract's factor in turn; every contract matches its twin."""
    import parcompfin_gb300 as pcf
    import random
    reqs, args = [], []
    for i, d in enumerate((20, 40, 64)):
        rng = random.Random(100 + d)
        S0 = [100.0 + rng.uniform(-5, 5) for _ in range(d)]
        sig = [rng.uniform(.15, .35) for _ in range(d)]
        corr = [1.0 if a == b else .25 for a in range(d) for b in range(d)]
        reqs.append(pcf.request("basket", 100, 100, .03, .25, 1.0, 30000, "call", assets=d,
                                basket_S0=S0, basket_sigma=sig, corr=corr, use_cv=True,
                                scale_by_sqrt_T=True, seed=21, stream=i))
        args.append((d, S0, sig, corr))
    out = pcf.price_batch(reqs, ctx=ctx)
    for (d, S0, sig, corr), r, i in zip(args, out, range(3)):
        s = (C.c_double * 5)()
        A = C.c_double * d
        orc.twin_mc_basket(d, A(*S0), A(*sig), (C.c_double * (d * d))(*_chol(corr, d)), .03, 1.0,
                           1.0, 100.0, 30000, 1, 21, i, s)
        for k in range(5):
            assert rel(r.sums[k], s[k]) < DET_REL, (d, k, r.sums[k], s[k])


def test_wide_basket_eigen_fallback(ctx):
    """A rank-one correlation of 24 assets takes the full (eigen) factor on
    the tensor-core path; identical assets with rho = 1 are one asset."""
    from parcompfin_gb300 import mc_basket_result
    d = 24
    res = mc_basket_result([100.0] * d, [.2] * d, [1.0] * (d * d), .05, 1.0, 100.0, 1 << 20, 1,
                           seed=9, use_cv=True, ctx=ctx)
    assert abs(res.price_cv - 10.450583572185565) < 4 * res.std_error_cv + 1e-4


def test_basket_eigen_fallback(ctx):
    """A singular (rank-deficient) correlation takes the eigen square root,
    like include/mvn.h:71-76; d identical assets with rho = 1 is one asset."""
    from parcompfin_gb300 import mc_basket_result, mc_eur_result
    d = 3
    corr = [1.0] * (d * d)
    res = mc_basket_result([100.0] * d, [.2] * d, corr, .05, 1.0, 100.0, 1 << 20, 1, seed=9,
                           use_cv=True, ctx=ctx)
    assert abs(res.price_cv - 10.450583572185565) < 4 * res.std_error_cv + 1e-4


def test_basket_book_full_size_matches_fp64_twin(orc, ctx):
    """The basket book at full size, as the benchmark prices it: d = 4, 16
    and 64 assets, sigma_i ~ U[.15,.35], correlation 0.7 (rho = 0.3) + 0.3
    normalised Wishart(d, d + 2) from seed 11, 2^22 paths each, one batch
    (d = 64 on the tensor cores). Every moment sum against the FP64 twin on
    the identical Philox draws: 1e-5 relative."""
    import numpy as np
    import parcompfin_gb300 as pcf
    from parcompfin_gb300 import workloads
    book = workloads.basket_book()
    reqs = [pcf.request("basket", 100.0, c["E"], c["r"], 0.2, c["T"], c["N"], "call",
                        assets=c["assets"], basket_S0=c["basket_S0"],
                        basket_sigma=c["basket_sigma"], corr=c["corr"], use_cv=True,
                        scale_by_sqrt_T=True, seed=11, stream=i) for i, c in enumerate(book)]
    out = pcf.price_batch(reqs, ctx=ctx)
    for i, (c, r) in enumerate(zip(book, out)):
        d = c["assets"]
        L = np.linalg.cholesky(np.array(c["corr"])).ravel()
        s = (C.c_double * 5)()
        A = C.c_double * d
        orc.twin_mc_basket(d, A(*c["basket_S0"]), A(*c["basket_sigma"]),
                           (C.c_double * (d * d))(*L), c["r"], c["T"], math.sqrt(c["T"]), c["E"],
                           c["N"], 1, 11, i, s)
        for k in range(5):
            assert rel(r.sums[k], s[k]) < DET_REL, (d, k, r.sums[k], s[k])
