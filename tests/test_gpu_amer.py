"""GPU parity of the Longstaff-Schwartz kernel (the reference's mc_amer).

Bars:
  * FP64 twin on identical Philox draws: the LSM price and the control
    variate within 3e-4 relative for puts and 1e-3 for calls (FP32 paths can
    flip the exercise decision of the paths whose continuation estimate lies
    within FP32 rounding of the exercise value; each flip moves the price by
    at most payoff/N);
  * puts against the reference's own lattice oracle binom_vanilla_amer
    (src/binom_vanilla_amer.cpp:5-40): LSM low bias (5 cents) + 4 SE;
  * the reference's own algorithm with its exercise rule
    (src/mc_amer.cpp:100, ref_exercise=1) within 3 combined SE.
"""
import ctypes as C
import math

import pytest

pytestmark = pytest.mark.gpu


def twin(orc, S0, E, r, sig, T, N, M, pf, ref_ex, seed):
    out = (C.c_double * 6)()
    orc.twin_mc_amer(S0, E, r, sig, T, N, M, pf, ref_ex, seed, 0, out)
    return list(out)


@pytest.mark.parametrize("pf", [-1, 1])
@pytest.mark.parametrize("N,M", [(20000, 50), (4096, 10), (65536, 50)])
def test_amer_matches_fp64_twin(orc, ctx, pf, N, M):
    from parcompfin_gb300 import mc_amer_result
    res = mc_amer_result(100, 100, .05, .3, 1.0, N, M, pf, seed=5, ctx=ctx)
    s = twin(orc, 100, 100, .05, .3, 1.0, N, M, pf, 0, 5)
    assert s[5] == 0
    # Calls on a non-dividend stock sit on the exercise boundary for many deep
    # in-the-money paths (early exercise is never optimal, the fit is only
    # just above the exercise value), so more decisions can flip: 1e-3.
    # The control variate is evaluated at each path's exercise date, so its
    # sums carry the same flips.
    tol = 3e-4 if pf == -1 else 1e-3
    for k in (0, 2):
        assert abs(res.sums[k] - s[k]) <= tol * abs(s[k]), (k, res.sums[k], s[k])


def test_amer_streaming_sweep_matches_fp64_twin(orc, ctx):
    """3.2e6 paths (a point of the reference's runscript_mc_amer.sh grid): the
    per-block slice exceeds shared memory, so the sweep streams its per-path
    state through device memory; the same bar as the shared-memory kernels."""
    from parcompfin_gb300 import mc_amer_result
    N, M = 3_200_000, 10
    res = mc_amer_result(100, 100, .05, .3, 1.0, N, M, -1, seed=5, ctx=ctx)
    s = twin(orc, 100, 100, .05, .3, 1.0, N, M, -1, 0, 5)
    assert s[5] == 0
    for k in (0, 2):
        assert abs(res.sums[k] - s[k]) <= 3e-4 * abs(s[k]), (k, res.sums[k], s[k])


def test_amer_streaming_sweep_reference_rule_call_matches_fp64_twin(orc, ctx):
    """The streaming sweep with the reference's exercise rule, on a call."""
    from parcompfin_gb300 import mc_amer_result
    N, M = 3_200_000, 8
    res = mc_amer_result(100, 95, .05, .3, 1.0, N, M, 1, ref_exercise=True, seed=6, ctx=ctx)
    s = twin(orc, 100, 95, .05, .3, 1.0, N, M, 1, 1, 6)
    assert s[5] == 0
    for k in (0, 2):
        assert abs(res.sums[k] - s[k]) <= 1e-3 * abs(s[k]), (k, res.sums[k], s[k])


def test_amer_streaming_sweep_against_lattice(orc, ctx):
    from parcompfin_gb300 import mc_amer_result
    lat = orc.ref_binom_vanilla_amer(100, 100, .05, .3, 1.0, 2000, -1.0)
    res = mc_amer_result(100, 100, .05, .3, 1.0, 4_000_000, 200, "put", seed=3, use_cv=True,
                         ctx=ctx)
    assert res.n_paths == 4_000_000
    assert abs(res.price_plain - lat) < 0.05 + 4 * res.std_error_plain, (res.price_plain, lat)
    assert abs(res.price_cv - lat) < 0.05 + 4 * res.std_error_cv, (res.price_cv, lat)


def test_amer_put_against_lattice(orc, ctx):
    from parcompfin_gb300 import mc_amer_result
    lat = orc.ref_binom_vanilla_amer(100, 100, .05, .3, 1.0, 2000, -1.0)
    res = mc_amer_result(100, 100, .05, .3, 1.0, 1 << 20, 50, "put", seed=1, use_cv=True, ctx=ctx)
    assert abs(res.price_plain - lat) < 0.05 + 4 * res.std_error_plain, (res.price_plain, lat)
    assert abs(res.price_cv - lat) < 0.05 + 4 * res.std_error_cv, (res.price_cv, lat)
    assert res.std_error_cv < res.std_error_plain


@pytest.mark.parametrize("E", [90.0, 110.0])
def test_amer_put_other_strikes(orc, ctx, E):
    from parcompfin_gb300 import mc_amer_result
    lat = orc.ref_binom_vanilla_amer(100, E, .05, .25, 1.0, 2000, -1.0)
    res = mc_amer_result(100, E, .05, .25, 1.0, 1 << 19, 50, -1, seed=2, ctx=ctx)
    assert abs(res.price_plain - lat) < 0.05 + 4 * res.std_error_plain, (res.price_plain, lat)


def test_amer_reference_exercise_rule_matches_reference(orc, ctx):
    """With ref_exercise=1 the GPU reproduces the reference's put (~94), which
    the reference's own code computes (oracle restatement, mt19937 draws)."""
    from parcompfin_gb300 import mc_amer_result
    N, M = 20000, 50
    ref = [orc.ref_mc_amer(100, 100, .05, .3, 1.0, N, M, -1.0, s) for s in range(1, 7)]
    ref_mean = sum(ref) / len(ref)
    ref_sd = math.sqrt(sum((x - ref_mean) ** 2 for x in ref) / (len(ref) - 1))
    res = mc_amer_result(100, 100, .05, .3, 1.0, 1 << 18, M, -1, ref_exercise=True, seed=3,
                         ctx=ctx)
    se = math.hypot(ref_sd / math.sqrt(len(ref)), res.std_error_plain)
    assert ref_mean > 50
    assert abs(res.price_plain - ref_mean) < 3 * se + 0.02, (res.price_plain, ref_mean, se)


def test_amer_call_is_a_lower_bound(orc, ctx):
    """No dividends: the American call equals the European call (Black-Scholes),
    and any exercise policy gives a lower bound. The quadratic-basis LSM policy
    exercises some deep in-the-money paths early, so it sits about 1.4% below
    (the FP64 twin shows the same 14.03 against 14.23 at this N)."""
    from parcompfin_gb300 import mc_amer_result
    bs = orc.orc_bs_price(100, 100, .05, .3, 1.0, 1)
    N = 1 << 19
    res = mc_amer_result(100, 100, .05, .3, 1.0, N, 50, 1, seed=4, use_cv=True, ctx=ctx)
    assert res.price_plain <= bs + 3 * res.std_error_plain
    assert res.price_plain > bs - 0.35
    s = twin(orc, 100, 100, .05, .3, 1.0, N, 50, 1, 0, 4)
    assert abs(res.price_plain - s[0] / (N // 2)) < 1e-3 * bs  # sums over N/2 pair means


def test_amer_reference_call(orc, ctx):
    """Reference rule on calls: GPU vs the reference's own algorithm."""
    from parcompfin_gb300 import mc_amer_result
    N, M = 20000, 20
    ref = [orc.ref_mc_amer(100, 90, .05, .3, 1.0, N, M, 1.0, s) for s in range(1, 7)]
    ref_mean = sum(ref) / len(ref)
    ref_sd = math.sqrt(sum((x - ref_mean) ** 2 for x in ref) / (len(ref) - 1))
    res = mc_amer_result(100, 90, .05, .3, 1.0, 1 << 18, M, 1, ref_exercise=True, seed=3,
                         ctx=ctx)
    se = math.hypot(ref_sd / math.sqrt(len(ref)), res.std_error_plain)
    assert abs(res.price_plain - ref_mean) < 3 * se + 0.02, (res.price_plain, ref_mean, se)


def test_amer_edge_cases(ctx):
    from parcompfin_gb300 import mc_amer, mc_amer_result
    with pytest.raises(ValueError, match="divisible by 2"):
        mc_amer(100, 100, .05, .3, 1.0, 1001, 50, -1, ctx=ctx)
    with pytest.raises(ValueError):
        mc_amer(100, 100, .05, .3, 1.0, 1000, 1, -1, ctx=ctx)
    # Tiny path counts take the <= 2 in-the-money branch of src/mc_amer.cpp:75-83.
    for N in (2, 4, 6):
        r = mc_amer_result(100, 100, .05, .3, 1.0, N, 5, -1, seed=1, ctx=ctx)
        assert r.price >= 0 and math.isfinite(r.price)
    # Deep in the money: the price is at least the immediate exercise value.
    v = mc_amer(100, 200, .05, .3, 1.0, 4096, 10, -1, ctx=ctx)
    assert v >= 100.0


def test_amer_deterministic(ctx):
    from parcompfin_gb300 import mc_amer
    a = mc_amer(100, 100, .05, .3, 1.0, 65536, 50, -1, seed=9, ctx=ctx)
    b = mc_amer(100, 100, .05, .3, 1.0, 65536, 50, -1, seed=9, ctx=ctx)
    assert a == b


def test_context_release_and_memory_limit(ctx):
    """The context keeps the LSM path matrix between calls; release frees it,
    and a memory limit below a call's need makes that call PCF_ENOMEM while
    smaller calls go on. The same contract prices to the same sums after."""
    from parcompfin_gb300 import mc_amer_result, mc_eur_result
    from parcompfin_gb300._lib import PcfError, PCF_ENOMEM
    args = (100, 100, .05, .3, 1.0, 1 << 20, 50, -1)
    first = mc_amer_result(*args, seed=8, ctx=ctx)     # a 210 MB path matrix
    ctx.release()
    ctx.set_memory_limit(64 << 20)
    with pytest.raises(PcfError) as e:
        mc_amer_result(*args, seed=8, ctx=ctx)
    assert e.value.status == PCF_ENOMEM
    small = mc_eur_result(100, 100, .05, .2, 1.0, 1 << 20, "call", seed=8, ctx=ctx)
    assert small.price > 0
    ctx.set_memory_limit(0)
    again = mc_amer_result(*args, seed=8, ctx=ctx)
    assert list(again.sums) == list(first.sums)
