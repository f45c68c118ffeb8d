"""GPU parity of the Longstaff-Schwartz kernel (the reference's mc_amer).

Bars:
  * the exercise policy, audited against FP64 (oracle twin_mc_amer_audit):
    replayed on the GPU's own FP32 paths and coefficients, the kernel's
    decisions are reproduced path for path; its regression sums and fitted
    continuation values agree with an FP64 regression of the same state
    (sums 1e-6 relative, fitted values 1e-6 of the strike); the price of its
    policy agrees with the FP64 value of the same exercise dates within
    1e-5; on FP64 paths with the GPU's coefficients every decision that
    differs is a boundary flip (the FP64 decision function changes sign
    between the FP64 and the FP32 path value, or sits within the FP32
    evaluation error of the kernel's formula), and the flip count is
    reported;
  * against the independent FP64 twin (its own regressions on FP64 paths):
    3e-4 relative for puts and 1e-3 for calls, the size of the boundary
    flips the audit counts (each moves a path's cash flow by up to its
    payoff);
  * puts against the reference's own lattice oracle binom_vanilla_amer
    (src/binom_vanilla_amer.cpp:5-40): the LSM estimator's low bias at these
    path counts (5 cents) + 4 SE;
  * the reference's own algorithm with its exercise rule
    (src/mc_amer.cpp:100, ref_exercise=1), at the reference's path count,
    within 3 combined standard errors of the seed-to-seed spread.
"""
import ctypes as C
import json
import math
import os

import pytest

pytestmark = pytest.mark.gpu

AUDIT_KEYS = ["r1_tau_mismatch", "r1_mode_mismatch", "sums_rel_err", "fit_err_over_E",
              "fit_err_solve_over_E", "fp64_coef_flips", "fp64_coef_flip_margin",
              "price_rel_err_same_policy", "cv_rel_err_same_policy", "max_du",
              "r2_flips", "r2_unexplained", "r2_tau_diff", "r2_price_rel",
              "gpu_vs_fp64_value_of_gpu_policy", "r3_tau_diff", "r3_price_rel", "r3_cv_rel",
              "r2_flip_margin_over_E", "regression_dates", "itm_path_dates",
              "r4_tau_diff", "r4_price_rel", "r3_vs_r4_tau_diff", "r3_vs_r4_price_rel",
              "r4_first_divergence_date", "r4_first_divergence_paths",
              "r4_first_divergence_margin_over_E", "r4_first_divergence_fit_diff_over_E"]


def twin(orc, S0, E, r, sig, T, N, M, pf, ref_ex, seed):
    out = (C.c_double * 6)()
    orc.twin_mc_amer(S0, E, r, sig, T, N, M, pf, ref_ex, seed, 0, out)
    return list(out)


def audit(orc, ctx, S0, E, r, sig, T, N, M, pf, ref_ex, seed):
    """GPU sweep with its audit record, checked by the FP64 audit twin."""
    from parcompfin_gb300.api import mc_amer_audit
    res, coef, sums, tau, u = mc_amer_audit(S0, E, r, sig, T, N, M, pf, ref_exercise=ref_ex,
                                            seed=seed, ctx=ctx)
    rep = (C.c_double * 29)()
    mom = (C.c_double * 5)(*res.sums)
    fp = C.POINTER(C.c_float)
    orc.twin_mc_amer_audit(S0, E, r, sig, T, N, M, pf, int(ref_ex), seed, 0,
                           coef.ctypes.data_as(fp), sums.ctypes.data_as(C.POINTER(C.c_double)),
                           tau.ctypes.data_as(C.POINTER(C.c_uint16)), u.ctypes.data_as(fp), mom,
                           rep)
    d = dict(zip(AUDIT_KEYS, rep))
    d.update(N=N, M=M, pf=pf, ref_exercise=int(ref_ex))
    log = os.environ.get("PCF_AUDIT_LOG")
    if log:
        with open(log, "a") as f:
            f.write(json.dumps(d) + "\n")
    return res, d


@pytest.mark.parametrize("pf", [-1, 1])
@pytest.mark.parametrize("N,M", [(20000, 50), (65536, 50), (1 << 20, 50), (4096, 10)])
def test_amer_policy_audit(orc, ctx, pf, N, M):
    """The GPU's exercise policy against FP64, date by date (module docstring)."""
    res, a = audit(orc, ctx, 100, 100, .05, .3, 1.0, N, M, pf, False, 5)
    # R1: the kernel's decisions and regression, replayed on its own paths.
    assert a["r1_tau_mismatch"] == 0, a
    assert a["r1_mode_mismatch"] == 0, a
    assert a["sums_rel_err"] < 1e-6, a
    assert a["fit_err_over_E"] < 1e-6, a
    assert a["fit_err_solve_over_E"] < 1e-6, a
    # A decision the FP64 coefficients would change lies within the fitted
    # values' difference (plus the FP32 evaluation error) of the boundary.
    assert a["fp64_coef_flip_margin"] <= a["fit_err_over_E"] + 1e-6, a
    assert a["price_rel_err_same_policy"] < 1e-5, a
    assert a["cv_rel_err_same_policy"] < 1e-5, a
    # R2: FP64 paths with the GPU's coefficients: only boundary flips.
    assert a["max_du"] < 1e-4, a
    assert a["r2_unexplained"] == 0, a
    assert a["gpu_vs_fp64_value_of_gpu_policy"] < 1e-5, a
    assert a["regression_dates"] == M - 1, a
    # R4: FP64 regressions and decisions on the GPU's paths. Up to the first
    # date where they differ, the two states are identical; the decisions
    # that differ there lie within the fitted values' difference (the FP32
    # rounding of the coefficients) plus the FP32 evaluation error of the
    # boundary. Later differences are that flip's cascade through the later
    # regressions, and the independent twin's differences (R3) are the same
    # cascade: R3 against R4 (FP64 against FP32 paths) differ far less.
    if a["r4_first_divergence_date"]:
        assert a["r4_first_divergence_margin_over_E"] <= (
            a["r4_first_divergence_fit_diff_over_E"] + 1e-6), a


@pytest.mark.parametrize("pf", [-1, 1])
@pytest.mark.parametrize("N,M", [(20000, 50), (4096, 10), (65536, 50)])
def test_amer_matches_fp64_twin(orc, ctx, pf, N, M):
    from parcompfin_gb300 import mc_amer_result
    res = mc_amer_result(100, 100, .05, .3, 1.0, N, M, pf, seed=5, ctx=ctx)
    s = twin(orc, 100, 100, .05, .3, 1.0, N, M, pf, 0, 5)
    assert s[5] == 0
    # The independent twin decides on FP64 paths with its own regressions;
    # the policy audit above shows every decision that differs is a boundary
    # flip. Calls on a non-dividend stock keep many deep in-the-money paths
    # near the boundary (early exercise is never optimal, the fit is only
    # just above the exercise value), so more decisions can flip: 1e-3.
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


def _seed_stats(xs):
    m = sum(xs) / len(xs)
    sd = math.sqrt(sum((x - m) ** 2 for x in xs) / (len(xs) - 1))
    return m, sd / math.sqrt(len(xs))


def test_amer_reference_exercise_rule_matches_reference(orc, ctx):
    """With ref_exercise=1 the GPU reproduces the reference's put (~94), which
    the reference's own code computes (oracle restatement, mt19937 draws): at
    the same path count, over eight seeds each, the means agree within three
    combined standard errors of their seed-to-seed spread."""
    from parcompfin_gb300 import mc_amer_result
    N, M = 20000, 50
    ref = [orc.ref_mc_amer(100, 100, .05, .3, 1.0, N, M, -1.0, s) for s in range(1, 9)]
    gpu = [mc_amer_result(100, 100, .05, .3, 1.0, N, M, -1, ref_exercise=True, seed=s,
                          ctx=ctx).price_plain for s in range(1, 9)]
    (rm, rse), (gm, gse) = _seed_stats(ref), _seed_stats(gpu)
    assert rm > 50
    assert abs(gm - rm) < 3 * math.hypot(rse, gse), (gm, rm, gse, rse)


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
    """Reference rule on calls: GPU vs the reference's own algorithm at the
    same path count, eight seeds each, within three combined standard errors."""
    from parcompfin_gb300 import mc_amer_result
    N, M = 20000, 20
    ref = [orc.ref_mc_amer(100, 90, .05, .3, 1.0, N, M, 1.0, s) for s in range(1, 9)]
    gpu = [mc_amer_result(100, 90, .05, .3, 1.0, N, M, 1, ref_exercise=True, seed=s,
                          ctx=ctx).price_plain for s in range(1, 9)]
    (rm, rse), (gm, gse) = _seed_stats(ref), _seed_stats(gpu)
    assert abs(gm - rm) < 3 * math.hypot(rse, gse), (gm, rm, gse, rse)


def test_amer_reference_rule_policy_audit(orc, ctx):
    """The reference's exercise rule through the same FP64 policy audit."""
    res, a = audit(orc, ctx, 100, 95, .05, .3, 1.0, 20000, 20, 1, True, 6)
    assert a["r1_tau_mismatch"] == 0, a
    assert a["fit_err_over_E"] < 1e-6, a
    assert a["price_rel_err_same_policy"] < 1e-5, a
    assert a["r2_unexplained"] == 0, a


def test_amer_singular_regression(orc, ctx):
    """A degenerate contract whose normal equations are exactly singular
    (sigma = 0 and r = 0: every path sits at S = 50 < E = 100, all in the
    money with the same regressor, a rank-one normal matrix). The reference's
    inverse() throws "Detereminant is not > 0" (include/common.h:115-117;
    the oracle's restatement returns NaN); the GPU returns PCF_ESINGULAR.
    The next call on the same context prices normally."""
    from parcompfin_gb300 import mc_amer_result
    from parcompfin_gb300._lib import PCF_ESINGULAR, PcfError
    assert math.isnan(orc.ref_mc_amer(50, 100, 0.0, 0.0, 1.0, 4096, 5, -1.0, 1))
    s = twin(orc, 50, 100, 0.0, 0.0, 1.0, 4096, 5, -1, 0, 1)
    assert s[5] == 1
    for N in (4096, 65536):
        with pytest.raises(PcfError) as e:
            mc_amer_result(50, 100, 0.0, 0.0, 1.0, N, 5, "put", seed=1, ctx=ctx)
        assert e.value.status == PCF_ESINGULAR
    ok = mc_amer_result(100, 100, .05, .3, 1.0, 4096, 10, "put", seed=5, ctx=ctx)
    t = twin(orc, 100, 100, .05, .3, 1.0, 4096, 10, -1, 0, 5)
    assert abs(ok.sums[0] - t[0]) <= 3e-4 * abs(t[0])


@pytest.mark.parametrize("N,M", [(65536, 50), (3_200_000, 10)])
def test_amer_barrier_timeout_then_recovers(ctx, N, M):
    """The bounded group barrier of the cooperative sweep (and of the
    streaming sweep at 3.2e6 paths) is made unable to complete through the
    test hook: the call returns PCF_ETIMEOUT instead of hanging, and the next
    normal call on the same context gives the same bits as before."""
    from parcompfin_gb300 import mc_amer_result
    from parcompfin_gb300._lib import PCF_ETIMEOUT, PcfError
    args = (100, 100, .05, .3, 1.0, N, M, "put")
    ctx.set_test_barrier(0)
    before = mc_amer_result(*args, seed=5, ctx=ctx)
    ctx.set_test_barrier(1, 2000)
    try:
        with pytest.raises(PcfError) as e:
            mc_amer_result(*args, seed=5, ctx=ctx)
        assert e.value.status == PCF_ETIMEOUT
    finally:
        ctx.set_test_barrier(0)
    after = mc_amer_result(*args, seed=5, ctx=ctx)
    assert list(after.sums) == list(before.sums)


def test_lattice_barrier_timeout_then_recovers(orc, ctx):
    from parcompfin_gb300 import binom_vanilla_amer
    from parcompfin_gb300._lib import PCF_ETIMEOUT, PcfError
    ref = orc.ref_binom_vanilla_amer(100, 100, .05, .3, 1.0, 20000, -1.0)
    ctx.set_test_barrier(1, 2000)
    try:
        with pytest.raises(PcfError) as e:
            binom_vanilla_amer(100, 100, .05, .3, 1.0, 20000, "put", ctx=ctx)
        assert e.value.status == PCF_ETIMEOUT
    finally:
        ctx.set_test_barrier(0)
    assert binom_vanilla_amer(100, 100, .05, .3, 1.0, 20000, "put", ctx=ctx) == ref


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
