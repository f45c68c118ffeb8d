"""The LSM policy audit (oracle twin_mc_amer_audit) checked on the CPU.

A record made by the oracle's FP32 emulation of the kernel's sweep
(orc_emulate_lsm_record: the twin's paths rounded to FP32, the kernel's
decision formulas, FP64 regressions rounded to FP32 coefficients) passes
the audit; the same record with a mistake planted in it (an exercise date,
a coefficient, a regression sum) fails the corresponding check. This is the
audit the GPU tests run on the kernel's own record (tests/test_gpu_amer.py).
"""
import ctypes as C

import numpy as np
import pytest

KEYS = ["r1_tau_mismatch", "r1_mode_mismatch", "sums_rel_err", "fit_err_over_E",
        "fit_err_solve_over_E", "fp64_coef_flips", "fp64_coef_flip_margin",
        "price_rel_err_same_policy", "cv_rel_err_same_policy", "max_du", "r2_flips",
        "r2_unexplained", "r2_tau_diff", "r2_price_rel", "gpu_vs_fp64_value_of_gpu_policy",
        "r3_tau_diff", "r3_price_rel", "r3_cv_rel", "r2_flip_margin_over_E", "regression_dates",
        "itm_path_dates", "r4_tau_diff", "r4_price_rel", "r3_vs_r4_tau_diff",
        "r3_vs_r4_price_rel", "r4_first_divergence_date", "r4_first_divergence_paths",
        "r4_first_divergence_margin_over_E", "r4_first_divergence_fit_diff_over_E"]
ARGS = (100.0, 100.0, .05, .3, 1.0)


def record(orc, N, M, pf, seed=5):
    coef = np.zeros((M, 4), np.float32)
    sums = np.zeros((M, 8))
    tau = np.zeros(N, np.uint16)
    u = np.zeros((M, N), np.float32)
    mom = np.zeros(5)
    fp, dp = C.POINTER(C.c_float), C.POINTER(C.c_double)
    orc.orc_emulate_lsm_record(*ARGS, N, M, pf, seed, 0, coef.ctypes.data_as(fp),
                               sums.ctypes.data_as(dp), tau.ctypes.data_as(C.POINTER(C.c_uint16)),
                               u.ctypes.data_as(fp), mom.ctypes.data_as(dp))
    return coef, sums, tau, u, mom


def audit(orc, N, M, pf, rec, seed=5):
    coef, sums, tau, u, mom = rec
    rep = (C.c_double * 29)()
    fp, dp = C.POINTER(C.c_float), C.POINTER(C.c_double)
    orc.twin_mc_amer_audit(*ARGS, N, M, pf, 0, seed, 0, coef.ctypes.data_as(fp),
                           sums.ctypes.data_as(dp), tau.ctypes.data_as(C.POINTER(C.c_uint16)),
                           u.ctypes.data_as(fp), mom.ctypes.data_as(dp), rep)
    return dict(zip(KEYS, rep))


@pytest.mark.parametrize("pf", [-1, 1])
def test_audit_accepts_a_consistent_record(orc, pf):
    N, M = 4096, 10
    a = audit(orc, N, M, pf, record(orc, N, M, pf))
    assert a["r1_tau_mismatch"] == 0 and a["r1_mode_mismatch"] == 0, a
    assert a["sums_rel_err"] < 1e-12 and a["fit_err_solve_over_E"] < 1e-6, a
    assert a["price_rel_err_same_policy"] < 1e-12, a
    assert a["max_du"] < 1e-6 and a["r2_unexplained"] == 0, a
    assert a["regression_dates"] == M - 1, a


def test_audit_catches_a_wrong_exercise_date(orc):
    N, M = 4096, 10
    coef, sums, tau, u, mom = record(orc, N, M, -1)
    k = int(np.argmax(tau < M))  # a path that exercised early
    assert tau[k] < M
    tau[k] = M
    a = audit(orc, N, M, -1, (coef, sums, tau, u, mom))
    assert a["r1_tau_mismatch"] == 1, a


def test_audit_catches_a_wrong_coefficient(orc):
    N, M = 4096, 10
    coef, sums, tau, u, mom = record(orc, N, M, -1)
    coef[5, 1] += 5.0  # date 5's constant term, 5 % of the strike too high
    a = audit(orc, N, M, -1, (coef, sums, tau, u, mom))
    assert a["fit_err_over_E"] > 1e-2 and a["r1_tau_mismatch"] > 0, a


def test_audit_catches_a_wrong_regression_sum(orc):
    N, M = 4096, 10
    coef, sums, tau, u, mom = record(orc, N, M, 1)
    sums[3, 6] *= 1.01
    a = audit(orc, N, M, 1, (coef, sums, tau, u, mom))
    assert a["sums_rel_err"] > 5e-3, a
