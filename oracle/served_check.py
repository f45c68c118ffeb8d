"""Served prices against the reference's pricers (TEST INFRASTRUCTURE ONLY).

Used by tests/test_gpu_serve.py and by the CPU-baseline leg of bench.py as
the checker of the engine's served prices; nothing on the product path
imports it. Each served result is compared with an independent price of the
same contract:

  European  Black-Scholes (orc_bs_price): z = (price - BS) / SE.
  Asian     the reference's own estimator (src/mc_asia_omp.cpp:5-48, the
            running sum I += S (1 + r dt/2 + sigma dB/2), mt19937 draws) with
            its sample variance (ref_mc_asia_omp_stats), at a path count
            bounded by a path-step budget: z over the combined SE. The
            engine's control-variate mean (the geometric average's closed
            form) is checked against the oracle's closed form to 1e-9.
  Basket    the oracle's FP64 restatement (twin_mc_basket) on an independent
            Philox stream with the same control-variate estimator: z over
            the combined SE (the reference's basket needs Eigen and Boost,
            which are absent). The geometric-basket closed form the engine
            uses is checked against orc_geo_basket_price to 1e-9.
  American  the reference's own lattice (src/binom_vanilla_amer.cpp:5-40,
            ref_binom_vanilla_amer, 2000 steps), which prices the American
            option; Longstaff-Schwartz on 50 exercise dates with a quadratic
            basis sits below it by its own bias (0.26-0.67 % for
            K in [90, 110], sigma in [0.2, 0.4], measured with the FP64
            restatement of the same algorithm at 2^16-2^18 paths). The bar
            is lattice (1 - 1 %) - 3 SE <= price <= lattice + 3 SE + 2e-3.
            The FP64 twin on the identical Philox draws (twin_mc_amer, same
            seed, stream and path count) must agree within 1e-3 relative:
            the policy audit (tests/test_gpu_amer.py) shows that the first
            decision in which the two differ is a boundary flip and that each
            flip moves the later regressions, which flips further paths (a
            cascade measured at 1e-5 to 4e-4 of the price at 2^16 paths).

Per kind the summary carries the number checked, how many fall outside
3 combined standard errors, the count expected there by chance
(0.27 % of those checked), and the largest |z|.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

Z3 = 3.0
AMER_BIAS = 0.01           # relative allowance below the lattice (see module docstring)
AMER_LATTICE_STEPS = 2000
AMER_TWIN_REL = 1e-3


def _cv_estimate(s, n, mu, disc):
    """The engine's control-variate estimator from moment sums over n samples."""
    yb, gb = s[0] / n, s[2] / n
    vy = s[1] / n - yb * yb
    vg = s[3] / n - gb * gb
    cov = s[4] / n - yb * gb
    b = cov / vg if vg > 0 else 0.0
    p = yb - b * (gb - mu)
    var = max(vy - 2 * b * cov + b * b * vg, 0.0) * n / (n - 1)
    return disc * p, disc * math.sqrt(var / n)


def _kind(q) -> str:
    return {0: "eur", 1: "asia", 2: "basket", 3: "amer"}[int(q["method"])]


def check(orc, reqs, results, *, threads=0, asia_path_steps=2e7, basket_flops=2e9,
          max_per_kind=None, amer_twin=True) -> dict:
    """Compare each served result with its reference price.

    reqs: request dicts (parcompfin_gb300.request), results: McResult-like
    objects with price, std_error, n_paths, sums, cv_mean. Returns a summary
    per kind plus the list of per-request records."""
    out = {}
    rows = []
    counts = {}
    for q, r in zip(reqs, results):
        k = _kind(q)
        counts[k] = counts.get(k, 0) + 1
        if max_per_kind and counts[k] > max_per_kind:
            continue
        if not (r.price == r.price) or r.std_error != r.std_error:
            rows.append({"kind": k, "status": "nan"})
            continue
        pf = int(q["payoff_fun"])
        S0, E, rr, sig, T = q["S0"], q["E"], q["r"], q["sigma"], q["T"]
        rec = {"kind": k, "price": r.price, "se": r.std_error, "n_paths": r.n_paths}
        if k == "eur":
            ref = orc.orc_bs_price(S0, E, rr, sig, T, pf)
            rec.update(ref=ref, ref_se=0.0)
        elif k == "asia":
            M = int(q["M"])
            n = int(max(2000, min(r.n_paths, asia_path_steps / M)))
            st = (C.c_double * 2)()
            orc.ref_mc_asia_omp_stats(S0, E, rr, sig, T, n, M, float(pf), 977 + len(rows),
                                      int(threads), st)
            rec.update(ref=st[0], ref_se=st[1], ref_paths=n)
            w = (C.c_double * (M + 1))()
            orc.orc_asian_geo_weights(M, int(q.get("mode", 0)), w)
            exact = orc.orc_geo_weighted_price(S0, E, rr, sig, T, M, w, pf, None) * math.exp(rr * T)
            rec["cv_mean_rel_err"] = abs(r.cv_mean - exact) / max(abs(exact), 1e-300)
        elif k == "basket":
            d = int(q["assets"])
            s0 = list(q["basket_S0"]) if q.get("basket_S0") else [S0] * d
            sg = list(q["basket_sigma"]) if q.get("basket_sigma") else [sig] * d
            if q.get("corr"):
                corr = np.array(q["corr"], dtype=float).reshape(d, d)
            else:
                corr = np.full((d, d), float(q["rho"]))
                np.fill_diagonal(corr, 1.0)
            L = np.linalg.cholesky(corr).ravel()
            ts = math.sqrt(T) if q.get("scale_by_sqrt_T") else 1.0
            n = int(max(4096, min(r.n_paths, basket_flops / (d * d + 8 * d))))
            A = C.c_double * d
            s = (C.c_double * 5)()
            orc.twin_mc_basket(d, A(*s0), A(*sg), (C.c_double * (d * d))(*L), rr, T, ts, E, n, pf,
                               9091, 0x5EED0000 + len(rows), s)
            mu = orc.orc_geo_basket_price(d, A(*s0), A(*sg), (C.c_double * (d * d))(*corr.ravel()),
                                          rr, T, ts, E, pf, None) * math.exp(rr * T)
            p, se = _cv_estimate(list(s), n, mu, math.exp(-rr * T))
            rec.update(ref=p, ref_se=se, ref_paths=n)
            rec["cv_mean_rel_err"] = abs(r.cv_mean - mu) / max(abs(mu), 1e-300)
        else:
            M = int(q["M"])
            lat = orc.ref_binom_vanilla_amer(S0, E, rr, sig, T, AMER_LATTICE_STEPS, float(pf))
            lo = lat * (1 - AMER_BIAS) - Z3 * r.std_error
            hi = lat + Z3 * r.std_error + 2e-3
            rec.update(ref=lat, ref_se=0.0, lattice_ok=bool(lo <= r.price <= hi),
                       rel_to_lattice=(r.price - lat) / lat)
            if amer_twin:
                s6 = (C.c_double * 6)()
                orc.twin_mc_amer(S0, E, rr, sig, T, int(r.n_paths), M, pf, int(q.get("mode", 0)),
                                 int(q["seed"]), int(q["stream"]), s6)
                rec["twin_rel"] = abs(r.sums[0] - s6[0]) / max(abs(s6[0]), 1e-300)
        if k != "amer":
            se = math.hypot(rec["se"], rec["ref_se"])
            rec["z"] = (rec["price"] - rec["ref"]) / se if se > 0 else float("inf")
        rows.append(rec)
    for k in ("eur", "asia", "basket", "amer"):
        rk = [x for x in rows if x["kind"] == k]
        if not rk:
            continue
        good = [x for x in rk if "price" in x]
        summ = {"checked": len(good), "nan": len(rk) - len(good)}
        if k == "amer":
            summ["outside_bar"] = sum(not x["lattice_ok"] for x in good)
            summ["rel_to_lattice_min"] = min((x["rel_to_lattice"] for x in good), default=None)
            summ["rel_to_lattice_max"] = max((x["rel_to_lattice"] for x in good), default=None)
            tw = [x["twin_rel"] for x in good if "twin_rel" in x]
            if tw:
                summ["twin_max_rel"] = max(tw)
                summ["twin_outside"] = sum(t > AMER_TWIN_REL for t in tw)
        else:
            zs = [abs(x["z"]) for x in good]
            summ["outside_3se"] = sum(z > Z3 for z in zs)
            summ["expected_outside_3se"] = round(0.0027 * len(good), 2)
            summ["max_abs_z"] = max(zs) if zs else None
            cm = [x["cv_mean_rel_err"] for x in good if "cv_mean_rel_err" in x]
            if cm:
                summ["cv_mean_max_rel_err"] = max(cm)
        out[k] = summ
    return {"per_kind": out, "rows": rows}
