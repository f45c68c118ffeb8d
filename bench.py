"""Throughput benchmark of the GB300 pricing engine.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload NAME] [--no-cpu]

Prints one JSON line (rank 0). A step is one pass of the engine over one
batch of synthetic pricing requests (--workload; parcompfin_gb300/workloads.py
builds the request sets):

  mixed   (default) the served mixed stream: 1000 requests per step, 30 %
          European, 20 % basket (2..32 assets), 30 % Asian, 20 % American put,
          each priced to a 5e-4 relative standard error with its control
          variate (path counts from an untimed pilot).
  eur     European call S0=K=100 r=.05 sigma=.2 T=1 (mc_eur,
          src/mc_eur.cpp:5-27), 2^28 paths per step.
  asia    Asian book: 256 Asian calls, M in {12,52,252}, N log-uniform in
          2^16..2^22 (mc_asia, src/mc_asia.cpp:5-40), one persistent launch,
          geometric control variate.
  basket  basket book: baskets of 4, 16, 64 assets, 2^22 paths each
          (mc_eur_multi, src/mc_eur_multi.cpp:6-35).
  lsm     American put by Longstaff-Schwartz, N = 2^20 paths, 50 dates
          (mc_amer, src/mc_amer.cpp:5-114).
  binom   binomial book: 1024 closed-binomial contracts, N uneven in 1e3..2e5
          (binom_embar, src/binom_embar.cpp:5-50), reference rounding order.
  amerbatch  64 American puts of 2^16 paths and 50 dates in one cluster launch
          (the mixed stream's American distribution).

value         units/s with the request tables already on the device, timed with
              CUDA events on the engine's stream around each step, L2 flushed
              between steps (outside the events).
e2e           the same units/s through the public C ABI from host parameters to
              host results (copies included), wall clock; for the mixed stream
              the serving loop (pcf_serve_trace), its pilot included.
roofline      the dominant kernel against its bound (SFU for the path
              generators, HBM for the LSM path matrix).
cpu_baseline  the reference's OpenMP code on all host cores (oracle/_ref where
              the reference was compiled on this machine, else the oracle's
              restatement of the same loops), on a bounded sample.
--impl reference prints that CPU arm alone.

Multi-GPU (torchrun): every rank prices its own copy of the batch with its own
Philox streams (weak scaling, no collective on the data path); value = all
ranks' units / the slowest rank's time.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

L2_FLUSH_BYTES = 256 << 20  # > the 129 MB L2 of a GB300
# The cache policy, stated in both arms' config (the same words, so that the
# two arms' configs compare equal).
L2_POLICY = ("GPU arm: L2 flushed between steps by a 256 MiB write outside the step's CUDA "
             "events; CPU arm: no device cache")


def _sfu_roofline(sfu_per_unit, units, ms, sms, sm_mhz):
    peak = sms * 16 * sm_mhz * 1e6 / 1e9  # G MUFU ops/s: 16 per SM per clock
    ach = sfu_per_unit * units / (ms * 1e-3) / 1e9
    return {"bound": "sfu", "achieved": ach, "peak": peak, "unit": "G SFU op/s",
            "frac": ach / peak, "traffic": None,
            "peak_source": f"{sms} SMs x 16 MUFU/clk x {sm_mhz:.0f} MHz (median SM clock "
                           "under load); compute-bound kernel, no HBM traffic to speak of"}


def _fp32_roofline(flop_per_unit, units, ms, sms, sm_mhz):
    peak = sms * 128 * 2 * sm_mhz * 1e6 / 1e12  # TFLOP/s: 128 FP32 FMA lanes per SM
    ach = flop_per_unit * units / (ms * 1e-3) / 1e12
    return {"bound": "fp32", "achieved": ach, "peak": peak, "unit": "TFLOP/s",
            "frac": ach / peak, "traffic": None,
            "peak_source": f"{sms} SMs x 128 FMA lanes x 2 flop x {sm_mhz:.0f} MHz (median SM "
                           "clock under load)"}


# --------------------------------------------------------------------------
# workloads
# --------------------------------------------------------------------------
# DRAM bytes per algorithmic byte of the American cluster kernel, from one
# `ncu --set full` capture of its launch on the amerbatch workload (64 puts,
# 2^16 paths, 50 dates; dram__bytes_read.sum + dram__bytes_write.sum =
# 1637.4 MB for 1677.7 MB algorithmic). Traffic grows with the path-dates, so
# other launches of the kernel scale by it.
LSM_TRAFFIC_PER_ALG_BYTE = 1637.4 / 1677.7
# What bounds the American cluster kernel, from the same capture.
LSM_LIMITER = ("the per-date regression chain, not HBM: each date is a fused pass over the "
               "CTA's paths, then one warp reduces, exchanges the sums across the cluster and "
               "solves while the other warps wait (ncu, 64-put launch: 56 % of issue slots "
               "busy, DRAM 38 % of peak, barrier the top stall)")


class EurWorkload:
    name = "eur"
    metric = "MC paths/sec (European GBM, S0=K=100, r=.05, sigma=.2, T=1 call)"
    unit = "paths/s"
    paths = 1 << 28
    dominant = "mc_kernel<0,...> (European)"

    def __init__(self, rank):
        import parcompfin_gb300 as pcf
        self.reqs = [pcf.request("eur", 100.0, 100.0, 0.05, 0.2, 1.0, self.paths, "call",
                                 seed=42, stream=rank)]

    def setup(self, ctx):
        import parcompfin_gb300 as pcf
        self.plan = pcf.Plan(self.reqs, ctx=ctx)

    def tune_requests(self):
        return self.reqs

    def step(self, ctx):
        self.plan.launch()

    def finish(self, ctx):
        r = self.plan.results()
        return {"price": r[0].price_plain, "std_error": r[0].std_error_plain}

    def e2e(self, ctx):
        # pcf_price_batch on host buffers: the request records (packed once,
        # like a caller's own input array) in, the results out, H2D tables and
        # D2H moments inside the call.
        from parcompfin_gb300 import _lib, api
        n = len(self.reqs)
        if not hasattr(self, "_e2e_in"):
            arr, keep = api._pack(self.reqs)
            self._e2e_in = (arr, keep, (_lib.McResult * n)())
        arr, _, out = self._e2e_in
        _lib.check(_lib.load().pcf_price_batch(api._h(ctx), n, arr, out))
        return C.sizeof(_lib.McRequest) * n, C.sizeof(_lib.McResult) * n

    def units(self):
        return float(self.paths)

    def config(self):
        return {"workload": "eur: European call S0=K=100 r=0.05 sigma=0.2 T=1, 2^28 paths/step, "
                            "Philox seed 42", "paths_per_step": self.paths, "contracts_per_step": 1}

    def roofline(self, ms, sms, mhz):
        # 3 SFU ops per path: 1/2 lg2 + 1/2 sqrt + 1/2 sin + 1/2 cos + 1 ex2
        return _sfu_roofline(3.0, self.units(), ms, sms, mhz)

    def cpu_reference(self, threads, budget_s):
        from oracle import loader
        ref = loader.load_ref("mc_eur_omp")
        orc = loader.load()
        if ref is not None:
            kind = "reference"
            run = lambda n: ref(100.0, 100.0, 0.05, 0.2, 1.0, n, 0, 1.0, threads, 42)
        else:
            kind = "port"
            run = lambda n: orc.ref_mc_eur_omp(100.0, 100.0, 0.05, 0.2, 1.0, n, 1.0, 42, threads)
        n = 1 << 20
        t0 = time.perf_counter()
        run(n)
        dt = max(time.perf_counter() - t0, 1e-6)
        n = int(min(2**31 - 1, max(n, n * budget_s / dt)))
        t0 = time.perf_counter()
        price = run(n)
        dt = time.perf_counter() - t0
        return {"value": n / dt, "unit": self.unit, "cores": threads, "kind": kind,
                "sample": f"mc_eur_omp on {n} paths of the ATM European call, price {price:.6f}, "
                          f"{dt:.2f} s"}


class AsiaWorkload:
    name = "asia"
    metric = "MC paths/sec (Asian batch, 256 contracts)"
    unit = "paths/s"
    dominant = "mc_kernel<1,...> (Asian, persistent)"

    def __init__(self, rank):
        import parcompfin_gb300 as pcf
        from parcompfin_gb300 import workloads
        self.cs = workloads.asian_book()
        self.reqs = [pcf.request("asia", c["S0"], c["E"], c["r"], c["sigma"], c["T"], c["N"], "call",
                                 M=c["M"], mode=0, use_cv=True, seed=13, stream=rank * 4096 + i)
                     for i, c in enumerate(self.cs)]

    setup = EurWorkload.setup
    tune_requests = EurWorkload.tune_requests
    step = EurWorkload.step

    def finish(self, ctx):
        r = self.plan.results()
        worst = max(x.std_error_cv / x.price_cv for x in r if x.price_cv > 0)
        return {"contracts": len(r), "worst_rel_se_cv": worst}

    e2e = EurWorkload.e2e

    def units(self):
        return float(sum(c["N"] for c in self.cs))

    def path_steps(self):
        return float(sum(c["N"] * c["M"] for c in self.cs))

    def config(self):
        return {"workload": "asia: 256 Asian calls (seed 13), K~U[90,110], "
                            "sigma~U[.15,.4], T~U[.5,2], M in {12,52,252}, N=2^U[16,22], "
                            "geometric control variate, one persistent launch",
                "paths_per_step": self.units(), "path_steps_per_step": self.path_steps(),
                "contracts_per_step": len(self.cs)}

    def roofline(self, ms, sms, mhz):
        # 3 SFU ops per path-step (normal: 2, ex2: 1)
        return _sfu_roofline(3.0, self.path_steps(), ms, sms, mhz)

    def cpu_reference(self, threads, budget_s):
        from oracle import loader
        ref = loader.load_ref("mc_asia_omp")
        orc = loader.load()
        kind = "reference" if ref is not None else "port"
        done_paths = done_steps = 0
        t0 = time.perf_counter()
        for c in self.cs:
            n = max(1000, c["N"] // 64)
            if ref is not None:
                ref(c["S0"], c["E"], c["r"], c["sigma"], c["T"], n, c["M"], 1.0, threads, 13)
            else:
                orc.ref_mc_asia_omp(c["S0"], c["E"], c["r"], c["sigma"], c["T"], n, c["M"], 1.0,
                                    13, threads)
            done_paths += n
            done_steps += n * c["M"]
            if time.perf_counter() - t0 > budget_s:
                break
        dt = time.perf_counter() - t0
        # Paths per second at this batch's mix of step counts.
        rate_steps = done_steps / dt
        value = rate_steps * self.units() / self.path_steps()
        return {"value": value, "unit": self.unit, "cores": threads, "kind": kind,
                "sample": f"mc_asia_omp on the Asian book at N/64 ({done_paths} paths, "
                          f"{done_steps} path-steps, {dt:.2f} s); paths/s scaled to the batch's "
                          "step mix"}


class BasketWorkload:
    name = "basket"
    metric = "MC paths/sec (basket, d in {4, 16, 64})"
    unit = "paths/s"
    dominant = "mc_basket_tc_kernel<64,...> (basket, L z on the tensor cores)"

    def __init__(self, rank):
        import parcompfin_gb300 as pcf
        from parcompfin_gb300 import workloads
        self.cs = workloads.basket_book()
        self.reqs = [pcf.request("basket", 100.0, c["E"], c["r"], 0.2, c["T"], c["N"], "call",
                                 assets=c["assets"], basket_S0=c["basket_S0"],
                                 basket_sigma=c["basket_sigma"], corr=c["corr"], use_cv=True,
                                 scale_by_sqrt_T=True, seed=11, stream=rank * 16 + i)
                     for i, c in enumerate(self.cs)]

    setup = EurWorkload.setup
    tune_requests = EurWorkload.tune_requests
    step = EurWorkload.step

    def finish(self, ctx):
        r = self.plan.results()
        self.last_results = r
        return {"prices_cv": [x.price_cv for x in r]}

    def reference_check(self, threads):
        """Error of each contract against the FP64 harness (the oracle's twin
        on the identical Philox draws, the same Cholesky factor), all five
        moment sums, at the full 2^22 paths."""
        import numpy as np
        from oracle import loader
        orc = loader.load()
        per = []
        for i, (c, r) in enumerate(zip(self.cs, self.last_results)):
            d = c["assets"]
            L = np.linalg.cholesky(np.array(c["corr"])).ravel()
            s = (C.c_double * 5)()
            A = C.c_double * d
            orc.twin_mc_basket(d, A(*c["basket_S0"]), A(*c["basket_sigma"]),
                               (C.c_double * (d * d))(*L), c["r"], c["T"], math.sqrt(c["T"]),
                               c["E"], c["N"], 1, 11, self.reqs[i]["stream"], s)
            err = max(abs(a - b) / abs(b) for a, b in zip(r.sums, s) if b != 0)
            per.append({"assets": d, "max_rel_err_moments": err})
        return {"fp64_harness": per,
                "fp64_harness_max_rel_err": max(x["max_rel_err_moments"] for x in per)}

    e2e = EurWorkload.e2e

    def units(self):
        return float(sum(c["N"] for c in self.cs))

    def config(self):
        return {"workload": "basket: d in {4,16,64}, S0=K=100, r=.03, T=1, "
                            "sigma_i~U[.15,.35], corr 0.7 equicorr(.3) + 0.3 Wishart(d,d+2) "
                            "seed 11, 2^22 paths each, geometric-basket control variate",
                "paths_per_step": self.units(), "contracts_per_step": len(self.cs)}

    def roofline(self, ms, sms, mhz):
        # Per path: 3 SFU ops per asset (normals, exp) on the CUDA cores. The
        # L z product (d(d+1) flops) runs on the tensor cores for d > 16
        # (3xTF32 tcgen05.mma), so the CUDA-core bound is the random stream:
        # SFU ops and issue. "fp32_equivalent" counts the whole product as if
        # it ran on the FP32 pipe: d(d+1) + 7.5 d + 11 flops per path.
        sfu = sum(c["N"] * 3.0 * c["assets"] for c in self.cs) / self.units()
        d_flop = lambda d: d * (d + 1) + 7.5 * d + 11
        flop = sum(c["N"] * d_flop(c["assets"]) for c in self.cs) / self.units()
        a = _sfu_roofline(sfu, self.units(), ms, sms, mhz)
        b = _fp32_roofline(flop, self.units(), ms, sms, mhz)
        a["fp32_equivalent"] = {k: b[k] for k in ("achieved", "peak", "unit", "frac")}
        return a

    def cpu_reference(self, threads, budget_s):
        # The reference's basket needs Eigen and Boost (include/mvn.h), absent
        # here: time the oracle's FP64 restatement on all cores instead.
        from oracle import loader
        orc = loader.load()
        import numpy as np
        done = 0
        t0 = time.perf_counter()
        for c in self.cs:
            d = c["assets"]
            L = np.linalg.cholesky(np.array(c["corr"])).ravel()
            A = C.c_double * d
            s = (C.c_double * 5)()
            n = 1 << 15
            orc.twin_mc_basket(d, A(*c["basket_S0"]), A(*c["basket_sigma"]),
                               (C.c_double * (d * d))(*L), c["r"], c["T"], math.sqrt(c["T"]),
                               c["E"], n, 1, 11, 0, s)
            done += n
        dt = time.perf_counter() - t0
        # Paths of the three contracts come in equal numbers in the batch.
        return {"value": done / dt, "unit": self.unit, "cores": threads,
                "kind": "port",
                "sample": f"oracle FP64 basket restatement (the reference's Eigen/Boost build is "
                          f"unavailable), 2^15 paths per contract, {dt:.2f} s"}


class LsmWorkload:
    name = "lsm"
    metric = "MC paths/sec (American put, Longstaff-Schwartz)"
    unit = "paths/s"
    N, M = 1 << 20, 50
    dominant = "lsm_kernel"

    def __init__(self, rank):
        self.rank = rank

    def setup(self, ctx):
        pass

    def step(self, ctx):
        import parcompfin_gb300 as pcf
        self.res = pcf.mc_amer_result(100.0, 100.0, 0.05, 0.3, 1.0, self.N, self.M, "put",
                                      seed=1 + self.rank, ctx=ctx)

    def finish(self, ctx):
        return {"price": self.res.price, "std_error": self.res.std_error}

    def e2e(self, ctx):
        self.step(ctx)
        return 4 * (self.M + 1), C.sizeof(C.c_double) * 5 + 16

    def units(self):
        return float(self.N)

    def config(self):
        return {"workload": "lsm: American put S0=K=100 r=.05 sigma=.3 T=1, 50 exercise dates, "
                            "2^20 paths (antithetic), basis {1,x,x^2}",
                "paths_per_step": self.N, "dates": self.M, "contracts_per_step": 1}

    def roofline(self, ms, sms, mhz, peaks):
        alg = 8.0 * self.N * self.M  # one FP32 write + one FP32 read per path-date
        ach = alg / (ms * 1e-3) / 1e9
        peak = peaks.get("hbm_gbs", 6800.0)
        return {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s",
                "frac": ach / peak, "traffic": None,
                "limiter": "the per-date chain of one contract spread over every SM: each of "
                           "the 49 dates ends with an exchange of the regression sums across "
                           "the whole grid (clusters, then their leaders in global memory) "
                           "before the next date can start",
                "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)" if peaks else
                               "fallback 6.8 TB/s"}

    def cpu_reference(self, threads, budget_s):
        from oracle import loader
        ref = loader.load_ref("mc_amer_omp")
        orc = loader.load()
        n = 1 << 16
        t0 = time.perf_counter()
        if ref is not None:
            kind = "reference"
            ref(100.0, 100.0, 0.05, 0.3, 1.0, n, self.M, -1.0, threads, 1)
        else:
            kind = "port"
            orc.ref_mc_amer_omp(100.0, 100.0, 0.05, 0.3, 1.0, n, self.M, -1.0, 1, threads)
        dt = time.perf_counter() - t0
        return {"value": n / dt, "unit": self.unit, "cores": threads, "kind": kind,
                "sample": f"mc_amer_omp on {n} paths, 50 dates, {threads} threads, {dt:.2f} s"}


class BinomWorkload:
    name = "binom"
    metric = "contracts/sec (closed binomial sum, 1024 contracts)"
    unit = "contracts/s"
    dominant = "binom_kernel"

    def __init__(self, rank):
        from parcompfin_gb300 import workloads
        self.cs = workloads.binom_book()

    def setup(self, ctx):
        pass

    def step(self, ctx):
        import parcompfin_gb300 as pcf
        self.prices = pcf.binom_embar_batch(self.cs, mode="reference", ctx=ctx)

    def finish(self, ctx):
        return {"first_prices": self.prices[:3]}

    def e2e(self, ctx):
        self.step(ctx)
        return 48 * len(self.cs), 8 * len(self.cs)

    def units(self):
        return float(len(self.cs))

    def config(self):
        return {"workload": "binom: 1024 contracts (seed 7), K~U[80,120], "
                            "r~U[.01,.06], sigma~U[.1,.5], T~U[.25,2], call/put 50/50, "
                            "N~U{1000..200000}, reference rounding order",
                "contracts_per_step": len(self.cs)}

    def roofline(self, ms, sms, mhz, peaks=None):
        return {"bound": "latency", "achieved": None, "peak": None, "unit": None, "frac": None,
                "traffic": None,
                "note": "FP64 and L2-latency bound binary searches over per-binade prefix "
                        "tables; no HBM or tensor bound applies"}

    def cpu_reference(self, threads, budget_s):
        from oracle import loader
        ref = loader.load_ref("binom_embar_omp")
        orc = loader.load()
        kind = "reference" if ref is not None else "port"
        # The full batch is ~25 CPU-hours (O(N^2) per contract). Time contracts
        # of growing N, fit a * N^2, extrapolate to the batch (labelled).
        samples = []
        t_all = time.perf_counter()
        for N in (1000, 2000, 4000, 8000, 12000):
            t0 = time.perf_counter()
            if ref is not None:
                ref(100.0, 100.0, 0.03, 0.3, 1.0, N, 0, 1.0, threads)
            else:
                orc.ref_binom_embar_omp(100.0, 100.0, 0.03, 0.3, 1.0, N, 1.0, threads)
            samples.append((N, time.perf_counter() - t0))
            if time.perf_counter() - t_all > budget_s:
                break
        a = sum(t * N * N for N, t in samples) / sum(N ** 4 for N, _ in samples)
        total = sum(a * c[5] ** 2 for c in self.cs)
        return {"value": len(self.cs) / total, "unit": self.unit, "cores": threads, "kind": kind,
                "sample": f"binom_embar_omp timed at N in {[n for n, _ in samples]}, fit "
                          f"t = {a:.3e} N^2 s, extrapolated to the 1024-contract batch "
                          f"({total / 3600:.1f} h)"}


class MixedWorkload:
    """The served mixed stream (1000 requests: European, basket, Asian and American)
    at a fixed relative standard error."""
    name = "mixed"
    metric = ("MC paths/sec at fixed std-error (5e-4 of price), mixed request stream; "
              "p50/p99 latency served")
    unit = "paths/s"
    dominant = "lsm_cluster_kernel (American, one cluster per contract)"
    R = 1000             # requests per step
    TARGET = 5e-4        # relative standard error
    LOADS = (1000, 10000, 50000)             # offered requests/s, 1 s of arrivals each
    SATURATION = (100000, 200000, 400000)    # beyond the engine's burst rate

    def __init__(self, rank):
        import parcompfin_gb300 as pcf
        from parcompfin_gb300 import workloads
        self.rank = rank
        self.spec = workloads.mixed_stream(self.R, seed=17 + 1000 * rank)
        self.base = [self._req(pcf, s, 0) for s in self.spec]

    @staticmethod
    def _req(pcf, s, N, use_cv=True):
        kw = dict(use_cv=use_cv, seed=4242, stream=s["id"])
        if s["kind"] == "eur":
            return pcf.request("eur", s["S0"], s["E"], s["r"], s["sigma"], s["T"], N or 4, "call", **kw)
        if s["kind"] == "asia":
            return pcf.request("asia", s["S0"], s["E"], s["r"], s["sigma"], s["T"], N or 4, "call",
                               M=s["M"], **kw)
        if s["kind"] == "basket":
            return pcf.request("basket", s["S0"], s["E"], s["r"], s["sigma"], s["T"], N or 4, "call",
                               assets=s["assets"], rho=s["rho"], basket_sigma=s["basket_sigma"],
                               scale_by_sqrt_T=True, **kw)
        return pcf.request("amer", s["S0"], s["E"], s["r"], s["sigma"], s["T"], N or 2, "put",
                           M=s["M"], **kw)

    PILOT = 1 << 14

    def _sizes(self, pilot):
        """Path counts at the target relative standard error from pilot
        estimates [(se_cv, price_cv, se_plain, price_plain)] at PILOT paths:
        the control-variate estimator for the engine, the plain one for the
        one-contract-per-launch baseline. American: [2^16, 2^21], even."""
        n0 = self.PILOT
        def need(se, price):
            if not (se > 0 and price > 0):
                return n0
            return int(min(1 << 40, max(n0, 1.05 * se * se * n0 / (self.TARGET * price) ** 2)))
        self.N, self.N_plain = [], []
        for q, (se_cv, p_cv, se_pl, p_pl) in zip(self.base, pilot):
            n_cv, n_pl = need(se_cv, abs(p_cv)), need(se_pl, abs(p_pl))
            if q["method"] == 3:
                n_cv = min(max(n_cv, 1 << 16), 1 << 21) // 2 * 2
                n_pl = min(max(n_pl, 1 << 16), 1 << 21) // 2 * 2
            else:
                n_cv = min(n_cv, 1 << 26)
                n_pl = min(n_pl, 1 << 28)
            self.N.append(n_cv)
            self.N_plain.append(n_pl)

    def setup(self, ctx):
        import parcompfin_gb300 as pcf
        # Pilot (outside the timed region): each request's path count at the
        # target standard error.
        res = pcf.price_batch([dict(q, N=self.PILOT) for q in self.base], ctx=ctx)
        self._sizes([(r.std_error_cv, r.price_cv, r.std_error_plain, r.price_plain)
                     for r in res])
        self.main = [dict(q, N=n) for q, n in zip(self.base, self.N)]
        self.plan = pcf.Plan(self.main, ctx=ctx)
        self.amer_idx = [i for i, q in enumerate(self.main) if q["method"] == 3]
        self.amer_plan = pcf.Plan([self.main[i] for i in self.amer_idx], ctx=ctx)

    def setup_cpu(self, threads):
        """The reference arm's sizing, without the engine: the same pilot on
        the oracle's FP64 restatements fed the identical Philox draws (same
        seeds and streams, PILOT paths), so the path counts are the engine's
        up to the restatements' FP64 rounding."""
        from oracle import loader
        from oracle.served_check import _cv_estimate
        import numpy as np
        orc = loader.load()
        n0 = self.PILOT
        pilot = []
        for q, sp in zip(self.base, self.spec):
            pf, S0, E, r, sig, T = q["payoff_fun"], q["S0"], q["E"], q["r"], q["sigma"], q["T"]
            s = (C.c_double * 6)()
            disc, n = math.exp(-r * T), n0
            if q["method"] == 0:
                orc.twin_mc_eur(S0, E, r, sig, T, n0, pf, q["seed"], q["stream"], s)
                mu = S0 * math.exp(r * T)
            elif q["method"] == 1:
                orc.twin_mc_asia(S0, E, r, sig, T, n0, q["M"], pf, q["mode"], q["seed"],
                                 q["stream"], s)
                w = (C.c_double * (q["M"] + 1))()
                orc.orc_asian_geo_weights(q["M"], q["mode"], w)
                mu = orc.orc_geo_weighted_price(S0, E, r, sig, T, q["M"], w, pf, None) / disc
            elif q["method"] == 2:
                d = q["assets"]
                corr = np.full((d, d), q["rho"])
                np.fill_diagonal(corr, 1.0)
                L = np.linalg.cholesky(corr).ravel()
                A = C.c_double * d
                sg = A(*sp["basket_sigma"])
                s0 = A(*([S0] * d))
                orc.twin_mc_basket(d, s0, sg, (C.c_double * (d * d))(*L), r, T, math.sqrt(T), E,
                                   n0, pf, q["seed"], q["stream"], s)
                mu = orc.orc_geo_basket_price(d, s0, sg, (C.c_double * (d * d))(*corr.ravel()), r,
                                              T, math.sqrt(T), E, pf, None) / disc
            else:
                orc.twin_mc_amer(S0, E, r, sig, T, n0, q["M"], pf, q["mode"], q["seed"],
                                 q["stream"], s)
                mu, disc, n = orc.orc_bs_price(S0, E, r, sig, T, pf), 1.0, n0 // 2
            p_cv, se_cv = _cv_estimate(list(s), n, mu, disc)
            m = s[0] / n
            se_pl = disc * math.sqrt(max(s[1] / n - m * m, 0.0) / (n - 1))
            pilot.append((se_cv, p_cv, se_pl, disc * m))
        self._sizes(pilot)

    def tune_requests(self):
        return self.main

    def step(self, ctx):
        self.plan.launch()

    def finish(self, ctx):
        res = self.plan.results()
        self.last_results = res
        rel = sorted(r.std_error / r.price for r in res if r.price > 0 and r.std_error == r.std_error)
        return {"requests": len(res), "median_rel_se": rel[len(rel) // 2], "max_rel_se": rel[-1],
                "paths_per_step": self.units()}

    def reference_check(self, threads):
        """The step's prices against the reference's pricers (oracle/served_check.py),
        on up to 40 requests of each kind."""
        from oracle import loader, served_check
        rep = served_check.check(loader.load(), self.main, self.last_results, threads=threads,
                                 max_per_kind=40)
        return rep["per_kind"]

    def e2e(self, ctx):
        # The C-ABI call of the serving loop on host buffers: the request
        # array (packed once, like a caller's own input records), pilot and
        # main passes, results back in host memory. The serving slots are the
        # context's, reserved by the first call (a warm-up step).
        import parcompfin_gb300 as pcf
        from parcompfin_gb300 import _lib, api
        n = len(self.base)
        if not hasattr(self, "_e2e_in"):
            arr, keep = api._pack(self.base)
            self._e2e_in = (arr, keep, (C.c_double * n)(*([0.0] * n)),
                            _lib.ServerConfig(self.TARGET, 1 << 14, 1 << 26, 1 << 21, 2048, 12, 0.5),
                            (_lib.ServedResult * n)(), _lib.ServerStats())
        arr, _, arrival, cfg, out, stats = self._e2e_in
        st = _lib.load().pcf_serve_trace(api._h(ctx), C.byref(cfg), n, arr, arrival, out,
                                         C.byref(stats))
        if st not in (_lib.PCF_OK, _lib.PCF_ESINGULAR):
            _lib.check(st)
        self.e2e_stats = stats
        return (C.sizeof(pcf._lib.McRequest) * n, C.sizeof(pcf._lib.ServedResult) * n)

    def e2e_units(self):
        return float(self.e2e_stats.paths)

    def units(self):
        return float(sum(self.N))

    def contracts(self):
        return float(len(self.N))

    def config(self):
        kinds = {}
        for s in self.spec:
            kinds[s["kind"]] = kinds.get(s["kind"], 0) + 1
        return {"workload": "mixed: served request stream, 1000 requests per step (seed 17): 30% European "
                            "(ATM call jittered), 20% basket d~U{2..32}, 30% Asian (Asian-book "
                            "distribution), 20% American put (LSM, 50 dates, N in 2^16..2^21); "
                            "each priced to a 5e-4 relative standard error with its control "
                            "variate",
                "requests_per_step": self.R, "kinds": kinds, "target_rel_se": self.TARGET}

    def roofline(self, ms, sms, mhz, peaks):
        import torch
        # The American sub-plan alone, timed the same way: HBM bytes of its path
        # matrices (8 B per path-date) over its kernel time.
        s = torch.cuda.ExternalStream(self.ctx_stream)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        self.amer_plan.launch()
        times = []
        for _ in range(3):
            e0.record(s)
            self.amer_plan.launch()
            e1.record(s)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
        t = min(times)
        alg = sum(8.0 * self.main[i]["N"] * self.main[i]["M"] for i in self.amer_idx)
        ach = alg / (t * 1e-3) / 1e9
        peak = peaks.get("hbm_gbs", 6800.0)
        return {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                "traffic": alg * LSM_TRAFFIC_PER_ALG_BYTE,
                "traffic_source": "ncu capture of the 64-put batch, scaled by path-dates",
                "limiter": LSM_LIMITER,
                "kernel_ms": t,
                "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)" if peaks else
                               "fallback 6.8 TB/s",
                "share_of_step": t / ms}

    def extra(self, ctx):
        """Served latency at offered loads, and the plain one-contract-per-launch path."""
        import parcompfin_gb300 as pcf
        from parcompfin_gb300 import workloads
        served, saturation = {}, {}
        for rate in self.LOADS + self.SATURATION:
            # At least one second of Poisson arrivals at each offered load.
            n = int(max(self.R, rate * 1.0))
            spec = workloads.mixed_stream(n, seed=29 + rate)
            reqs = [self._req(pcf, s, 0) for s in spec]
            arr = workloads.poisson_arrivals(n, rate, seed=31 + rate)
            out, st = pcf.serve_trace(reqs, arr, target_rel_se=self.TARGET, ctx=ctx)
            rec = {"offered_per_s": rate, "requests": n, "arrivals_s": arr[-1],
                   "p50_ms": st.p50_ms, "p99_ms": st.p99_ms, "mean_ms": st.mean_ms,
                   "max_ms": st.max_ms, "contracts_per_s": st.contracts_per_s,
                   "paths_per_s": st.paths_per_s, "batches": st.batches}
            (served if rate in self.LOADS else saturation)[str(rate)] = rec
        # Plain path: each request alone, plain estimator, at the path count the
        # plain estimator needs for the same standard error.
        k = min(60, len(self.spec))
        t0 = time.perf_counter()
        paths = 0
        for i in range(k):
            q = self.base[i]
            N = self.N_plain[i]
            paths += N
            if q["method"] == 0:
                pcf.mc_eur_result(q["S0"], q["E"], q["r"], q["sigma"], q["T"], N, q["payoff_fun"],
                                  seed=7, ctx=ctx)
            elif q["method"] == 1:
                pcf.mc_asia_result(q["S0"], q["E"], q["r"], q["sigma"], q["T"], N, q["M"],
                                   q["payoff_fun"], seed=7, ctx=ctx)
            elif q["method"] == 2:
                s = self.spec[i]
                pcf.mc_basket_result([q["S0"]] * s["assets"], s["basket_sigma"],
                                     [1.0 if a == b else s["rho"] for a in range(s["assets"])
                                      for b in range(s["assets"])], q["r"], q["T"], q["E"], N,
                                     q["payoff_fun"], seed=7, ctx=ctx)
            else:
                pcf.mc_amer_result(q["S0"], q["E"], q["r"], q["sigma"], q["T"], N, q["M"],
                                   q["payoff_fun"], seed=7, ctx=ctx)
        dt = time.perf_counter() - t0
        plain = {"contracts_per_s": k / dt, "paths_per_s": paths / dt, "sample_requests": k,
                 "note": "each request alone through its single-contract entry point, plain "
                         "estimator, at the path count the plain estimator needs for the same "
                         "5e-4 relative standard error (American capped at 2^21)"}
        return {"served": served, "saturation": saturation, "plain_gpu": plain}

    def cpu_reference(self, threads, budget_s, step=0):
        """The reference's OpenMP pricers on the host cores, for the same
        requests at the same path counts as the engine's step, extrapolated
        from a timed sample: each sampled request runs at its own parameters
        on a reduced path count n, its time per path gives the per-kind cost
        model (European per path, Asian per path-step, basket per path as a
        function of d, American per path-date), and the model prices every
        request at its N. A linear model from small n leaves out the cache
        misses of large N, so it understates the CPU time. The basket uses the
        oracle's FP64 restatement (the reference's needs Eigen and Boost)."""
        import numpy as np
        from oracle import loader
        orc = loader.load()
        refs = {k: loader.load_ref(k) for k in ("mc_eur_omp", "mc_asia_omp", "mc_amer_omp")}
        kind = "reference" if all(refs.values()) else "port"
        by = {k: [i for i, sp in enumerate(self.spec) if sp["kind"] == k]
              for k in ("eur", "asia", "basket", "amer")}
        # Per step a rotating, bounded sample of each kind.
        per = {"eur": 6, "asia": 8, "basket": 8, "amer": 3}
        if budget_s >= 5:
            per = {k: 3 * v for k, v in per.items()}
        samples = {}
        for k, idx in by.items():
            n = min(per[k], len(idx))
            off = (step * n) % max(1, len(idx))
            samples[k] = [idx[(off + j) % len(idx)] for j in range(n)]
        cost = {k: [] for k in by}  # (request, seconds per unit)
        t_all = time.perf_counter()
        for k in ("eur", "asia", "basket", "amer"):
            for i in samples[k]:
                sp, q = self.spec[i], self.base[i]
                S0, E, r, sig, T = sp["S0"], sp["E"], sp["r"], sp["sigma"], sp["T"]
                if k == "eur":
                    n = 1 << 19
                    t0 = time.perf_counter()
                    if refs["mc_eur_omp"]:
                        refs["mc_eur_omp"](S0, E, r, sig, T, n, 0, 1.0, threads, 1)
                    else:
                        orc.ref_mc_eur_omp(S0, E, r, sig, T, n, 1.0, 1, threads)
                    units = n
                elif k == "asia":
                    n = max(2000, int(4e6 / sp["M"]))
                    t0 = time.perf_counter()
                    if refs["mc_asia_omp"]:
                        refs["mc_asia_omp"](S0, E, r, sig, T, n, sp["M"], 1.0, threads, 1)
                    else:
                        orc.ref_mc_asia_omp(S0, E, r, sig, T, n, sp["M"], 1.0, 1, threads)
                    units = n * sp["M"]
                elif k == "basket":
                    d, n = sp["assets"], 1 << 14
                    corr = np.full((d, d), sp["rho"])
                    np.fill_diagonal(corr, 1.0)
                    L = np.linalg.cholesky(corr).ravel()
                    A = C.c_double * d
                    sums = (C.c_double * 5)()
                    t0 = time.perf_counter()
                    orc.twin_mc_basket(d, A(*([S0] * d)), A(*sp["basket_sigma"]),
                                       (C.c_double * (d * d))(*L), r, T, math.sqrt(T), E, n, 1,
                                       1, 0, sums)
                    units = n * (d * d + 8 * d + 20)
                else:
                    n = 1 << 14
                    t0 = time.perf_counter()
                    if refs["mc_amer_omp"]:
                        refs["mc_amer_omp"](S0, E, r, sig, T, n, sp["M"], -1.0, threads, 1)
                    else:
                        orc.ref_mc_amer_omp(S0, E, r, sig, T, n, sp["M"], -1.0, 1, threads)
                    units = n * sp["M"]
                cost[k].append(max(time.perf_counter() - t0, 1e-9) / units)
        sampled = time.perf_counter() - t_all
        unit_cost = {k: statistics.median(v) for k, v in cost.items() if v}

        def units_of(i, N):
            sp = self.spec[i]
            if sp["kind"] == "eur":
                return N
            if sp["kind"] == "basket":
                d = sp["assets"]
                return N * (d * d + 8 * d + 20)
            return N * sp["M"]

        secs = {k: sum(unit_cost[k] * units_of(i, self.N[i]) for i in idx) for k, idx in by.items()}
        total = sum(secs.values())
        paths = float(sum(self.N))
        return {"value": paths / total, "unit": self.unit, "cores": threads, "kind": kind,
                "ms_per_step": 1e3 * total, "contracts_per_s": len(self.N) / total,
                "extrapolated": True,
                "seconds_by_kind": {k: round(v, 3) for k, v in secs.items()},
                "sample": f"the reference's OpenMP pricers (mc_eur_omp, mc_asia_omp, mc_amer_omp; "
                          f"basket: the oracle's FP64 restatement) on the host cores, timed on "
                          f"{sum(len(v) for v in samples.values())} requests of the mix at their "
                          f"own parameters and reduced path counts ({sampled:.1f} s), then "
                          f"extrapolated to the same {len(self.N)} requests at the engine's path "
                          f"counts ({paths:.3e} paths): {total:.2f} s per step (extrapolated)"}


class AmerBatchWorkload:
    """The American leg of the mixed stream alone: 64 puts, one cluster each."""
    name = "amerbatch"
    metric = "MC paths/sec (American puts, batched Longstaff-Schwartz)"
    unit = "paths/s"
    dominant = "lsm_cluster_kernel"
    C, N, M = 64, 1 << 16, 50

    def __init__(self, rank):
        import random
        import parcompfin_gb300 as pcf
        rng = random.Random(41 + rank)
        self.reqs = [pcf.request("amer", 100.0, rng.uniform(90, 110), 0.05, rng.uniform(0.2, 0.4),
                                 1.0, self.N, "put", M=self.M, use_cv=True, seed=7,
                                 stream=rank * 4096 + i) for i in range(self.C)]

    setup = EurWorkload.setup
    tune_requests = EurWorkload.tune_requests
    step = EurWorkload.step
    e2e = EurWorkload.e2e

    def finish(self, ctx):
        r = self.plan.results()
        return {"median_rel_se_cv": sorted(x.std_error_cv / x.price_cv for x in r)[len(r) // 2]}

    def units(self):
        return float(self.C * self.N)

    def contracts(self):
        return float(self.C)

    def config(self):
        return {"workload": "amerbatch: 64 American puts (the mixed stream's American "
                            "distribution: K~U[90,110], sigma~U[.2,.4], r=.05, T=1, 50 "
                            "dates), 2^16 paths each, one 8-CTA cluster per contract",
                "paths_per_step": self.units(), "contracts_per_step": self.C}

    def roofline(self, ms, sms, mhz, peaks):
        alg = 8.0 * self.C * self.N * self.M
        ach = alg / (ms * 1e-3) / 1e9
        peak = peaks.get("hbm_gbs", 6800.0)
        return {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                "traffic": alg * LSM_TRAFFIC_PER_ALG_BYTE,
                "traffic_source": "ncu capture of this launch (dram bytes read + written)",
                "limiter": LSM_LIMITER,
                "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)"}

    def cpu_reference(self, threads, budget_s):
        return LsmWorkload.cpu_reference(self, threads, budget_s)


WORKLOADS = {w.name: w for w in (MixedWorkload, EurWorkload, AsiaWorkload, BasketWorkload,
                                  LsmWorkload, BinomWorkload, AmerBatchWorkload)}


# --------------------------------------------------------------------------
# helpers
# --------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during a region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = [ln.split(", ") for ln in self.lines if ln]
        if not rows:
            return None
        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [v for v in (num(r[1]) for r in rows if len(r) > 2) if v is not None]
        mx = [v for v in (num(r[2]) for r in rows if len(r) > 2) if v is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4)
                          if len(r) > 5 + i and r[5 + i].strip() == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons, "samples": len(rows)}


def measured_peaks() -> dict:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f)
    return {}


def dist_env():
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def run_reference(args, wl_cls):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    wl = wl_cls(0)
    if hasattr(wl, "setup_cpu"):
        wl.setup_cpu(threads)
    vals, ms_vals, sample = [], [], None
    for i in range(args.warmup + args.steps):
        if hasattr(wl, "setup_cpu"):
            r = wl.cpu_reference(threads, budget_s=2.0, step=i)
        else:
            r = wl.cpu_reference(threads, budget_s=2.0)
        if i >= args.warmup:
            vals.append(r["value"])
            ms_vals.append(r.get("ms_per_step", 1e3 * wl.units() / r["value"]))
            sample = r
    value = statistics.median(vals)
    ms_step = statistics.median(ms_vals)
    line = {"impl": "reference", "metric": wl.metric, "value": value, "unit": wl.unit,
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": dict(wl.config(), l2=L2_POLICY),
            "paths_per_step": wl.units() if wl.unit == "paths/s" else None,
            "cpu_baseline": {"value": value, "unit": wl.unit, "cores": sample["cores"],
                             "kind": sample["kind"], "sample": sample["sample"],
                             **{k: sample[k] for k in ("extrapolated", "contracts_per_s",
                                                       "seconds_by_kind") if k in sample}},
            "e2e": {"value": value, "unit": wl.unit, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args, wl_cls):
    import torch
    import parcompfin_gb300 as pcf

    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = local
    torch.cuda.set_device(dev)
    wl = wl_cls(rank)
    ctx = pcf.Context(dev)
    wl.ctx_stream = ctx.stream
    stream = torch.cuda.ExternalStream(ctx.stream, device=dev)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=dev)
    wl.setup(ctx)
    tune_reqs = wl.tune_requests() if hasattr(wl, "tune_requests") else None
    if args.no_tune or not tune_reqs:
        tuning = {"table": ctx.tuning()["table"], "changed": [],
                  "note": "built-in work shapes" if args.no_tune else
                          "no launch of this workload takes its shape from the table"}
    else:
        # The autotuner times candidate work shapes on this workload's own
        # batch (untimed), then the workload is set up again under the table
        # it chose; the bench line reports that table.
        t0 = time.perf_counter()
        rep = ctx.autotune(requests=tune_reqs)
        tuning = {"seconds": time.perf_counter() - t0, "mode": rep["mode"], "table": rep["table"],
                  "changed": sorted(k for k in rep["table"]
                                    if k != "tuned" and rep["table"][k] != rep["built_in"][k])}
        if args.tune_report:
            with open(args.tune_report, "w") as f:
                json.dump(rep, f)
        wl.setup(ctx)

    def barrier():
        torch.cuda.synchronize(dev)
        if ws > 1:
            torch.distributed.barrier()

    with torch.cuda.stream(stream):
        flush.zero_()
    for _ in range(args.warmup):
        wl.step(ctx)
    check = wl.finish(ctx)
    barrier()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    l0 = ctx.launches
    clocks = ClockSampler(dev)
    clocks.start()
    time.sleep(0.3)
    barrier()
    t_wall0 = time.perf_counter()
    with torch.cuda.stream(stream):
        for i in range(args.steps):
            flush.zero_()  # evict L2 between steps (outside the step events)
            starts[i].record(stream)
            wl.step(ctx)
            ends[i].record(stream)
    barrier()
    t_wall = time.perf_counter() - t_wall0
    launches = ctx.launches - l0
    check = wl.finish(ctx)
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    ms = sum(step_ms) / len(step_ms)
    e2e_ms, io = [], (0, 0)
    if not args.no_e2e:
        barrier()
        wl.e2e(ctx)  # untimed warm-up: first-call set-up (serving slots, scratch)
        for _ in range(max(3, args.steps)):
            t0 = time.perf_counter()
            io = wl.e2e(ctx)
            e2e_ms.append(1e3 * (time.perf_counter() - t0))
    clk = clocks.stop()
    e2e_med = statistics.median(e2e_ms) if e2e_ms else float("nan")
    if ws > 1:
        t = torch.tensor([ms, e2e_med], device=dev, dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms, e2e_med = float(t[0]), float(t[1])
    units = wl.units() * ws
    value = units / (ms * 1e-3)
    e2e_units = (wl.e2e_units() if hasattr(wl, "e2e_units") and e2e_ms else wl.units()) * ws
    if rank != 0:
        torch.distributed.destroy_process_group()
        return
    peaks = measured_peaks()
    sm_mhz = (clk or {}).get("sm_mhz") or peaks.get("sm_max_mhz", 2070.0)
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    try:
        roof = wl.roofline(ms, sms, sm_mhz, peaks)
    except TypeError:
        roof = wl.roofline(ms, sms, sm_mhz)
    roof["kernel"] = wl.dominant
    line = {
        "metric": wl.metric, "value": value, "unit": wl.unit, "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 paths, f64 sums" if wl.name != "binom" else "f64", "data": "synthetic",
        "config": dict(wl.config(), l2=L2_POLICY),
        "wall_ms_per_step": 1e3 * t_wall / args.steps,
        "paths_per_step": wl.units() if wl.unit == "paths/s" else None,
        "roofline": roof,
        "e2e": {"value": e2e_units / (e2e_med * 1e-3) if e2e_ms else None, "unit": wl.unit,
                "h2d_bytes_per_step": io[0], "d2h_bytes_per_step": io[1], "ms_per_step": e2e_med},
        "gpu_launches": launches,
        "tuning": tuning,
        "clocks": clk,
        "check": check,
    }
    if hasattr(wl, "contracts"):
        line["contracts_per_s"] = wl.contracts() * ws / (ms * 1e-3)
    if hasattr(wl, "extra") and not args.no_e2e:
        line.update(wl.extra(ctx))
        if "plain_gpu" in line and "contracts_per_s" in line:
            line["plain_gpu"]["engine_over_plain_contracts"] = (
                line["contracts_per_s"] / line["plain_gpu"]["contracts_per_s"])
    if not args.no_cpu:
        threads = os.cpu_count() or 1
        try:
            line["cpu_baseline"] = wl.cpu_reference(threads, budget_s=10.0)
        except Exception as e:  # noqa: BLE001
            line["cpu_baseline"] = {"error": repr(e)}
        if hasattr(wl, "reference_check"):
            # The CPU leg is where the oracle runs, as the checker of the
            # step's results (never inside the timed region).
            try:
                line["check"]["vs_reference"] = wl.reference_check(threads)
            except Exception as e:  # noqa: BLE001
                line["check"]["vs_reference"] = {"error": repr(e)}
    print(json.dumps(line), flush=True)
    ctx.close()
    if ws > 1:
        torch.distributed.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="mixed", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline (profiling)")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end leg (profiling)")
    ap.add_argument("--no-tune", action="store_true", help="keep the built-in work shapes")
    ap.add_argument("--tune-report", default="", help="write the autotuner's full report here")
    args = ap.parse_args()
    if args.impl == "ours":
        args.warmup = max(args.warmup, 3)
    wl = WORKLOADS[args.workload]
    if args.impl == "reference":
        run_reference(args, wl)
    else:
        run_ours(args, wl)


if __name__ == "__main__":
    main()
