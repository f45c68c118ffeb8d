"""Throughput benchmark of the GB300 pricing engine.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload NAME]

Prints one JSON line (rank 0). A step is one pass of the engine over one
batch of synthetic pricing requests (--workload):

  eur   European calls, the single-step GBM Monte Carlo of the reference's
        mc_eur (src/mc_eur.cpp:5-27) at the config-0 contract (S0=K=100,
        r=0.05, sigma=0.2, T=1), 2^28 paths per step, seed 42.

value      paths/s with the request tables already resident in HBM: kernels
           only, timed with CUDA events on the engine's stream, per step.
e2e        the same paths/s through the public C ABI (pcf_price_batch) from
           host parameters to host results, copies included, wall clock.
roofline   the dominant kernel against its compute bound.
cpu_baseline  the reference's own CPU code (oracle/_ref when it was compiled
           on this machine, else the oracle's restatement of it) on all host
           cores, on a bounded sample of the same workload.
--impl reference runs only that CPU arm and prints its line.

Multi-GPU (torchrun): every rank prices its own copy of the batch on its own
GPU with its own Philox streams (weak scaling, no collective on the data
path); value = all ranks' paths / the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

L2_FLUSH_BYTES = 256 << 20  # > the 129 MB L2 of a GB300


# --------------------------------------------------------------------------
# workloads
# --------------------------------------------------------------------------
class EurWorkload:
    name = "eur"
    metric = "MC paths/sec (European GBM, config-0 contract)"
    unit = "paths/s"
    paths = 1 << 28
    # Per path: 3 SFU ops (1/2 lg2 + 1/2 sqrt + 1/2 sin + 1/2 cos + 1 ex2).
    sfu_per_unit = 3.0

    def __init__(self, rank: int):
        self.rank = rank

    def requests(self):
        import parcompfin_gb300 as pcf
        return [pcf.request("eur", 100.0, 100.0, 0.05, 0.2, 1.0, self.paths, "call", seed=42,
                            stream=self.rank)]

    def units_per_step(self) -> float:
        return float(self.paths)

    def config(self) -> dict:
        return {"workload": "eur: European call S0=K=100 r=0.05 sigma=0.2 T=1, "
                            "2^28 paths/step, Philox seed 42",
                "paths_per_step": self.paths, "contracts_per_step": 1}

    def cpu_reference(self, threads: int, budget_s: float):
        """Time the reference's mc_eur_omp (or its restatement) on host cores."""
        from oracle import loader
        ref = loader.load_ref("mc_eur_omp")
        orc = loader.load()
        if ref is not None:
            kind = "reference"
            run = lambda n: ref(100.0, 100.0, 0.05, 0.2, 1.0, n, 0, 1.0, threads, 42)
        else:
            kind = "port"
            run = lambda n: orc.ref_mc_eur_omp(100.0, 100.0, 0.05, 0.2, 1.0, n, 1.0, 42,
                                               threads)
        n = 1 << 20
        t0 = time.perf_counter()
        run(n)
        dt = max(time.perf_counter() - t0, 1e-6)
        n = int(min(2**31 - 1, max(n, n * budget_s / dt)))
        t0 = time.perf_counter()
        price = run(n)
        dt = time.perf_counter() - t0
        return {"value": n / dt, "unit": self.unit, "cores": threads, "kind": kind,
                "sample": f"mc_eur_omp on {n} paths (config-0 contract), price {price:.6f}, "
                          f"{dt:.2f} s"}


WORKLOADS = {"eur": EurWorkload}


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

    def stop(self) -> dict | None:
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
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4)
                          if len(r) > 5 + i and r[5 + i].strip() == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(rows)}


def measured_peaks() -> dict:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f)
    return {}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def run_reference(args, wl_cls):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    wl = wl_cls(0)
    vals = []
    sample = None
    for i in range(args.warmup + args.steps):
        r = wl.cpu_reference(threads, budget_s=2.0)
        if i >= args.warmup:
            vals.append(r["value"])
            sample = r
    value = statistics.median(vals)
    line = {"impl": "reference", "metric": wl.metric, "value": value, "unit": wl.unit,
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * wl.units_per_step() / value, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": wl.config(),
            "cpu_baseline": {"value": value, "unit": wl.unit, "cores": threads,
                             "kind": sample["kind"], "sample": sample["sample"]},
            "e2e": {"value": value, "unit": wl.unit, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args, wl_cls):
    import torch
    import parcompfin_gb300 as pcf
    from parcompfin_gb300 import _lib

    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = local
    torch.cuda.set_device(dev)
    wl = wl_cls(rank)
    ctx = pcf.Context(dev)
    stream = torch.cuda.ExternalStream(ctx.stream, device=dev)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=dev)
    reqs = wl.requests()
    plan = pcf.Plan(reqs, ctx=ctx)

    def barrier():
        torch.cuda.synchronize(dev)
        if ws > 1:
            torch.distributed.barrier()

    # warm-up
    for _ in range(args.warmup):
        plan.launch()
    plan.results()
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
            plan.launch()
            ends[i].record(stream)
    barrier()
    t_wall = time.perf_counter() - t_wall0
    launches = ctx.launches - l0
    res = plan.results()
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    ms = sum(step_ms) / len(step_ms)
    # e2e: the public API from host parameters to host results, every step.
    barrier()
    e2e_ms = []
    for i in range(max(3, args.steps)):
        t0 = time.perf_counter()
        out = pcf.price_batch(reqs, ctx=ctx)
        e2e_ms.append(1e3 * (time.perf_counter() - t0))
    clk = clocks.stop()
    e2e_med = statistics.median(e2e_ms)
    if ws > 1:
        t = torch.tensor([ms, e2e_med], device=dev, dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms, e2e_med = float(t[0]), float(t[1])
    units = wl.units_per_step() * ws
    value = units / (ms * 1e-3)
    e2e_value = units / (e2e_med * 1e-3)
    if rank != 0:
        torch.distributed.destroy_process_group()
        return
    peaks = measured_peaks()
    sm_mhz = (clk or {}).get("sm_mhz") or peaks.get("sm_max_mhz", 2070.0)
    props = torch.cuda.get_device_properties(dev)
    sfu_peak = props.multi_processor_count * 16 * sm_mhz * 1e6 / 1e9  # G SFU ops/s
    sfu_ach = wl.sfu_per_unit * wl.units_per_step() / (ms * 1e-3) / 1e9
    h2d = len(reqs) * C_SIZEOF_REQUEST
    d2h = len(reqs) * C_SIZEOF_RESULT
    line = {
        "metric": wl.metric, "value": value, "unit": wl.unit, "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 paths, f64 sums", "data": "synthetic",
        "config": dict(wl.config(), l2="flushed: 256 MiB write between steps, "
                                       "outside the per-step CUDA events",
                       wall_ms_per_step=1e3 * t_wall / args.steps),
        "roofline": {"bound": "sfu", "achieved": sfu_ach, "peak": sfu_peak,
                     "unit": "G SFU op/s", "frac": sfu_ach / sfu_peak, "traffic": None,
                     "peak_source": f"{props.multi_processor_count} SMs x 16 MUFU/clk x "
                                    f"{sm_mhz:.0f} MHz (median SM clock under load)"},
        "e2e": {"value": e2e_value, "unit": wl.unit, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": e2e_med},
        "gpu_launches": launches,
        "clocks": clk,
        "check": {"price": res[0].price_plain, "std_error": res[0].std_error_plain},
    }
    if rank == 0:
        threads = os.cpu_count() or 1
        try:
            line["cpu_baseline"] = wl.cpu_reference(threads, budget_s=10.0)
        except Exception as e:  # noqa: BLE001
            line["cpu_baseline"] = {"error": repr(e)}
    print(json.dumps(line), flush=True)
    plan.close()
    ctx.close()
    if ws > 1:
        torch.distributed.destroy_process_group()


def _sizes():
    from parcompfin_gb300 import _lib
    import ctypes as C
    return C.sizeof(_lib.McRequest), C.sizeof(_lib.McResult)


C_SIZEOF_REQUEST, C_SIZEOF_RESULT = _sizes()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="eur", choices=sorted(WORKLOADS))
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3) if args.impl == "ours" else args.warmup
    wl = WORKLOADS[args.workload]
    if args.impl == "reference":
        run_reference(args, wl)
    else:
        run_ours(args, wl)


if __name__ == "__main__":
    main()
