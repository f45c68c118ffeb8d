"""The reference's experiment sweeps, run against the drop-in GPU programs.

Each of the reference's runscript_<method>.sh writes
results/results_<method>.csv: a header line, then one CSV line per run of
bin/<method>, bin/<method>_omp, mpirun bin/<method>_mpi and mpirun
bin/<method>_hybrid over a grid of path counts and thread / process counts,
after writing include/comparison.h with the value each run is compared
against (a lattice price from bin/binom_vanilla_eur or _amer, or a constant).

run_sweep() runs the same grid, in the same order, with the same header and
columns, through this package's programs (parcompfin_gb300/_lib/bin, built
by build.py). The comparison value is passed as PCF_COMPARISON; lattice
comparisons are priced by the GPU lattice programs, as the scripts do. The
MPI and hybrid programs run as one process (there is one GPU); PCF_RANKS
makes them report the process count the script would have launched.

    python -m parcompfin_gb300.sweeps mc_eur results/results_mc_eur.csv [--max-n N]
"""
from __future__ import annotations

import argparse
import os
import subprocess
import sys

from . import build as _build

HEADER = ("Method,Payoff,S0,E,r,sigma,T,N,M,Parallel,Nr_of_assets,T_overall,T_calculation,"
          "Result,Abs_Error,Error")
THREADS = (1, 8, 16, 32, 64)
PROCS = (1, 8, 16, 32, 64)
HYBRID = (1, 4, 8)
_N_LONG = (10000, 80000, 100000, 160000, 320000, 640000, 800000, 1000000, 1600000, 3200000,
           6400000, 8000000, 10000000, 16000000, 32000000, 64000000, 80000000, 100000000)

# Grids and comparison values of runscript_mc_eur.sh, runscript_mc_asia.sh,
# runscript_mc_amer.sh, runscript_binom_embar.sh, runscript_mc_eur_multi.sh.
SWEEPS = {
    "mc_eur": dict(payoff="call", S0=100, E=110, r=0.02, sigma=0.75, T=1, Ns=_N_LONG,
                   comparison=("binom_vanilla_eur", 100000), serial=True),
    "mc_asia": dict(payoff="call", S0=100, E=110, r=0.02, sigma=0.75, T=1, M=200,
                    Ns=(100000, 160000, 320000, 640000, 800000, 1000000, 1600000, 3200000,
                        6400000, 8000000, 10000000),
                    comparison=13.71, serial=False),
    "mc_amer": dict(payoff="call", S0=100, E=110, r=0.02, sigma=0.75, T=1, M=200,
                    Ns=(10000, 80000, 100000, 160000, 320000, 640000, 800000, 1000000, 1600000,
                        3200000, 6400000, 8000000, 10000000),
                    comparison=("binom_vanilla_amer", 10000), serial=True),
    "binom_embar": dict(payoff="call", S0=100, E=110, r=0.02, sigma=0.75, T=1,
                        Ns=(100, 800, 1000, 1600, 3200, 6400, 8000, 10000, 32000, 64000, 80000,
                            100000),
                        comparison=26.61224, serial=True, with_vanilla=True),
    "mc_eur_multi": dict(payoff="call", S0=100, E=100, r=0.1, sigma=0.2, T=1, assets=4, rho=0.5,
                         Ns=_N_LONG, comparison=11.90, serial=True),
}


def _args(method, cfg, N):
    a = [cfg["payoff"], cfg["S0"], cfg["E"], cfg["r"], cfg["sigma"], cfg["T"], N]
    if method == "mc_eur_multi":
        a += [cfg["assets"], cfg["rho"]]
    elif "M" in cfg:
        a += [cfg["M"]]
    return [str(x) for x in a]


def commands(method: str, max_n: int | None = None, variants=("serial", "omp", "mpi", "hybrid")):
    """The runs of the sweep, in the script's order: (program, argv, ranks)."""
    cfg = SWEEPS[method]
    Ns = [n for n in cfg["Ns"] if max_n is None or n <= max_n]
    out = []
    if "serial" in variants and cfg.get("serial", True):
        for N in Ns:
            out.append((method, _args(method, cfg, N), 1))
            if cfg.get("with_vanilla"):
                out.append(("binom_vanilla_eur", _args(method, cfg, N), 1))
    if "omp" in variants:
        for N in Ns:
            for t in THREADS:
                out.append((method + "_omp", _args(method, cfg, N) + [str(t)], 1))
    if "mpi" in variants:
        for N in Ns:
            for p in PROCS:
                out.append((method + "_mpi", _args(method, cfg, N), p))
    if "hybrid" in variants:
        for N in Ns:
            for h in HYBRID:
                out.append((method + "_hybrid", _args(method, cfg, N) + [str(h)], h))
    return out


def _run(program, argv, env):
    r = subprocess.run([os.path.join(_build.CLI_BIN, program), *argv], capture_output=True,
                       text=True, env=env, timeout=3600)
    if r.returncode != 0:
        raise RuntimeError(f"{program} {' '.join(argv)}: {r.stderr.strip()}")
    return r.stdout.strip()


def comparison(method: str, env=None) -> float:
    cfg = SWEEPS[method]
    c = cfg["comparison"]
    if isinstance(c, tuple):  # a lattice price, column 14 (Result) of its CSV line
        prog, N = c
        argv = [str(x) for x in (cfg["payoff"], cfg["S0"], cfg["E"], cfg["r"], cfg["sigma"],
                                 cfg["T"], N)]
        e = dict(env or os.environ)
        e["PCF_FULL_PRECISION"] = "1"
        return float(_run(prog, argv, e).split(",")[13])
    return float(c)


def run_sweep(method: str, results: str, max_n: int | None = None,
              variants=("serial", "omp", "mpi", "hybrid"), seed: int | None = None) -> int:
    """Writes `results` like runscript_<method>.sh; returns the number of runs."""
    _build.build()
    env = dict(os.environ)
    if seed is not None:
        env["PCF_SEED"] = str(seed)
    env["PCF_COMPARISON"] = repr(comparison(method, env))
    os.makedirs(os.path.dirname(os.path.abspath(results)), exist_ok=True)
    runs = commands(method, max_n, variants)
    with open(results, "w") as f:
        f.write(HEADER + "\n")
        for program, argv, ranks in runs:
            e = dict(env)
            e["PCF_RANKS"] = str(ranks)
            f.write(_run(program, argv, e) + "\n")
            f.flush()
    return len(runs)


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("method", choices=sorted(SWEEPS))
    ap.add_argument("results")
    ap.add_argument("--max-n", type=int, default=None, help="skip path counts above this")
    ap.add_argument("--variants", default="serial,omp,mpi,hybrid")
    ap.add_argument("--seed", type=int, default=None)
    a = ap.parse_args(argv)
    n = run_sweep(a.method, a.results, a.max_n, tuple(a.variants.split(",")), a.seed)
    print(f"{n} runs -> {a.results}", file=sys.stderr)
    return 0


if __name__ == "__main__":
    sys.exit(main())
