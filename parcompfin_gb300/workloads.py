"""Synthetic request sets with the shapes of the reference's benchmark runs.

Each generator is seeded, so every run prices the same requests. There is no
public dataset: the reference's experiments are parameter sweeps
(runscript_*.sh), and these sets follow five benchmark workloads:

  eur_contract()  European call, S0=K=100, r=.05, sigma=.2, T=1 (mc_eur)
  binom_book()    1024 closed-binomial contracts, uneven N (binom_embar)
  basket_book()   baskets of 4, 16, 64 assets, Wishart-blended correlation (mc_eur_multi)
  asian_book()    256 Asian contracts, M in {12, 52, 252}, N log-uniform (mc_asia)
  mixed_stream()  the mixed request stream: European / basket / Asian / American
"""
from __future__ import annotations

import math
import random

import numpy as np


def eur_contract(N: int = 1_000_000, seed: int = 42) -> dict:
    return dict(S0=100.0, E=100.0, r=0.05, sigma=0.2, T=1.0, N=N, payoff_fun=1, seed=seed)


def binom_book(n: int = 1024, seed: int = 7) -> list:
    """(S0, E, r, sigma, T, N, payoff_fun) for the closed binomial sum."""
    rng = random.Random(seed)
    out = []
    for _ in range(n):
        out.append((100.0, rng.uniform(80, 120), rng.uniform(0.01, 0.06), rng.uniform(0.1, 0.5),
                    rng.uniform(0.25, 2.0), rng.randint(1000, 200000), rng.choice([1, -1])))
    return out


def wishart_corr(d: int, seed: int = 11) -> np.ndarray:
    """0.7 * (all-pairs rho = 0.3) + 0.3 * normalised Wishart(d, d + 2)."""
    rs = np.random.default_rng(seed)
    X = rs.standard_normal((d, d + 2))
    W = X @ X.T
    s = np.sqrt(np.diag(W))
    Cw = W / np.outer(s, s)
    Ce = np.full((d, d), 0.3)
    np.fill_diagonal(Ce, 1.0)
    C = 0.7 * Ce + 0.3 * Cw
    C = 0.5 * (C + C.T)
    np.fill_diagonal(C, 1.0)
    np.linalg.cholesky(C)  # SPD check
    return C


def basket_book(dims=(4, 16, 64), N: int = 1 << 22, seed: int = 11) -> list:
    """Basket calls, equal weights, S0_i = 100, K = 100, r = .03, T = 1."""
    rng = random.Random(seed)
    out = []
    for d in dims:
        sig = [rng.uniform(0.15, 0.35) for _ in range(d)]
        out.append(dict(assets=d, basket_S0=[100.0] * d, basket_sigma=sig,
                        corr=wishart_corr(d, seed).tolist(), r=0.03, T=1.0, E=100.0, N=N,
                        payoff_fun=1))
    return out


def asian_book(n: int = 256, seed: int = 13) -> list:
    """Asian fixed-strike arithmetic calls, r = .04."""
    rng = random.Random(seed)
    out = []
    for _ in range(n):
        out.append(dict(S0=100.0, E=rng.uniform(90, 110), r=0.04, sigma=rng.uniform(0.15, 0.4),
                        T=rng.uniform(0.5, 2.0), M=rng.choice([12, 52, 252]),
                        N=int(2 ** rng.uniform(16, 22)), payoff_fun=1))
    return out


def mixed_stream(n: int, seed: int = 17) -> list:
    """The mixed request stream: 30% European (the eur_contract parameters jittered),
    20% basket (d ~ U{2..32}), 30% Asian (the asian_book distribution), 20%
    American put by Longstaff-Schwartz (S0 = 100, K ~ U[90,110], r = .05,
    sigma ~ U[.2,.4], T = 1, 50 exercise dates)."""
    rng = random.Random(seed)
    out = []
    for i in range(n):
        u = rng.random()
        if u < 0.3:
            out.append(dict(kind="eur", S0=100.0, E=100.0 * rng.uniform(0.9, 1.1),
                            r=0.05 * rng.uniform(0.8, 1.2), sigma=0.2 * rng.uniform(0.8, 1.2),
                            T=rng.uniform(0.8, 1.2), payoff_fun=1))
        elif u < 0.5:
            d = rng.randint(2, 32)
            out.append(dict(kind="basket", S0=100.0, E=100.0, r=0.03, sigma=0.25, T=1.0,
                            assets=d, rho=0.3,
                            basket_sigma=[rng.uniform(0.15, 0.35) for _ in range(d)],
                            payoff_fun=1))
        elif u < 0.8:
            out.append(dict(kind="asia", S0=100.0, E=rng.uniform(90, 110), r=0.04,
                            sigma=rng.uniform(0.15, 0.4), T=rng.uniform(0.5, 2.0),
                            M=rng.choice([12, 52, 252]), payoff_fun=1))
        else:
            out.append(dict(kind="amer", S0=100.0, E=rng.uniform(90, 110), r=0.05,
                            sigma=rng.uniform(0.2, 0.4), T=1.0, M=50, payoff_fun=-1))
        out[-1]["id"] = i
    return out


def poisson_arrivals(n: int, rate: float, seed: int = 23) -> list:
    """Arrival times (seconds) of n requests at `rate` per second."""
    rng = random.Random(seed)
    t, out = 0.0, []
    for _ in range(n):
        t += rng.expovariate(rate)
        out.append(t)
    return out


def log2_paths(x: float) -> int:
    return int(math.ceil(math.log2(max(1.0, x))))
