"""Exact closed binomial sums for the accurate binom_embar mode.

For each contract, the lattice parameters u, d, p, q are the doubles the
reference computes (src/binom_embar.cpp:19-27, via the oracle's
ref_lattice). The sum e^{-rT} sum_k C(N,k) p^k q^{N-k} payoff(S0 u^k d^{N-k})
is then evaluated with those doubles taken as exact numbers, in 50-digit
arithmetic (mpmath). Writes tests/golden/binom_exact.json.

    python tests/golden/gen_binom_exact.py
"""
from __future__ import annotations

import ctypes as C
import json
import os
import sys

import mpmath as mp

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

CONTRACTS = [
    (100.0, 100.0, 0.05, 0.2, 1.0, 1000, 1),
    (100.0, 100.0, 0.05, 0.2, 1.0, 1000, -1),
    (100.0, 110.0, 0.02, 0.75, 1.0, 1001, 1),
    (100.0, 90.0, 0.03, 0.4, 0.5, 4000, -1),
    (100.0, 120.0, 0.06, 0.1, 2.0, 5000, 1),
    (100.0, 80.0, 0.01, 0.5, 0.25, 7777, -1),
    (100.0, 100.0, 0.05, 0.2, 1.0, 20000, 1),
]


def exact(orc, S0, E, r, sigma, T, N, pf):
    lat = (C.c_double * 5)()
    orc.ref_lattice(r, sigma, T, N, lat)
    u, d, p, q = (mp.mpf(lat[i]) for i in range(4))
    S0m, Em = mp.mpf(S0), mp.mpf(E)
    total = mp.mpf(0)
    w = q ** N  # C(N,0) p^0 q^N
    ratio = p / q
    for k in range(N + 1):
        if k:
            w = w * (N - k + 1) / k * ratio
        S = S0m * u ** k * d ** (N - k)
        pay = max(pf * (S - Em), 0)
        total += w * pay
    return float(mp.e ** (-mp.mpf(r) * mp.mpf(T)) * total)


def main():
    from oracle import loader
    orc = loader.load()
    mp.mp.dps = 50
    out = []
    for c in CONTRACTS:
        v = exact(orc, *c)
        ref = orc.ref_binom_embar(*c[:6], float(c[6]))
        out.append({"contract": list(c), "exact": v, "reference": ref})
        print(c, v, ref, (ref - v) / v)
    with open(os.path.join(HERE, "binom_exact.json"), "w") as f:
        json.dump({"source": "50-digit mpmath sum with the reference's double lattice "
                             "parameters; 'reference' is the reference's own binom()",
                   "cases": out}, f, indent=1)


if __name__ == "__main__":
    main()
