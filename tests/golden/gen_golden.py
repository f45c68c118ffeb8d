"""Generate the golden fixtures that pin the oracle.

Run from the repository root, on a machine where the reference sources are
present, with their location as the argument:

    sh oracle/build_ref.sh REFERENCE_ROOT      # compiles oracle/_ref/*.so
    python tests/golden/gen_golden.py

Writes
  tests/golden/philox_kat.json  -- Philox4x32-10 known answers produced by an
      independent implementation (triton.language.random.philox_impl run in
      triton's CPU interpreter), including the three published Random123
      test vectors (zero, all-ones, pi digits).
  tests/golden/ref_outputs.json -- outputs of the reference's own serial
      pricing functions (oracle/_ref, compiled from the reference sources)
      for fixed parameters and injected time() seeds. Values are stored as
      float.hex() so the comparison is bit-exact.
"""
from __future__ import annotations

import json
import os
import random
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def philox_kat() -> list[dict]:
    os.environ["TRITON_INTERPRET"] = "1"
    import torch
    import triton
    import triton.language as tl

    @triton.jit
    def kat(c_ptr, out_ptr):
        c0 = tl.load(c_ptr + 0).to(tl.uint32, bitcast=True)
        c1 = tl.load(c_ptr + 1).to(tl.uint32, bitcast=True)
        c2 = tl.load(c_ptr + 2).to(tl.uint32, bitcast=True)
        c3 = tl.load(c_ptr + 3).to(tl.uint32, bitcast=True)
        k0 = tl.load(c_ptr + 4).to(tl.uint32, bitcast=True)
        k1 = tl.load(c_ptr + 5).to(tl.uint32, bitcast=True)
        a, b, c, d = tl.random.philox_impl(c0, c1, c2, c3, k0, k1, 10)
        tl.store(out_ptr + 0, a.to(tl.int32, bitcast=True))
        tl.store(out_ptr + 1, b.to(tl.int32, bitcast=True))
        tl.store(out_ptr + 2, c.to(tl.int32, bitcast=True))
        tl.store(out_ptr + 3, d.to(tl.int32, bitcast=True))

    cases = [((0, 0, 0, 0), (0, 0)),
             ((0xFFFFFFFF,) * 4, (0xFFFFFFFF, 0xFFFFFFFF)),
             ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0))]
    rng = random.Random(20211)
    for _ in range(13):
        cases.append((tuple(rng.getrandbits(32) for _ in range(4)),
                      tuple(rng.getrandbits(32) for _ in range(2))))
    out = []
    for ctr, key in cases:
        v = [x - (1 << 32) if x >= (1 << 31) else x for x in list(ctr) + list(key)]
        ci = torch.tensor(v, dtype=torch.int32)
        o = torch.zeros(4, dtype=torch.int32)
        kat[(1,)](ci, o)
        out.append({"ctr": list(ctr), "key": list(key),
                    "out": [int(x) & 0xFFFFFFFF for x in o]})
    return out


def ref_outputs() -> list[dict]:
    from oracle import loader

    cases = []

    def add(name, args, **kw):
        lib = loader.load_ref(name)
        if lib is None:
            raise SystemExit(f"oracle/_ref/ref_{name}.so missing: run oracle/build_ref.sh")
        S0, E, r, sigma, T, N, M, pf = args
        seed = kw.get("seed", 0)
        threads = kw.get("threads", 0)
        v = lib(S0, E, r, sigma, T, N, M, pf, threads, seed)
        case = {"fn": name, "S0": S0, "E": E, "r": r, "sigma": sigma, "T": T, "N": N,
                "M": M, "payoff_fun": pf, "seed": seed, "value": v.hex(), "value_repr": repr(v)}
        if threads:
            case["threads"] = threads
        cases.append(case)

    for seed in (1, 42, 1234):
        add("mc_eur", (100.0, 100.0, 0.05, 0.2, 1.0, 20000, 0, 1.0), seed=seed)
        add("mc_eur", (100.0, 110.0, 0.02, 0.75, 1.0, 10000, 0, -1.0), seed=seed)
        add("mc_asia", (100.0, 100.0, 0.05, 0.2, 1.0, 4000, 52, 1.0), seed=seed)
        add("mc_asia", (100.0, 95.0, 0.04, 0.3, 0.5, 3000, 12, -1.0), seed=seed)
        add("mc_amer", (100.0, 100.0, 0.05, 0.3, 1.0, 2000, 50, -1.0), seed=seed)
        add("mc_amer", (100.0, 90.0, 0.05, 0.3, 1.0, 2000, 20, 1.0), seed=seed)
        # The OpenMP build on one thread (its reductions then run in path order).
        add("mc_amer_omp", (100.0, 100.0, 0.05, 0.3, 1.0, 2000, 50, -1.0), seed=seed, threads=1)
        add("mc_amer_omp", (100.0, 90.0, 0.05, 0.3, 1.0, 2000, 20, 1.0), seed=seed, threads=1)
        add("mc_amer_omp", (100.0, 100.0, 0.05, 0.3, 1.0, 1000, 3, 1.0), seed=seed, threads=1)
    for N in (2, 3, 100, 1000, 1001, 5000, 20000):
        for pf in (1.0, -1.0):
            add("binom_embar", (100.0, 110.0, 0.02, 0.75, 1.0, N, 0, pf))
            add("binom_embar", (100.0, 100.0, 0.05, 0.2, 1.0, N, 0, pf))
    add("binom_embar", (100.0, 100.0, 0.05, 0.2, 1.0, 50000, 0, 1.0))
    for pf in (1.0, -1.0):
        add("binom_vanilla_eur", (100.0, 110.0, 0.02, 0.75, 1.0, 2000, 0, pf))
        add("binom_vanilla_amer", (100.0, 100.0, 0.05, 0.3, 1.0, 2000, 0, pf))
    return cases


def main() -> None:
    kat = philox_kat()
    with open(os.path.join(HERE, "philox_kat.json"), "w") as f:
        json.dump({"generator": "triton.language.random.philox_impl (CPU interpreter)",
                   "vectors": kat}, f, indent=1)
    refs = ref_outputs()
    with open(os.path.join(HERE, "ref_outputs.json"), "w") as f:
        json.dump({"source": "reference serial functions compiled by oracle/build_ref.sh; "
                             "time() returns `seed`",
                   "cases": refs}, f, indent=1)
    print(f"{len(kat)} Philox vectors, {len(refs)} reference outputs")


if __name__ == "__main__":
    main()
