"""GPU parity of the closed binomial sum (the reference's binom_embar).

Bars:
  * mode "reference" against the reference's own FP64 result
    (tests/golden/ref_outputs.json, produced by the reference's code) and the
    oracle restatement: 1e-10 relative (the stated bar; the kernel reproduces
    the reference's comb() rounding, so the observed gap is ~1e-14);
  * mode "accurate" against exact 50-digit sums (tests/golden/binom_exact.json):
    1e-12 relative.
"""
import ctypes as C
import json
import math
import os
import random

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
REF_TOL = 1e-10
EXACT_TOL = 1e-12


def _golden(name):
    with open(os.path.join(HERE, "golden", name)) as f:
        return json.load(f)


def rel(a, b):
    return abs(a - b) / max(abs(b), 1e-300)


@pytest.mark.parametrize("case", [c for c in _golden("ref_outputs.json")["cases"]
                                  if c["fn"] == "binom_embar"],
                         ids=lambda c: f"N{c['N']}-E{int(c['E'])}-pf{int(c['payoff_fun'])}")
def test_reference_mode_matches_reference_outputs(ctx, case):
    from parcompfin_gb300 import binom_embar
    v = binom_embar(case["S0"], case["E"], case["r"], case["sigma"], case["T"], case["N"],
                    case["payoff_fun"], ctx=ctx)
    ref = float.fromhex(case["value"])
    assert rel(v, ref) < REF_TOL, (v, ref, rel(v, ref))


def test_reference_mode_random_contracts_vs_oracle(orc, ctx):
    """Contracts drawn like the 1024-contract book (K, r, sigma, T, call/put)
    at N the O(N^2) oracle finishes quickly; one batched launch."""
    from parcompfin_gb300 import binom_embar_batch
    rng = random.Random(7)
    cs = []
    for _ in range(24):
        cs.append((100.0, rng.uniform(80, 120), rng.uniform(.01, .06), rng.uniform(.1, .5),
                   rng.uniform(.25, 2.0), rng.randint(1, 3000), rng.choice([1, -1])))
    got = binom_embar_batch(cs, ctx=ctx)
    worst = 0.0
    for c, v in zip(cs, got):
        ref = orc.ref_binom_embar(*c[:6], float(c[6]))
        worst = max(worst, rel(v, ref))
        assert rel(v, ref) < REF_TOL, (c, v, ref)
    print("worst relative gap", worst)


@pytest.mark.parametrize("N", [199_999, 200_000])
def test_reference_mode_large_n_vs_windowed_oracle(orc, ctx, N):
    """At the largest binomial-book N the full O(N^2) oracle is too slow; the
    oracle's windowed restatement runs the same exact comb() chain for every
    pair index near N/2 (where all of the weight is)."""
    from parcompfin_gb300 import binom_embar
    S0, E, r, sig, T = 100.0, 105.0, .03, .3, 1.5
    w = int(9 * math.sqrt(N)) + 400
    for pf in (1, -1):
        v = binom_embar(S0, E, r, sig, T, N, pf, ctx=ctx)
        part = orc.ref_binom_embar_window(S0, E, r, sig, T, N, float(pf), N // 2 - w, N)
        ref = math.exp(-r * T) * part
        assert rel(v, ref) < REF_TOL, (pf, v, ref)


def test_binomial_book_stratified_sample_vs_reference(orc, ctx):
    """The binomial book (1024 contracts from seed 7, N uneven in
    1e3..2e5) priced in one launch, as the benchmark runs it; a stratified
    sample of 32 contracts, one from each N-stratum of 32, against the
    reference's sum at 1e-10. The oracle restates comb()'s exact sequential
    chain for every pair index within 9 sqrt(N) + 400 of the binomial
    weights' centres (N p and N p u / R, and their mirrors), which holds all
    of the weight; the full O(N^2) sum would take ~25 CPU-hours for the book.
    The sample's oracle sums run in parallel threads (ctypes releases the
    interpreter lock)."""
    from concurrent.futures import ThreadPoolExecutor

    import parcompfin_gb300 as pcf
    from parcompfin_gb300 import workloads
    book = workloads.binom_book()
    got = pcf.binom_embar_batch(book, ctx=ctx)
    order = sorted(range(len(book)), key=lambda i: book[i][5])
    sample = order[16::32]
    assert len(sample) == 32 and book[sample[0]][5] < 10_000 and book[sample[-1]][5] > 190_000

    def ref(i):
        S0, E, r, sig, T, N, pf = book[i]
        lat = (C.c_double * 5)()
        orc.ref_lattice(r, sig, T, N, lat)
        p, u, R = lat[2], lat[0], lat[4]
        centre = min(N * p, N * (1 - p), N * p * u / R, N * (1 - p * u / R))
        lo = max(0, int(centre - 9 * math.sqrt(N) - 400))
        return math.exp(-r * T) * orc.ref_binom_embar_window(S0, E, r, sig, T, N, float(pf), lo, N)

    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        refs = list(ex.map(ref, sample))
    worst = 0.0
    for i, v in zip(sample, refs):
        worst = max(worst, rel(got[i], v))
        assert rel(got[i], v) < REF_TOL, (book[i], got[i], v)
    print("binomial book sample: worst relative gap", worst)


def test_reference_50000_survey_value(ctx):
    from parcompfin_gb300 import binom_embar
    v = binom_embar(100, 100, .05, .2, 1, 50000, 1, ctx=ctx)
    assert rel(v, 10.450553297126545) < REF_TOL


@pytest.mark.parametrize("case", _golden("binom_exact.json")["cases"],
                         ids=lambda c: f"N{c['contract'][5]}")
def test_accurate_mode_matches_exact_sum(ctx, case):
    from parcompfin_gb300 import binom_embar
    c = case["contract"]
    v = binom_embar(*c, mode="accurate", ctx=ctx)
    assert rel(v, case["exact"]) < EXACT_TOL, (v, case["exact"])
    vr = binom_embar(*c, mode="reference", ctx=ctx)
    assert rel(vr, case["reference"]) < REF_TOL


def test_accurate_mode_converges_to_black_scholes(orc, ctx):
    from parcompfin_gb300 import binom_embar
    bs = orc.orc_bs_price(100, 100, .05, .2, 1.0, 1)
    v = binom_embar(100, 100, .05, .2, 1.0, 200_000, 1, mode="accurate", ctx=ctx)
    assert abs(v - bs) < 1e-4


def test_batch_equals_single(ctx):
    from parcompfin_gb300 import binom_embar, binom_embar_batch
    cs = [(100.0, 95.0, .02, .25, 1.0, 1234, 1), (100.0, 101.0, .04, .35, .75, 5001, -1),
          (100.0, 110.0, .02, .75, 1.0, 1000, 1)]
    b = binom_embar_batch(cs, ctx=ctx)
    for c, v in zip(cs, b):
        assert v == binom_embar(*c, ctx=ctx)


def test_edge_cases(orc, ctx):
    from parcompfin_gb300 import binom_embar
    for N in (1, 2, 3, 4):
        for pf in (1, -1):
            v = binom_embar(100, 100, .05, .2, 1, N, pf, ctx=ctx)
            ref = orc.ref_binom_embar(100, 100, .05, .2, 1, N, float(pf))
            assert rel(v, ref) < REF_TOL
    with pytest.raises(ValueError):
        binom_embar(100, 100, .05, .2, 1, 0, 1, ctx=ctx)
    with pytest.raises(ValueError):
        binom_embar(100, 100, .05, .2, 1, 2_000_000, 1, ctx=ctx)
    with pytest.raises(ValueError, match="Unknown payoff"):
        binom_embar(100, 100, .05, .2, 1, 100, "straddle", ctx=ctx)
