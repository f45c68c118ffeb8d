"""The oracle is pinned before it is trusted (CPU only).

1. Its Philox4x32-10 matches the known-answer vectors of an independent
   implementation (tests/golden/philox_kat.json).
2. Its restatements of the reference's functions reproduce, bit for bit, the
   outputs of the reference's own code (tests/golden/ref_outputs.json, written
   by tests/golden/gen_golden.py from oracle/_ref).
3. Where the reference sources are compiled here (oracle/_ref), further seeds
   are compared live.
"""
import ctypes as C
import json
import math
import os

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def _golden(name):
    with open(os.path.join(HERE, "golden", name)) as f:
        return json.load(f)


def test_philox_known_answers(orc):
    vecs = _golden("philox_kat.json")["vectors"]
    assert len(vecs) >= 3
    for v in vecs:
        ctr = (C.c_uint32 * 4)(*v["ctr"])
        key = (C.c_uint32 * 2)(*v["key"])
        out = (C.c_uint32 * 4)()
        orc.orc_philox4x32_10(ctr, key, out)
        assert list(out) == v["out"], v


def test_philox_published_vectors_present():
    vecs = _golden("philox_kat.json")["vectors"]
    # Random123's three published philox4x32-10 test vectors.
    assert vecs[0]["out"] == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert vecs[1]["out"] == [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]
    assert vecs[2]["out"] == [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


def _call_oracle(orc, c):
    fn, pf = c["fn"], c["payoff_fun"]
    a = (c["S0"], c["E"], c["r"], c["sigma"], c["T"])
    if fn == "mc_eur":
        return orc.ref_mc_eur(*a, c["N"], pf, c["seed"])
    if fn == "mc_asia":
        return orc.ref_mc_asia(*a, c["N"], c["M"], pf, c["seed"])
    if fn == "mc_amer":
        return orc.ref_mc_amer(*a, c["N"], c["M"], pf, c["seed"])
    if fn == "mc_amer_omp":
        return orc.ref_mc_amer_omp(*a, c["N"], c["M"], pf, c["seed"], c["threads"])
    if fn == "binom_embar":
        return orc.ref_binom_embar(*a, c["N"], pf)
    if fn == "binom_vanilla_eur":
        return orc.ref_binom_vanilla_eur(*a, c["N"], pf)
    if fn == "binom_vanilla_amer":
        return orc.ref_binom_vanilla_amer(*a, c["N"], pf)
    raise AssertionError(fn)


@pytest.mark.parametrize("case", _golden("ref_outputs.json")["cases"],
                         ids=lambda c: f"{c['fn']}-N{c['N']}-pf{int(c['payoff_fun'])}-s{c['seed']}")
def test_oracle_matches_reference_bitwise(orc, case):
    if case["fn"] == "binom_embar" and case["N"] > 20000:
        pytest.skip("large-N lattice case is checked by the slow GPU parity test")
    got = _call_oracle(orc, case)
    assert got.hex() == case["value"], (got, case["value_repr"])


def test_reference_put_bug_is_reproduced(orc):
    # src/mc_amer.cpp:100 exercises at payoff(S - E, E): the reference American
    # put is far above the lattice value. The restatement must keep that.
    ref = orc.ref_mc_amer(100.0, 100.0, 0.05, 0.3, 1.0, 2000, 50, -1.0, 7)
    lat = orc.ref_binom_vanilla_amer(100.0, 100.0, 0.05, 0.3, 1.0, 2000, -1.0)
    assert ref > 50 and abs(lat - 9.87) < 0.02


def test_live_reference_if_built(orc):
    from oracle import loader
    lib = loader.load_ref("mc_eur")
    if lib is None:
        pytest.skip("oracle/_ref not built on this machine")
    for seed in (3, 99, 2021):
        assert lib(100, 100, .05, .2, 1, 5000, 0, 1.0, 0, seed) == \
            orc.ref_mc_eur(100, 100, .05, .2, 1, 5000, 1.0, seed)
    lib = loader.load_ref("binom_embar")
    for N in (7, 64, 999):
        assert lib(100, 90, .03, .4, .5, N, 0, -1.0) == \
            orc.ref_binom_embar(100, 90, .03, .4, .5, N, -1.0)


def test_closed_forms_known_values(orc):
    assert orc.orc_bs_price(100, 100, .05, .2, 1, 1) == pytest.approx(10.450583572185565, rel=1e-14)
    assert orc.orc_bs_price(100, 110, .02, .75, 1, 1) == pytest.approx(26.612236351476916, rel=1e-14)
    assert orc.orc_bs_price(100, 100, .05, .3, 1, -1) == pytest.approx(9.354197236057232, rel=1e-14)
    # A geometric average over one date (w_M = 1) is the Black-Scholes price.
    w = (C.c_double * 2)(0.0, 1.0)
    g = orc.orc_geo_weighted_price(100, 95, .03, .25, 2.0, 1, w, 1, None)
    assert g == pytest.approx(orc.orc_bs_price(100, 95, .03, .25, 2.0, 1), rel=1e-13)


def test_lattice_converges_to_black_scholes(orc):
    v = orc.ref_binom_vanilla_eur(100, 100, .05, .2, 1, 4000, 1.0)
    assert abs(v - 10.450583572185565) < 2e-3


def _price_se(s, n, disc):
    m = s[0] / n
    var = (s[1] - n * m * m) / (n - 1)
    return disc * m, disc * math.sqrt(var / n)


def test_twin_mc_eur_near_black_scholes(orc):
    s = (C.c_double * 5)()
    n = 400_000
    orc.twin_mc_eur(100, 100, .05, .2, 1, n, 1, 42, 0, s)
    p, se = _price_se(s, n, math.exp(-.05))
    assert abs(p - 10.450583572185565) < 4 * se
    # E[S_T] = S0 e^{rT}: the control variate's mean.
    gbar = s[2] / n
    assert abs(gbar - 100 * math.exp(.05)) < 4 * 20.5 / math.sqrt(n)


@pytest.mark.parametrize("mode", [0, 1])
def test_twin_asia_geometric_mean_matches_closed_form(orc, mode):
    s = (C.c_double * 5)()
    n, M = 200_000, 12
    orc.twin_mc_asia(100, 100, .04, .3, 1.0, n, M, 1, mode, 13, 1, s)
    p, se = _price_se([s[2], s[3]], n, math.exp(-.04))
    exact = orc.orc_geo_asian_price(100, 100, .04, .3, 1.0, M, mode, 1, None)
    assert abs(p - exact) < 4 * se


def test_twin_basket_geometric_mean_matches_closed_form(orc):
    d = 5
    S0 = (C.c_double * d)(*[100.0] * d)
    sig = (C.c_double * d)(.15, .2, .25, .3, .35)
    rho = .4
    corr = [1.0 if i == j else rho for i in range(d) for j in range(d)]
    # Cholesky of the equicorrelation matrix.
    L = [0.0] * (d * d)
    for i in range(d):
        for j in range(i + 1):
            v = corr[i * d + j] - sum(L[i * d + k] * L[j * d + k] for k in range(j))
            L[i * d + j] = math.sqrt(v) if i == j else v / L[j * d + j]
    s = (C.c_double * 5)()
    n = 100_000
    orc.twin_mc_basket(d, S0, sig, (C.c_double * (d * d))(*L), .03, 1.0, 1.0, 100.0, n, 1, 11,
                       0, s)
    p, se = _price_se([s[2], s[3]], n, math.exp(-.03))
    exact = orc.orc_geo_basket_price(d, S0, sig, (C.c_double * (d * d))(*corr), .03, 1.0, 1.0,
                                     100.0, 1, None)
    assert abs(p - exact) < 4 * se


def test_twin_amer_put_near_lattice(orc):
    out = (C.c_double * 6)()
    n = 100_000
    orc.twin_mc_amer(100, 100, .05, .3, 1, n, 50, -1, 0, 5, 0, out)
    pairs = n // 2  # the moment sums run over antithetic pair means
    p, se = _price_se(out, pairs, 1.0)
    lat = orc.ref_binom_vanilla_amer(100, 100, .05, .3, 1, 2000, -1.0)
    # LSM is low-biased by a few cents at 50 dates; allow that plus 4 SE.
    assert abs(p - lat) < 0.05 + 4 * se, (p, lat, se)
    assert out[5] == 0
    # The martingale control variate has the European price as its mean and
    # cuts the variance sharply.
    g, se_g = _price_se([out[2], out[3]], pairs, 1.0)
    assert abs(g - orc.orc_bs_price(100, 100, .05, .3, 1, -1)) < 4 * se_g
    ybar, gbar = out[0] / pairs, out[2] / pairs
    vy = out[1] / pairs - ybar * ybar
    vg = out[3] / pairs - gbar * gbar
    cov = out[4] / pairs - ybar * gbar
    assert vy - cov * cov / vg < 0.2 * vy
