"""GPU backward induction on the reference's lattice (binom_vanilla_eur /
binom_vanilla_amer) against the oracle's restatement, which is pinned bit for
bit to the reference's own outputs: the prices must be identical."""
import pytest

pytestmark = pytest.mark.gpu

CASES = [(100, 100, .05, .2, 1.0), (100, 110, .02, .75, 1.0), (100, 90, .03, .4, .5),
         (50, 60, .08, .3, 2.0)]


@pytest.mark.parametrize("american", [False, True])
@pytest.mark.parametrize("pf", [1, -1])
@pytest.mark.parametrize("N", [1, 2, 7, 100, 1000, 2047, 2048, 2049, 2177, 5000, 20000])
def test_lattice_bit_exact(orc, ctx, N, pf, american):
    import parcompfin_gb300 as pcf
    fn = pcf.binom_vanilla_amer if american else pcf.binom_vanilla_eur
    ref = orc.ref_binom_vanilla_amer if american else orc.ref_binom_vanilla_eur
    for S0, E, r, sig, T in CASES[:1 if N > 5000 else 4]:
        got = fn(S0, E, r, sig, T, N, pf, ctx=ctx)
        want = ref(S0, E, r, sig, T, N, float(pf))
        assert got == want, (S0, E, r, sig, T, N, pf, american, got, want)


def test_lattice_converges_and_orders(orc, ctx):
    import parcompfin_gb300 as pcf
    bs = orc.orc_bs_price(100, 100, .05, .3, 1.0, -1)
    eur = pcf.binom_vanilla_eur(100, 100, .05, .3, 1.0, 100000, "put", ctx=ctx)
    amer = pcf.binom_vanilla_amer(100, 100, .05, .3, 1.0, 100000, "put", ctx=ctx)
    assert abs(eur - bs) < 1e-3
    assert amer > eur + 0.4  # early-exercise premium of the put
    # the American call on a non-dividend stock is the European call
    c_am = pcf.binom_vanilla_amer(100, 100, .05, .3, 1.0, 20000, "call", ctx=ctx)
    c_eu = pcf.binom_vanilla_eur(100, 100, .05, .3, 1.0, 20000, "call", ctx=ctx)
    assert abs(c_am - c_eu) < 1e-12 * c_eu


def test_lattice_rejects_bad_input(ctx):
    import parcompfin_gb300 as pcf
    with pytest.raises(ValueError):
        pcf.binom_vanilla_eur(100, 100, .05, .3, 1.0, 0, "put", ctx=ctx)
    with pytest.raises(ValueError):
        pcf.binom_vanilla_amer(100, 100, .05, .3, 1.0, 3_000_000, "put", ctx=ctx)
