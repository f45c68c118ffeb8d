"""Batched pricing (pcf_price_batch / pcf_plan_*).

  * a batch of European / Asian / basket contracts reproduces, bit for bit,
    the moment sums of the single-contract entry points (each work item is
    computed and reduced the same way; the finaliser sums items in order);
  * American requests (one thread-block cluster per contract, or the
    cooperative kernel for the largest) match the FP64 twin within the LSM
    tolerance of test_gpu_amer.py;
  * each request prices the same alone and inside a mixed batch;
  * replaying a plan is deterministic.
"""
import ctypes as C
import math

import pytest

pytestmark = pytest.mark.gpu


def _mixed(pcf):
    return [
        pcf.request("eur", 100, 95, .05, .2, 1.0, 300_001, "call", use_cv=True, seed=1, stream=1),
        pcf.request("asia", 100, 105, .04, .3, 1.5, 40_000, "call", M=52, use_cv=True, seed=1,
                    stream=2),
        pcf.request("basket", 100, 100, .03, .25, 1.0, 50_000, "call", assets=7, rho=.3,
                    use_cv=True, seed=1, stream=3),
        pcf.request("amer", 100, 105, .05, .3, 1.0, 1 << 16, "put", M=50, use_cv=True, seed=1,
                    stream=4),
        pcf.request("eur", 100, 110, .02, .75, 1.0, 12_345, "put", seed=2, stream=5),
        pcf.request("amer", 100, 95, .05, .25, 1.0, 20_000, "put", M=20, seed=2, stream=6),
    ]


def test_batch_matches_single_calls(ctx):
    import parcompfin_gb300 as pcf
    out = pcf.price_batch(_mixed(pcf), ctx=ctx)
    a = pcf.mc_eur_result(100, 95, .05, .2, 1.0, 300_001, "call", seed=1, use_cv=True, ctx=ctx)
    # the single-call entry points use Philox stream 0; the batch used stream 1
    assert out[0].n_paths == a.n_paths
    b = pcf.price_batch([pcf.request("eur", 100, 95, .05, .2, 1.0, 300_001, "call", use_cv=True,
                                     seed=1, stream=0)], ctx=ctx)[0]
    assert list(a.sums) == list(b.sums)
    b = pcf.price_batch([pcf.request("asia", 100, 105, .04, .3, 1.5, 40_000, "call", M=52,
                                     use_cv=True, seed=1, stream=0)], ctx=ctx)[0]
    a = pcf.mc_asia_result(100, 105, .04, .3, 1.5, 40_000, 52, "call", seed=1, use_cv=True,
                           ctx=ctx)
    assert list(a.sums) == list(b.sums)


def test_same_alone_and_in_the_mix(ctx):
    import parcompfin_gb300 as pcf
    reqs = _mixed(pcf)
    mix = pcf.price_batch(reqs, ctx=ctx)
    for q, m in zip(reqs, mix):
        alone = pcf.price_batch([q], ctx=ctx)[0]
        # A launch computes the control-variate sums when any request of its
        # method asks for them; the payoff sums, the price and its standard
        # error do not depend on that.
        k = 5 if q["use_cv"] else 2
        assert list(alone.sums)[:k] == list(m.sums)[:k], q
        assert alone.price == m.price and alone.std_error == m.std_error


@pytest.mark.parametrize("N", [4096, 1 << 16, 1 << 18, 1 << 20])
def test_american_batch_against_twin(orc, ctx, N):
    import parcompfin_gb300 as pcf
    reqs = [pcf.request("amer", 100, 100, .05, .3, 1.0, N, "put", M=50, seed=5, stream=0),
            pcf.request("amer", 100, 110, .05, .25, 1.0, N, "put", M=50, seed=5, stream=0)]
    out = pcf.price_batch(reqs, ctx=ctx)
    for q, r in zip(reqs, out):
        s = (C.c_double * 6)()
        orc.twin_mc_amer(100, q["E"], .05, q["sigma"], 1.0, N, 50, -1, 0, 5, 0, s)
        for k in (0, 2):
            assert abs(r.sums[k] - s[k]) <= 3e-4 * abs(s[k]), (N, k, r.sums[k], s[k])


def test_american_batch_long_and_mixed_dates_against_twin(orc, ctx):
    """Contracts of different date counts in one cluster launch (the launch
    sizes its shared memory for the longest), including more than 255
    dates (16-bit exercise dates): each against the FP64 twin, and each the
    same bits alone and in the batch."""
    import parcompfin_gb300 as pcf
    spec = [(100.0, .3, 300, 3), (105.0, .25, 30, 4), (95.0, .35, 61, 5), (100.0, .2, 7, 6)]
    reqs = [pcf.request("amer", 100, E, .05, sig, 1.0, 1 << 15, "put", M=M, seed=11, stream=st)
            for E, sig, M, st in spec]
    out = pcf.price_batch(reqs, ctx=ctx)
    for q, r, (E, sig, M, st) in zip(reqs, out, spec):
        s = (C.c_double * 6)()
        orc.twin_mc_amer(100, E, .05, sig, 1.0, 1 << 15, M, -1, 0, 11, st, s)
        for k in (0, 2):
            assert abs(r.sums[k] - s[k]) <= 3e-4 * abs(s[k]), (M, k, r.sums[k], s[k])
        alone = pcf.price_batch([q], ctx=ctx)[0]
        assert list(alone.sums) == list(r.sums), M


def test_american_batch_against_lattice(orc, ctx):
    import parcompfin_gb300 as pcf
    reqs = [pcf.request("amer", 100, E, .05, .3, 1.0, 1 << 17, "put", M=50, use_cv=True, seed=9,
                        stream=k) for k, E in enumerate((90.0, 100.0, 110.0))]
    for q, r in zip(reqs, pcf.price_batch(reqs, ctx=ctx)):
        lat = orc.ref_binom_vanilla_amer(100, q["E"], .05, .3, 1.0, 2000, -1.0)
        assert abs(r.price_cv - lat) < 0.05 + 4 * r.std_error_cv, (q["E"], r.price_cv, lat)


def test_plan_replay_is_deterministic(ctx):
    import parcompfin_gb300 as pcf
    with pcf.Plan(_mixed(pcf), ctx=ctx) as plan:
        assert plan.kernel_count >= 4
        plan.launch()
        first = plan.results()
        for _ in range(2):
            plan.launch()
        again = plan.results()
    for a, b in zip(first, again):
        assert list(a.sums) == list(b.sums)


def test_batch_rejects_bad_requests(ctx):
    import parcompfin_gb300 as pcf
    with pytest.raises(ValueError, match="divisible by 2"):
        pcf.price_batch([pcf.request("amer", 100, 100, .05, .3, 1.0, 1001, "put", M=50)], ctx=ctx)
    with pytest.raises(ValueError):
        pcf.price_batch([pcf.request("asia", 100, 100, .05, .3, 1.0, 1000, "put", M=0)], ctx=ctx)


def test_plan_graph_replay_matches_direct_launches(ctx):
    """From its second launch a plan replays a CUDA graph of its launch
    sequence; the sums are the same bits as direct launches."""
    import parcompfin_gb300 as pcf
    reqs = _mixed(pcf)
    with pcf.Plan(reqs, ctx=ctx, graph=False) as direct:
        for _ in range(2):
            direct.launch()
        a = direct.results()
        assert not direct.uses_graph
    with pcf.Plan(reqs, ctx=ctx) as plan:
        plan.launch()
        first = plan.results()
        assert not plan.uses_graph
        before = ctx.launches
        for _ in range(3):
            plan.launch()
        again = plan.results()
        assert plan.uses_graph
        assert ctx.launches - before == 3 * plan.kernel_count
    for x, y, z in zip(a, first, again):
        assert list(x.sums) == list(y.sums) == list(z.sums)


def test_plan_graph_with_a_cooperative_contract(orc, ctx):
    """An American contract too large for one cluster runs the cooperative
    kernel; its plan replays the same sums whether or not the capture of a
    cooperative launch is supported."""
    import parcompfin_gb300 as pcf
    reqs = [pcf.request("amer", 100, 100, .05, .3, 1.0, 1 << 19, "put", M=50, seed=5, stream=0),
            pcf.request("eur", 100, 95, .05, .2, 1.0, 100_000, "call", seed=1, stream=1)]
    with pcf.Plan(reqs, ctx=ctx) as plan:
        plan.launch()
        first = plan.results()
        for _ in range(2):
            plan.launch()
        again = plan.results()
    for x, y in zip(first, again):
        assert list(x.sums) == list(y.sums)
    s = (C.c_double * 6)()
    orc.twin_mc_amer(100, 100, .05, .3, 1.0, 1 << 19, 50, -1, 0, 5, 0, s)
    assert abs(again[0].sums[0] - s[0]) <= 3e-4 * abs(s[0])


def test_batch_with_a_streaming_contract(ctx):
    """An American contract beyond shared memory (3.2e6 paths) in a batch runs
    the streaming sweep on the same grid as pricing it alone: the same sums."""
    import parcompfin_gb300 as pcf
    from parcompfin_gb300 import mc_amer_result
    N, M = 3_200_000, 10
    reqs = [pcf.request("eur", 100, 95, .05, .2, 1.0, 100_000, "call", seed=1, stream=1),
            pcf.request("amer", 100, 100, .05, .3, 1.0, N, "put", M=M, seed=5, stream=0),
            pcf.request("amer", 100, 105, .05, .3, 1.0, 1 << 16, "put", M=M, seed=5, stream=2)]
    with pcf.Plan(reqs, ctx=ctx) as plan:
        plan.launch()
        got = plan.results()
        plan.launch()
        again = plan.results()
    alone = mc_amer_result(100, 100, .05, .3, 1.0, N, M, -1, seed=5, ctx=ctx)
    assert list(got[1].sums) == list(alone.sums)
    for x, y in zip(got, again):
        assert list(x.sums) == list(y.sums)
