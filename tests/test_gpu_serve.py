"""The continuous-batching serving loop (pcf_serve_trace).

  * every request of a timed mixed trace completes, at (about) its target
    relative standard error, unless its path count hit the cap;
  * each served result is the same as pricing that request alone at the same
    path count. Where one run priced it (American requests, and requests whose
    pilot reached the target) the tolerance is exact equality of the moment
    sums: a request's work items and their reduction do not depend on what
    else is in its batch. A European, Asian or basket request whose main run
    continued its pilot (paths [n0, N) after paths [0, n0)) has the same
    paths in two partial sums, grouped differently into per-thread FP32
    partials: equal to 1e-8 relative (measured ~1e-10; other paths would
    differ by the Monte Carlo noise, ~1e-3);
  * requests arriving while other batches run are admitted into other slots
    (more than one batch in flight).
"""
import ctypes as C
import math

import pytest

pytestmark = pytest.mark.gpu

TARGET = 5e-4
PILOT = 1 << 14


def _trace(pcf, n, rate, seed):
    from parcompfin_gb300 import workloads
    spec = workloads.mixed_stream(n, seed=seed)
    reqs = []
    for s in spec:
        kw = dict(use_cv=True, seed=99, stream=s["id"])
        if s["kind"] == "eur":
            reqs.append(pcf.request("eur", s["S0"], s["E"], s["r"], s["sigma"], s["T"], 4, "call", **kw))
        elif s["kind"] == "asia":
            reqs.append(pcf.request("asia", s["S0"], s["E"], s["r"], s["sigma"], s["T"], 4, "call",
                                    M=s["M"], **kw))
        elif s["kind"] == "basket":
            reqs.append(pcf.request("basket", s["S0"], s["E"], s["r"], s["sigma"], s["T"], 4, "call",
                                    assets=s["assets"], rho=s["rho"],
                                    basket_sigma=s["basket_sigma"], **kw))
        else:
            reqs.append(pcf.request("amer", s["S0"], s["E"], s["r"], s["sigma"], s["T"], 2, "put",
                                    M=s["M"], **kw))
    return reqs, workloads.poisson_arrivals(n, rate, seed=seed + 1)


def test_served_trace_meets_target_and_matches_alone(ctx):
    import parcompfin_gb300 as pcf
    reqs, arr = _trace(pcf, 240, 4000.0, 3)
    out, st = pcf.serve_trace(reqs, arr, target_rel_se=TARGET, ctx=ctx)
    assert st.completed == len(reqs)
    assert st.p50_ms <= st.p99_ms <= st.max_ms
    assert st.batches >= 2
    rels = []
    for q, o in zip(reqs, out):
        assert o.status == 0
        r = o.result
        assert o.done_s >= o.admit_s >= o.arrival_s - 1e-9
        main_n = r.n_paths
        capped = q["method"] == 3 and main_n >= (1 << 21)
        rel = r.std_error / abs(r.price)
        rels.append(rel)
        if not capped:
            # the pilot's variance estimate is itself noisy: allow 35 %
            assert rel < 1.35 * TARGET, (q, rel)
    # Same alone: re-price a sample of requests alone at the served path count.
    continued = 0
    for i in range(0, len(reqs), 6):
        q = dict(reqs[i], N=out[i].result.n_paths)
        alone = pcf.price_batch([q], ctx=ctx)[0]
        if q["method"] == 3 or q["N"] <= PILOT:
            assert list(alone.sums) == list(out[i].result.sums), q
        else:
            continued += 1
            for a, b in zip(alone.sums, out[i].result.sums):
                assert abs(a - b) <= 1e-8 * max(abs(a), abs(b)), (q, a, b)
            assert out[i].paths == q["N"]  # the pilot's paths are part of the estimate
            assert abs(alone.price - out[i].result.price) <= 1e-8 * abs(alone.price)
    assert continued > 0
    assert sorted(rels)[len(rels) // 2] < TARGET


def test_served_european_prices_agree_with_black_scholes(orc, ctx):
    import parcompfin_gb300 as pcf
    reqs = [pcf.request("eur", 100, E, .05, .2, 1.0, 4, "call", use_cv=True, seed=5, stream=k)
            for k, E in enumerate((90.0, 100.0, 110.0, 120.0))]
    out, st = pcf.serve_trace(reqs, [0.0] * 4, target_rel_se=TARGET, ctx=ctx)
    for q, o in zip(reqs, out):
        bs = orc.orc_bs_price(100, q["E"], .05, .2, 1.0, 1)
        assert abs(o.result.price - bs) < 4 * o.result.std_error + 1e-9


def test_serving_without_target_uses_request_sizes(ctx):
    import parcompfin_gb300 as pcf
    reqs = [pcf.request("eur", 100, 100, .05, .2, 1.0, 100_000 + k, "call", seed=1, stream=k)
            for k in range(20)]
    out, st = pcf.serve_trace(reqs, [0.001 * k for k in range(20)], target_rel_se=0.0, ctx=ctx)
    assert st.completed == 20
    for q, o in zip(reqs, out):
        assert o.result.n_paths == q["N"] and o.paths == q["N"]


def test_request_whose_pilot_reaches_the_target_is_done_after_it(ctx):
    """A deep in-the-money European call with its control variate (g = S_T)
    has almost no residual variance: the pilot's 2^14 paths already reach the
    target, so the pilot is its result."""
    import parcompfin_gb300 as pcf
    reqs = [pcf.request("eur", 100, 20, .05, .2, 1.0, 4, "call", use_cv=True, seed=3, stream=0),
            pcf.request("eur", 100, 100, .05, .2, 1.0, 4, "call", use_cv=True, seed=3, stream=1)]
    out, st = pcf.serve_trace(reqs, [0.0, 0.0], target_rel_se=TARGET, ctx=ctx)
    assert st.completed == 2
    deep, atm = out[0], out[1]
    assert deep.result.n_paths == PILOT and deep.paths == PILOT
    assert deep.result.std_error / deep.result.price < TARGET
    alone = pcf.price_batch([dict(reqs[0], N=PILOT)], ctx=ctx)[0]
    assert list(alone.sums) == list(deep.result.sums)
    assert atm.result.n_paths > PILOT and atm.paths == atm.result.n_paths


def test_price_batch_arena_grows_and_is_reused(ctx):
    """pcf_price_batch builds in the context's arena: a small batch, a much
    larger one (the arena grows), then the small one again give the same sums
    as plans built on their own."""
    import parcompfin_gb300 as pcf
    small = [pcf.request("eur", 100, 100, .05, .2, 1.0, 100_000, "call", seed=1, stream=0)]
    big = [pcf.request("amer", 100, 95 + k, .05, .3, 1.0, 1 << 18, "put", M=50, seed=2, stream=k)
           for k in range(12)] + small
    a = pcf.price_batch(small, ctx=ctx)
    b = pcf.price_batch(big, ctx=ctx)
    c = pcf.price_batch(small, ctx=ctx)
    with pcf.Plan(big, ctx=ctx) as plan:
        plan.launch()
        ref = plan.results()
    assert list(a[0].sums) == list(c[0].sums) == list(b[-1].sums)
    for x, y in zip(b, ref):
        assert list(x.sums) == list(y.sums)


def test_served_prices_agree_with_the_reference(orc, ctx):
    """A seeded mixed trace of 300 requests through the serving loop, each
    served price against its reference (oracle/served_check.py): European
    against Black-Scholes, Asian against the reference's own estimator
    (src/mc_asia_omp.cpp) at a combined standard error, basket against the
    FP64 restatement on independent draws, American puts against the
    reference's lattice (src/binom_vanilla_amer.cpp) within the LSM bias and
    against the FP64 twin on identical draws. Outside three combined standard
    errors, 0.27 % of the checked requests are expected by chance: at most
    two per kind, and none beyond 4.5."""
    import json
    import os

    import parcompfin_gb300 as pcf
    from oracle import served_check
    reqs, arr = _trace(pcf, 300, 4000.0, 41)
    out, st = pcf.serve_trace(reqs, arr, target_rel_se=TARGET, ctx=ctx)
    assert st.completed == len(reqs)
    rep = served_check.check(orc, reqs, [o.result for o in out])
    log = os.environ.get("PCF_AUDIT_LOG")
    if log:
        with open(log, "a") as f:
            f.write(json.dumps({"served_check": rep["per_kind"]}) + "\n")
    pk = rep["per_kind"]
    assert set(pk) == {"eur", "asia", "basket", "amer"}
    for k in ("eur", "asia", "basket"):
        assert pk[k]["nan"] == 0 and pk[k]["checked"] > 30, (k, pk[k])
        assert pk[k]["outside_3se"] <= 2, (k, pk[k])
        assert pk[k]["max_abs_z"] < 4.5, (k, pk[k])
    for k in ("asia", "basket"):
        assert pk[k]["cv_mean_max_rel_err"] < 1e-9, (k, pk[k])
    assert pk["amer"]["checked"] > 30 and pk["amer"]["outside_bar"] == 0, pk["amer"]
    assert pk["amer"]["twin_outside"] == 0, pk["amer"]


def test_live_server_admits_while_running_and_matches_alone(ctx):
    """The live server (pcf_server_*): two host threads submit a mixed stream
    while earlier batches run. Every request completes near its target; some
    are admitted while others are still on the device (more than one batch
    in flight); and each result is the one that request gets alone at the
    same path count (exactly, or to 1e-8 where its main run continued its
    pilot, as in the trace replay)."""
    import threading
    import time

    import parcompfin_gb300 as pcf
    reqs, _ = _trace(pcf, 200, 4000.0, 5)
    srv = pcf.Server(ctx, target_rel_se=TARGET)
    tickets = {}
    lock = threading.Lock()

    def feed(lo, hi, gap):
        for i in range(lo, hi):
            t = srv.submit(reqs[i])
            with lock:
                tickets[i] = t
            time.sleep(gap)

    th = [threading.Thread(target=feed, args=(0, 100, 4e-4)),
          threading.Thread(target=feed, args=(100, 200, 3e-4))]
    for t in th:
        t.start()
    first = srv.poll(tickets.get(0, 0)) if tickets else None  # may well be pending
    for t in th:
        t.join()
    out = {i: srv.wait(tickets[i], 120.0) for i in range(200)}
    stats = srv.stop()
    assert first is None or first.status == 0
    assert all(o is not None and o.status == 0 for o in out.values())
    assert stats.completed == 200 and stats.batches >= 2
    assert stats.p50_ms <= stats.p99_ms <= stats.max_ms
    ad = sorted((o.admit_s, o.done_s) for o in out.values())
    overlap = sum(1 for k in range(1, len(ad)) if ad[k][0] < max(d for _, d in ad[:k]) and
                  ad[k][0] > ad[k - 1][0])
    assert overlap > 0
    for i, o in out.items():
        assert o.done_s >= o.admit_s >= o.arrival_s - 1e-9
        if not (reqs[i]["method"] == 3 and o.result.n_paths >= (1 << 21)):
            assert o.result.std_error / abs(o.result.price) < 1.35 * TARGET
    continued = 0
    for i in range(0, 200, 5):
        q = dict(reqs[i], N=out[i].result.n_paths)
        alone = pcf.price_batch([q], ctx=ctx)[0]
        if q["method"] == 3 or q["N"] <= PILOT:
            assert list(alone.sums) == list(out[i].result.sums), q
        else:
            continued += 1
            for a, b in zip(alone.sums, out[i].result.sums):
                assert abs(a - b) <= 1e-8 * max(abs(a), abs(b)), (q, a, b)
    assert continued > 0


def test_stop_while_other_threads_wait(ctx):
    """pcf_server_stop called while other threads are blocked in
    pcf_server_wait: stop drains every request, the waiters return with
    their results, and the server is freed only after they have returned."""
    import threading
    import time

    import parcompfin_gb300 as pcf
    reqs = [pcf.request("amer", 100.0, 100.0 + k % 7, .05, .3, 1.0, 1 << 20, "put", M=50,
                        seed=3, stream=k) for k in range(24)]
    reqs += [pcf.request("eur", 100.0, 100.0, .05, .2, 1.0, 1 << 22, "call", seed=3, stream=100 + k)
             for k in range(16)]
    srv = pcf.Server(ctx, target_rel_se=0.0)
    tickets = [srv.submit(q) for q in reqs]
    got = {}
    ready = threading.Barrier(4)

    def waiter(t):  # one call each: no call may start once stop has returned
        ready.wait()
        got[t] = srv.wait(t, -1.0)

    watched = [tickets[23], tickets[-2], tickets[-1]]
    th = [threading.Thread(target=waiter, args=(t,)) for t in watched]
    for t in th:
        t.start()
    ready.wait()
    time.sleep(0.05)  # the waiters are inside pcf_server_wait by now
    stats = srv.stop()
    for t in th:
        t.join(60)
        assert not t.is_alive()
    assert stats.completed == len(reqs)
    assert sorted(got) == sorted(watched)
    for t in watched:
        assert got[t].status == 0 and got[t].result.n_paths == reqs[t]["N"]
        assert math.isfinite(got[t].result.price) and got[t].result.price > 0


def test_empty_inputs(ctx):
    """An empty trace, and a live server that serves nothing, finish with
    nothing completed; an empty batch prices nothing."""
    import parcompfin_gb300 as pcf
    out, st = pcf.serve_trace([], [], target_rel_se=TARGET, ctx=ctx)
    assert out == [] and st.completed == 0
    srv = pcf.Server(ctx, target_rel_se=TARGET)
    stats = srv.stop()
    assert stats.completed == 0
    assert pcf.price_batch([], ctx=ctx) == []


def test_smallest_contracts_in_one_batch(orc, ctx):
    """One path (European, Asian, basket) and one antithetic pair (American)
    in one batch: every result is finite and equals the contract alone."""
    import parcompfin_gb300 as pcf
    reqs = [pcf.request("eur", 100, 100, .05, .2, 1.0, 1, "call", seed=1, stream=0),
            pcf.request("asia", 100, 100, .04, .3, 1.0, 1, "put", M=7, seed=1, stream=1),
            pcf.request("basket", 100, 100, .03, .25, 1.0, 1, "call", assets=5, rho=.2,
                        seed=1, stream=2),
            pcf.request("amer", 100, 110, .05, .3, 1.0, 2, "put", M=3, seed=1, stream=3)]
    out = pcf.price_batch(reqs, ctx=ctx)
    for q, r in zip(reqs, out):
        assert r.n_paths == q["N"] and math.isfinite(r.price), (q, r.price)
        alone = pcf.price_batch([q], ctx=ctx)[0]
        assert list(alone.sums) == list(r.sums)
    s = (C.c_double * 6)()
    orc.twin_mc_eur(100, 100, .05, .2, 1.0, 1, 1, 1, 0, s)
    assert abs(out[0].sums[0] - s[0]) <= 1e-5 * max(abs(s[0]), 1e-9)
