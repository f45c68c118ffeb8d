"""The work-shape table and the autotuner (pcf_autotune, pcf_tune_*).

A work shape changes how paths are grouped into per-thread and per-block
partial sums, never which paths are priced: under any table every kernel
still matches its FP64 twin on the identical Philox draws (1e-5 relative;
3e-4 for American puts, the policy audit's boundary-flip bar), and a
contract's sums are the same alone and inside a batch.
"""
import ctypes as C
import json
import os
import subprocess
import sys
import textwrap

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHECK = textwrap.dedent('''
    import ctypes as C, math, sys
    sys.path.insert(0, sys.argv[1])
    import numpy as np
    import parcompfin_gb300 as pcf
    from oracle import loader
    orc = loader.load()
    rel = lambda a, b: abs(a - b) / abs(b)
    with pcf.Context(0) as ctx:
        t = ctx.tuning()["table"]
        assert t["tuned"] and t["eur_block"] == int(sys.argv[2]), t
        reqs = [pcf.request("eur", 100, 100, .05, .2, 1.0, 300_001, "call", seed=5, stream=0),
                pcf.request("asia", 100, 95, .04, .3, 1.0, 20_000, "call", M=52, seed=5, stream=1)]
        bask = []
        for i, d in enumerate((4, 8, 16, 24)):
            corr = np.full((d, d), .3); np.fill_diagonal(corr, 1.0)
            sig = [.15 + .2 * a / d for a in range(d)]
            reqs.append(pcf.request("basket", 100, 100, .03, .25, 1.0, 30_000, "call", assets=d,
                                    basket_sigma=sig, corr=corr.tolist(), use_cv=True, seed=7,
                                    stream=10 + i))
            bask.append((d, sig, np.linalg.cholesky(corr).ravel()))
        reqs.append(pcf.request("amer", 100, 100, .05, .3, 1.0, 1 << 17, "put", M=50, seed=5,
                                stream=20))
        out = pcf.price_batch(reqs, ctx=ctx)
        s = (C.c_double * 6)()
        orc.twin_mc_eur(100, 100, .05, .2, 1.0, 300_001, 1, 5, 0, s)
        assert rel(out[0].sums[0], s[0]) < 1e-5, (out[0].sums[0], s[0])
        orc.twin_mc_asia(100, 95, .04, .3, 1.0, 20_000, 52, 1, 0, 5, 1, s)
        assert rel(out[1].sums[0], s[0]) < 1e-5
        for i, (d, sig, L) in enumerate(bask):
            A = C.c_double * d
            orc.twin_mc_basket(d, A(*[100.0] * d), A(*sig), (C.c_double * (d * d))(*L), .03, 1.0,
                               1.0, 100.0, 30_000, 1, 7, 10 + i, s)
            for k in range(5):
                assert rel(out[2 + i].sums[k], s[k]) < 1e-5, (d, k)
        orc.twin_mc_amer(100, 100, .05, .3, 1.0, 1 << 17, 50, -1, 0, 5, 20, s)
        assert rel(out[-1].sums[0], s[0]) < 3e-4
        alone = pcf.price_batch([reqs[3]], ctx=ctx)[0]
        assert list(alone.sums) == list(out[3].sums)
    print("SHAPES OK")
''')


@pytest.mark.parametrize("shape", [
    dict(eur_block=128, eur_items="8,16,64,128", asia_block=512, asia_steps="128,256,1024,2048",
         basket_block="128,512,128,256", basket_ppt="2,32,4,4", tc_tiles="2,16", tc_min_d=33,
         lsm_shift="0,0,1,1,1,1,1,0"),
    dict(eur_block=512, eur_items="128,64,16,8", asia_block=128, asia_steps="2048,1024,256,128",
         basket_block="512,128,512,128", basket_ppt="32,2,16,2", tc_tiles="32,4", tc_min_d=20,
         lsm_shift="0,0,-1,-1,-1,-1,-1,0"),
])
def test_every_work_shape_matches_the_twins(ctx, tmp_path, shape):
    """A tuning cache with non-default shapes (block sizes 128 and 512, other
    items per thread and tiles per item, other LSM cluster shapes) is loaded
    by a fresh process, whose prices match the FP64 twins."""
    dev = ctx.tuning()["device"]
    f = tmp_path / "tune.txt"
    lines = [f"device={dev}", "eur_max_quads=64"] + [f"{k}={v}" for k, v in shape.items()]
    f.write_text("\n".join(lines) + "\n")
    env = dict(os.environ, PCF_TUNE_CACHE=str(f))
    r = subprocess.run([sys.executable, "-c", CHECK, ROOT, str(shape["eur_block"])],
                       capture_output=True, text=True, env=env, timeout=600)
    assert r.returncode == 0 and "SHAPES OK" in r.stdout, r.stdout + r.stderr


def test_autotune_then_results_hold_and_reset(orc, ctx):
    """pcf_autotune times its candidates and keeps a table of valid shapes;
    afterwards the engine still matches its twins and a contract is the same
    alone and in a batch; pcf_tune_reset restores the built-in table."""
    import parcompfin_gb300 as pcf
    rep = ctx.autotune()
    try:
        t = ctx.tuning()["table"]
        assert t["tuned"]
        assert t["eur_block"] in (128, 256, 512) and t["asia_block"] in (128, 256, 512)
        assert rep["table"] == t and len(rep["trials"]) > 50
        assert 17 <= t["tc_min_d"] <= 33
        assert {x["knob"] for x in rep["trials"]} >= {"eur_block", "asia_block", "lsm_shift[2]"}
        reqs = [pcf.request("eur", 100, 100, .05, .2, 1.0, 1 << 20, "call", seed=3, stream=0),
                pcf.request("asia", 100, 100, .04, .3, 1.0, 50_000, "call", M=252, seed=3,
                            stream=1),
                pcf.request("amer", 100, 95, .05, .3, 1.0, 1 << 16, "put", M=50, seed=3,
                            stream=2)]
        out = pcf.price_batch(reqs, ctx=ctx)
        s = (C.c_double * 6)()
        orc.twin_mc_eur(100, 100, .05, .2, 1.0, 1 << 20, 1, 3, 0, s)
        assert abs(out[0].sums[0] - s[0]) < 1e-5 * s[0]
        orc.twin_mc_asia(100, 100, .04, .3, 1.0, 50_000, 252, 1, 0, 3, 1, s)
        assert abs(out[1].sums[0] - s[0]) < 1e-5 * s[0]
        orc.twin_mc_amer(100, 95, .05, .3, 1.0, 1 << 16, 50, -1, 0, 3, 2, s)
        assert abs(out[2].sums[0] - s[0]) < 3e-4 * s[0]
        for i, q in enumerate(reqs):
            assert list(pcf.price_batch([q], ctx=ctx)[0].sums) == list(out[i].sums)
    finally:
        ctx.tune_reset()
    t = ctx.tuning()["table"]
    assert not t["tuned"] and t["eur_block"] == 256 and t["basket_ppt"] == [16, 8, 8, 4]
    assert t["tc_min_d"] == 24


def test_autotune_on_a_batch_tunes_only_what_the_batch_uses(orc, ctx):
    """pcf_autotune_batch times every knob on the caller's batch and leaves
    alone the knobs that shape none of it (European-only batch: no Asian,
    basket or American knob is timed); prices stay at the twins' values."""
    import parcompfin_gb300 as pcf
    reqs = [pcf.request("eur", 100, 90 + 2 * k, .05, .2, 1.0, 1 << 20, "call", seed=9, stream=k)
            for k in range(16)]
    try:
        rep = ctx.autotune(requests=reqs)
        assert rep["mode"] == "batch"
        knobs = {x["knob"] for x in rep["trials"]}
        assert "eur_block" in knobs and "eur_items[1]" in knobs
        assert not any(k.startswith(("asia", "basket", "tc_", "lsm")) for k in knobs), knobs
        out = pcf.price_batch(reqs, ctx=ctx)
        s = (C.c_double * 6)()
        for k in (0, 15):
            orc.twin_mc_eur(100, 90 + 2 * k, .05, .2, 1.0, 1 << 20, 1, 9, k, s)
            assert abs(out[k].sums[0] - s[0]) < 1e-5 * s[0]
    finally:
        ctx.tune_reset()
