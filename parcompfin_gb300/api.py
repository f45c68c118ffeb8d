"""Python mirror of the reference's pricing functions, priced on the GPU.

Each function keeps the name, argument order and meaning of the reference
function it replaces and returns the price as a float, as the reference
does:

    mc_eur(S0, E, r, sigma, T, N, payoff_fun)            src/mc_eur.cpp:5-27
    mc_eur_multi(S0, E, r, sigma, T, N, payoff_fun, assets, rho)
                                                          src/mc_eur_multi.cpp:6-35
    mc_asia(S0, E, r, sigma, T, N, M, payoff_fun)        src/mc_asia.cpp:5-40
    mc_amer(S0, E, r, sigma, T, N, M, payoff_fun)        src/mc_amer.cpp:5-114
    binom_embar(S0, E, r, sigma, T, N, payoff_fun)       src/binom_embar.cpp:5-50
    binom_vanilla_eur(S0, E, r, sigma, T, N, payoff_fun) src/binom_vanilla_eur.cpp:5-39
    binom_vanilla_amer(S0, E, r, sigma, T, N, payoff_fun)
                                                          src/binom_vanilla_amer.cpp:5-40

payoff_fun is +1/-1 (the reference's encoding, include/common.h:56-60) or
the strings "call"/"put" its command lines accept (src/mc_eur.cpp:39-42).
Anything else raises ValueError("Unknown payoff function"), like the
reference's std::invalid_argument. Keyword-only extras (seed, use_cv, mode,
ctx) select what the reference fixes: the reference seeds from time(), and
here the Philox seed is explicit and defaults to 0. The *_result variants
return the full McResult (price, standard error, control-variate estimate,
raw moment sums).
"""
from __future__ import annotations

import ctypes as C

from . import _lib


def payoff_code(payoff_fun) -> int:
    if isinstance(payoff_fun, str):
        if payoff_fun == "call":
            return 1
        if payoff_fun == "put":
            return -1
        raise ValueError("Unknown payoff function")
    if payoff_fun in (1, 1.0):
        return 1
    if payoff_fun in (-1, -1.0):
        return -1
    raise ValueError("Unknown payoff function")


class Context:
    """A libpcf context: one CUDA stream plus resident device scratch."""

    def __init__(self, device: int = 0):
        lib = _lib.load()
        h = C.c_void_p()
        _lib.check(lib.pcf_ctx_create(int(device), C.byref(h)))
        self._h = h
        self.device = device

    @property
    def handle(self):
        return self._h

    @property
    def stream(self) -> int:
        return _lib.load().pcf_ctx_stream(self._h) or 0

    @property
    def launches(self) -> int:
        return int(_lib.load().pcf_ctx_launch_count(self._h))

    def release(self) -> None:
        """Free the device and pinned memory kept between calls."""
        _lib.check(_lib.load().pcf_ctx_release(self._h))

    def set_memory_limit(self, nbytes: int) -> None:
        """Cap each device buffer the context allocates (0: no cap)."""
        _lib.check(_lib.load().pcf_ctx_set_memory_limit(self._h, int(nbytes)))

    def set_test_barrier(self, extra_arrivals: int, poll_limit: int = 1) -> None:
        """Test hook: make the cooperative group barriers of mc_amer and the
        lattice pricers unable to complete (extra_arrivals > 0) so that they
        give up after poll_limit polls; 0 restores normal operation."""
        _lib.check(_lib.load().pcf_ctx_set_test_barrier(self._h, int(extra_arrivals),
                                                         int(poll_limit)))

    def autotune(self, mc: bool = True, lsm: bool = True, save: bool = False,
                 requests=None) -> dict:
        """Time candidate work shapes on this device and keep the fastest
        (pcf_autotune; with `requests`, pcf_autotune_batch times every knob on
        that batch); returns the JSON report as a dict."""
        import json
        flags = (_lib.TUNE_MC if mc else 0) | (_lib.TUNE_LSM if lsm else 0) | \
            (_lib.TUNE_SAVE if save else 0)
        buf = C.create_string_buffer(1 << 16)
        if requests:
            arr, keep = _pack(requests)
            _lib.check(_lib.load().pcf_autotune_batch(self._h, flags, len(requests), arr, buf,
                                                      len(buf)))
        else:
            _lib.check(_lib.load().pcf_autotune(self._h, flags, buf, len(buf)))
        return json.loads(buf.value.decode())

    def tuning(self) -> dict:
        """The work-shape table in force on this device."""
        import json
        buf = C.create_string_buffer(4096)
        _lib.check(_lib.load().pcf_tune_report(self._h, buf, len(buf)))
        return json.loads(buf.value.decode())

    def tune_reset(self) -> None:
        """Restore the built-in work shapes on this device."""
        _lib.check(_lib.load().pcf_tune_reset(self._h))

    def close(self) -> None:
        if self._h:
            _lib.load().pcf_ctx_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def _h(ctx):
    return None if ctx is None else ctx.handle


def mc_eur_result(S0, E, r, sigma, T, N, payoff_fun, *, seed=0, use_cv=False, ctx=None):
    lib = _lib.load()
    out = _lib.McResult()
    _lib.check(lib.pcf_mc_eur(_h(ctx), S0, E, r, sigma, T, int(N), payoff_code(payoff_fun),
                              int(seed), int(bool(use_cv)), C.byref(out)))
    return out


def mc_eur(S0, E, r, sigma, T, N, payoff_fun, *, seed=0, use_cv=False, ctx=None) -> float:
    return mc_eur_result(S0, E, r, sigma, T, N, payoff_fun, seed=seed, use_cv=use_cv,
                         ctx=ctx).price


def mc_asia_result(S0, E, r, sigma, T, N, M, payoff_fun, *, mode=0, seed=0, use_cv=False,
                   ctx=None):
    lib = _lib.load()
    out = _lib.McResult()
    _lib.check(lib.pcf_mc_asia(_h(ctx), S0, E, r, sigma, T, int(N), int(M),
                               payoff_code(payoff_fun), int(mode), int(seed),
                               int(bool(use_cv)), C.byref(out)))
    return out


def mc_asia(S0, E, r, sigma, T, N, M, payoff_fun, *, mode=0, seed=0, use_cv=False,
            ctx=None) -> float:
    return mc_asia_result(S0, E, r, sigma, T, N, M, payoff_fun, mode=mode, seed=seed,
                          use_cv=use_cv, ctx=ctx).price


def mc_eur_multi_result(S0, E, r, sigma, T, N, payoff_fun, assets, rho, *, seed=0,
                        use_cv=False, ctx=None):
    lib = _lib.load()
    out = _lib.McResult()
    _lib.check(lib.pcf_mc_eur_multi(_h(ctx), S0, E, r, sigma, T, int(N),
                                    payoff_code(payoff_fun), int(assets), float(rho),
                                    int(seed), int(bool(use_cv)), C.byref(out)))
    return out


def mc_eur_multi(S0, E, r, sigma, T, N, payoff_fun, assets, rho, *, seed=0, use_cv=False,
                 ctx=None) -> float:
    return mc_eur_multi_result(S0, E, r, sigma, T, N, payoff_fun, assets, rho, seed=seed,
                               use_cv=use_cv, ctx=ctx).price


def mc_amer_result(S0, E, r, sigma, T, N, M, payoff_fun, *, ref_exercise=False, seed=0,
                   use_cv=False, ctx=None):
    lib = _lib.load()
    out = _lib.McResult()
    _lib.check(lib.pcf_mc_amer(_h(ctx), S0, E, r, sigma, T, int(N), int(M),
                               payoff_code(payoff_fun), int(bool(ref_exercise)), int(seed),
                               int(bool(use_cv)), C.byref(out)))
    return out


def mc_amer(S0, E, r, sigma, T, N, M, payoff_fun, *, ref_exercise=False, seed=0, use_cv=False,
            ctx=None) -> float:
    """src/mc_amer.cpp:5-114. ref_exercise=True reproduces the reference's
    exercise value payoff(S - E, E) (src/mc_amer.cpp:100)."""
    return mc_amer_result(S0, E, r, sigma, T, N, M, payoff_fun, ref_exercise=ref_exercise,
                          seed=seed, use_cv=use_cv, ctx=ctx).price


BINOM_MODES = {"reference": 0, "accurate": 1}


def mc_amer_audit(S0, E, r, sigma, T, N, M, payoff_fun, *, ref_exercise=False, seed=0,
                  want_paths=True, ctx=None):
    """mc_amer with the audit record of the sweep (pcf_mc_amer_audit).

    Returns (result, coef[M][4], sums[M][8], tau[N], u[M][N] or None) as
    numpy arrays; see include/pcf.h for their meaning. A status other than
    PCF_OK or PCF_ESINGULAR raises; on PCF_ESINGULAR the record is returned
    with result = None."""
    import numpy as np
    lib = _lib.load()
    out = _lib.McResult()
    N, M = int(N), int(M)
    coef = np.zeros((M, 4), np.float32)
    sums = np.zeros((M, 8), np.float64)
    tau = np.zeros(N, np.uint16)
    u = np.zeros((M, N), np.float32) if want_paths else None
    fp = C.POINTER(C.c_float)
    st = lib.pcf_mc_amer_audit(
        _h(ctx), S0, E, r, sigma, T, N, M, payoff_code(payoff_fun), int(bool(ref_exercise)),
        int(seed), C.byref(out), coef.ctypes.data_as(fp),
        sums.ctypes.data_as(C.POINTER(C.c_double)), tau.ctypes.data_as(C.POINTER(C.c_ushort)),
        u.ctypes.data_as(fp) if u is not None else None)
    if st == _lib.PCF_ESINGULAR:
        return None, coef, sums, tau, u
    _lib.check(st)
    return out, coef, sums, tau, u


def binom_embar(S0, E, r, sigma, T, N, payoff_fun, *, mode="reference", ctx=None) -> float:
    """src/binom_embar.cpp:5-50 (function binom). mode "reference" reproduces
    the reference's FP64 result; "accurate" uses exact-to-rounding weights."""
    lib = _lib.load()
    out = C.c_double()
    _lib.check(lib.pcf_binom_embar(_h(ctx), S0, E, r, sigma, T, int(N), payoff_code(payoff_fun),
                                   BINOM_MODES.get(mode, mode), C.byref(out)))
    return out.value


def binom_embar_batch(contracts, *, mode="reference", ctx=None) -> list:
    """contracts: iterable of (S0, E, r, sigma, T, N, payoff_fun); one launch."""
    lib = _lib.load()
    cs = list(contracts)
    arr = (_lib.BinomContract * len(cs))()
    for k, (S0, E, r, sigma, T, N, pf) in enumerate(cs):
        arr[k] = _lib.BinomContract(S0, E, r, sigma, T, int(N), payoff_code(pf))
    out = (C.c_double * len(cs))()
    _lib.check(lib.pcf_binom_embar_batch(_h(ctx), len(cs), arr, BINOM_MODES.get(mode, mode), out))
    return list(out)


def _binom_vanilla(S0, E, r, sigma, T, N, payoff_fun, american, ctx):
    lib = _lib.load()
    out = C.c_double()
    _lib.check(lib.pcf_binom_vanilla(_h(ctx), S0, E, r, sigma, T, int(N), payoff_code(payoff_fun),
                                     1 if american else 0, C.byref(out)))
    return out.value


def binom_vanilla_eur(S0, E, r, sigma, T, N, payoff_fun, *, ctx=None) -> float:
    """src/binom_vanilla_eur.cpp:5-39 (function binom): European backward
    induction on the reference's lattice, bit for bit its FP64 result."""
    return _binom_vanilla(S0, E, r, sigma, T, N, payoff_fun, False, ctx)


def binom_vanilla_amer(S0, E, r, sigma, T, N, payoff_fun, *, ctx=None) -> float:
    """src/binom_vanilla_amer.cpp:5-40 (function binom): American backward
    induction on the reference's lattice, bit for bit its FP64 result."""
    return _binom_vanilla(S0, E, r, sigma, T, N, payoff_fun, True, ctx)


METHODS = {"eur": _lib.METHOD_EUR, "asia": _lib.METHOD_ASIA, "basket": _lib.METHOD_BASKET,
           "amer": _lib.METHOD_AMER}


def request(method, S0, E, r, sigma, T, N, payoff_fun, *, M=0, mode=0, use_cv=False,
            assets=0, rho=0.0, basket_S0=None, basket_sigma=None, corr=None,
            scale_by_sqrt_T=True, seed=0, stream=0) -> dict:
    """One pricing request for price_batch / Plan (a dict of pcf_mc_request fields)."""
    return dict(method=METHODS[method] if isinstance(method, str) else int(method),
                payoff_fun=payoff_code(payoff_fun), S0=float(S0), E=float(E), r=float(r),
                sigma=float(sigma), T=float(T), N=int(N), M=int(M), mode=int(mode),
                use_cv=int(bool(use_cv)), assets=int(assets), rho=float(rho),
                basket_S0=basket_S0, basket_sigma=basket_sigma, corr=corr,
                scale_by_sqrt_T=int(bool(scale_by_sqrt_T)), seed=int(seed), stream=int(stream))


def _pack(reqs):
    arr = (_lib.McRequest * len(reqs))()
    keep = []
    for i, q in enumerate(reqs):
        x = arr[i]
        for k, v in q.items():
            if k in ("basket_S0", "basket_sigma", "corr"):
                if v is None:
                    continue
                flat = [float(t) for row in v for t in row] if hasattr(v[0], "__len__") else \
                    [float(t) for t in v]
                buf = (C.c_double * len(flat))(*flat)
                keep.append(buf)
                setattr(x, k, C.cast(buf, C.POINTER(C.c_double)))
            else:
                setattr(x, k, v)
    return arr, keep


class Plan:
    """Device-resident batch: upload once, launch many times. From the second
    launch on the launch sequence replays a CUDA graph (graph=False: always
    launch directly)."""

    def __init__(self, reqs, ctx=None, graph=True):
        lib = _lib.load()
        arr, keep = _pack(reqs)
        h = C.c_void_p()
        _lib.check(lib.pcf_plan_create(_h(ctx), len(reqs), arr, C.byref(h)))
        self._h, self.n = h, len(reqs)
        if not graph:
            _lib.check(lib.pcf_plan_set_graph(self._h, 0))

    @property
    def uses_graph(self) -> bool:
        return bool(_lib.load().pcf_plan_uses_graph(self._h))

    def launch(self):
        _lib.check(_lib.load().pcf_plan_launch(self._h))

    def results(self):
        out = (_lib.McResult * self.n)()
        _lib.check(_lib.load().pcf_plan_results(self._h, out))
        return list(out)

    @property
    def kernel_count(self) -> int:
        return int(_lib.load().pcf_plan_kernel_count(self._h))

    def close(self):
        if self._h:
            _lib.load().pcf_plan_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def serve_trace(reqs, arrivals, *, target_rel_se=5e-4, pilot_paths=1 << 14, max_paths=1 << 26,
                max_amer_paths=1 << 21, max_batch=2048, slots=12, hbm_fraction=0.5, ctx=None):
    """Serve request() dicts arriving at `arrivals` (seconds, non-decreasing)
    with the continuous-batching loop; returns (per-request ServedResult list,
    ServerStats)."""
    lib = _lib.load()
    arr, keep = _pack(reqs)
    t = (C.c_double * len(reqs))(*map(float, arrivals))
    cfg = _lib.ServerConfig(float(target_rel_se), int(pilot_paths), int(max_paths),
                            int(max_amer_paths), int(max_batch), int(slots), float(hbm_fraction))
    out = (_lib.ServedResult * len(reqs))()
    stats = _lib.ServerStats()
    st = lib.pcf_serve_trace(_h(ctx), C.byref(cfg), len(reqs), arr, t, out, C.byref(stats))
    if st not in (_lib.PCF_OK, _lib.PCF_ESINGULAR):
        _lib.check(st)
    return list(out), stats


def price_batch(reqs, ctx=None):
    """Price a list of request() dicts in one call; returns McResult per request."""
    lib = _lib.load()
    arr, keep = _pack(reqs)
    out = (_lib.McResult * len(reqs))()
    _lib.check(lib.pcf_price_batch(_h(ctx), len(reqs), arr, out))
    return list(out)


def mc_basket_result(S0s, sigmas, corr, r, T, E, N, payoff_fun, *, scale_by_sqrt_T=True,
                     seed=0, use_cv=False, ctx=None):
    """General basket: per-asset spots and vols, full correlation matrix."""
    lib = _lib.load()
    d = len(S0s)
    flat = [float(x) for row in corr for x in row] if hasattr(corr[0], "__len__") else \
        [float(x) for x in corr]
    if len(sigmas) != d or len(flat) != d * d:
        raise ValueError("S0s, sigmas and corr sizes do not match")
    A = C.c_double * d
    out = _lib.McResult()
    _lib.check(lib.pcf_mc_basket(_h(ctx), d, A(*map(float, S0s)), A(*map(float, sigmas)),
                                 (C.c_double * (d * d))(*flat), r, T, E, int(N),
                                 payoff_code(payoff_fun), int(bool(scale_by_sqrt_T)),
                                 int(seed), int(bool(use_cv)), C.byref(out)))
    return out


class Server:
    """The live continuous-batching server (pcf_server_*): start it on a
    context, submit requests from any thread while it runs, poll or wait for
    each result by its ticket, stop it to drain and get the latency stats.
    The context belongs to the server until stop()."""

    def __init__(self, ctx, *, target_rel_se=5e-4, pilot_paths=1 << 14, max_paths=1 << 26,
                 max_amer_paths=1 << 21, max_batch=2048, slots=12, hbm_fraction=0.5):
        lib = _lib.load()
        cfg = _lib.ServerConfig(float(target_rel_se), int(pilot_paths), int(max_paths),
                                int(max_amer_paths), int(max_batch), int(slots),
                                float(hbm_fraction))
        h = C.c_void_p()
        _lib.check(lib.pcf_server_start(_h(ctx), C.byref(cfg), C.byref(h)))
        self._h = h
        self._keep = []

    def submit(self, req) -> int:
        arr, keep = _pack([req])
        self._keep.append(keep)
        t = C.c_longlong()
        _lib.check(_lib.load().pcf_server_submit(self._h, arr, C.byref(t)))
        return t.value

    def poll(self, ticket):
        """The ServedResult if finished, else None."""
        out = _lib.ServedResult()
        st = _lib.load().pcf_server_poll(self._h, int(ticket), C.byref(out))
        if st == _lib.PCF_PENDING:
            return None
        _lib.check(st)
        return out

    def wait(self, ticket, timeout_s=-1.0):
        out = _lib.ServedResult()
        st = _lib.load().pcf_server_wait(self._h, int(ticket), float(timeout_s), C.byref(out))
        if st == _lib.PCF_PENDING:
            return None
        _lib.check(st)
        return out

    def stop(self):
        """Drain, stop and return the ServerStats."""
        stats = _lib.ServerStats()
        st = _lib.load().pcf_server_stop(self._h, C.byref(stats))
        self._h = None
        if st not in (_lib.PCF_OK, _lib.PCF_ESINGULAR):
            _lib.check(st)
        return stats
