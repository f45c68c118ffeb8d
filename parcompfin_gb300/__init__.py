"""GB300-native pricing engine for the hot path of moledoc/parcompfin.

The pricing functions run hand-written sm_103a CUDA kernels in libpcf.so
through its C ABI (include/pcf.h); see api.py for the functions that mirror
the reference's.
"""
from .api import (  # noqa: F401
    Context,
    Plan,
    Server,
    binom_embar,
    binom_embar_batch,
    binom_vanilla_amer,
    binom_vanilla_eur,
    price_batch,
    serve_trace,
    request,
    mc_amer,
    mc_amer_audit,
    mc_amer_result,
    mc_asia,
    mc_asia_result,
    mc_basket_result,
    mc_eur,
    mc_eur_multi,
    mc_eur_multi_result,
    mc_eur_result,
    payoff_code,
)
from ._lib import McResult, PcfError, load  # noqa: F401
