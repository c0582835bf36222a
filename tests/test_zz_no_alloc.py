"""cf_aad_risk_aggregate_noalloc: the AAD-risk entry point for callers that cannot let a
library allocate device memory during a call (device memory already held by another
allocator, or a cudaMalloc / cudaFree stall is not acceptable).  Its device storage is one
static 64 MiB array; its results must equal the allocating entry point's, call after call.

Collected last on purpose (file name) so that a failure here does not hide other tests.
"""
import ctypes

import numpy as np
import pytest

from compfinance_gb300 import Engine, NumericalParam
from compfinance_gb300 import workloads as W
from compfinance_gb300.api import _check, _p, lib

pytestmark = pytest.mark.gpu


def _noalloc(eng, mid, pid, w, num):
    npay, npar, _ = eng.shapes(mid, pid)
    v, r = np.zeros(npay), np.zeros(npar)
    agg = ctypes.c_double()
    nc = num.c()
    _check(lib().cf_aad_risk_aggregate_noalloc(eng._h, mid.encode(), pid.encode(), _p(np.ascontiguousarray(w)),
                                               ctypes.byref(nc), _p(v), ctypes.byref(agg), _p(r)))
    return v, agg.value, r


def test_noalloc_matches_allocating_entry_point_twice():
    eng = Engine(0)
    s, t, v = W.dupire_surface(60, 30)
    u = W.UOC_BARRIER
    eng.putDupire(W.DUPIRE_SPOT, s, t, v, W.DUPIRE_MAXDT, "na_dup")
    eng.putBarrier(u["strike"], u["barrier"], u["maturity"], u["monitor_freq"], u["smooth"], 0, "na_uoc")
    eng.shapes("na_dup", "na_uoc")  # lower the pair (allocating) before the allocation-free calls
    w = np.array([1.0, 0.5])
    for prec in ("fp64", "fp32"):
        num = NumericalParam(numPath=1 << 17, precision=prec)
        ref = eng.AADriskAggregate("na_dup", "na_uoc", w, num)
        scale = np.abs(ref["risks"]).max()
        for _ in range(2):  # two calls in a row: the shared array is cleared by each call
            vals, agg, risks = _noalloc(eng, "na_dup", "na_uoc", w, num)
            assert np.abs(vals - ref["payoffValues"]).max() <= 1e-12 * np.abs(ref["payoffValues"]).max()
            assert abs(agg - ref["riskPayoffValue"]) <= 1e-12 * abs(ref["riskPayoffValue"])
            assert np.abs(risks - ref["risks"]).max() <= 1e-12 * scale
    eng.close()


def test_noalloc_rejects_unlowered_pair():
    eng = Engine(0)
    eng.putBlackScholes(100.0, 0.2, 0, 0.02, 0.0, "na_bs")
    eng.putEuropean(100.0, 1.0, 1.0, "na_eu")
    v, r = np.zeros(1), np.zeros(4)
    agg = ctypes.c_double()
    nc = NumericalParam(numPath=1024, useSobol=True).c()
    rc = lib().cf_aad_risk_aggregate_noalloc(eng._h, b"na_bs", b"na_eu", _p(np.ones(1)), ctypes.byref(nc), _p(v),
                                             ctypes.byref(agg), _p(r))
    assert rc != 0
    eng.close()
