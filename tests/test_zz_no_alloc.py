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


def _same_twice(eng, mid, pid, w, num):
    ref = eng.AADriskAggregate(mid, pid, w, num)
    scale = np.abs(ref["risks"]).max()
    for _ in range(2):  # two calls in a row: the shared array is cleared by each call
        vals, agg, risks = _noalloc(eng, mid, pid, w, num)
        assert np.abs(vals - ref["payoffValues"]).max() <= 1e-12 * np.abs(ref["payoffValues"]).max()
        assert abs(agg - ref["riskPayoffValue"]) <= 1e-12 * abs(ref["riskPayoffValue"])
        assert np.abs(risks - ref["risks"]).max() <= 1e-12 * scale


@pytest.mark.parametrize("sobol", [0, 1])
def test_noalloc_matches_allocating_entry_point_twice(sobol):
    # 2^17 paths: more blocks than the array's reverse-sweep scratch holds, so the
    # allocation-free grid is capped below the allocating entry point's
    eng = Engine(0)
    s, t, v = W.dupire_surface(60, 30)
    u = W.UOC_BARRIER
    eng.putDupire(W.DUPIRE_SPOT, s, t, v, W.DUPIRE_MAXDT, "na_dup")
    eng.putBarrier(u["strike"], u["barrier"], u["maturity"], u["monitor_freq"], u["smooth"], 0, "na_uoc")
    eng.shapes("na_dup", "na_uoc")  # lower the pair (allocating) before the allocation-free calls
    w = np.array([1.0, 0.5])
    for prec in ("fp64", "fp32"):
        _same_twice(eng, "na_dup", "na_uoc", w, NumericalParam(numPath=1 << 17, useSobol=bool(sobol), precision=prec))
    eng.close()


@pytest.mark.parametrize("sobol", [0, 1])
def test_noalloc_black_scholes_european_twice(sobol):
    eng = Engine(0)
    b = W.BS_EUROPEAN
    eng.putBlackScholes(b["spot"], b["vol"], 0, b["rate"], b["div"], "na_bs")
    eng.putEuropean(b["strike"], b["maturity"], b["maturity"], "na_eu")
    eng.shapes("na_bs", "na_eu")
    for prec in ("fp64", "fp32"):
        _same_twice(eng, "na_bs", "na_eu", np.ones(1), NumericalParam(numPath=1 << 16, useSobol=bool(sobol),
                                                                        precision=prec))
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


def test_noalloc_refuses_multi_asset_model():
    # the multi-asset model runs other kernels: refused before anything is launched
    eng = Engine(0)
    W.put_md4(eng)
    npay, npar, _ = eng.shapes("md4", "md4_bk")
    v, r = np.zeros(npay), np.zeros(npar)
    agg = ctypes.c_double()
    nc = NumericalParam(numPath=1024, useSobol=True).c()
    rc = lib().cf_aad_risk_aggregate_noalloc(eng._h, b"md4", b"md4_bk", _p(np.ones(npay)), ctypes.byref(nc), _p(v),
                                             ctypes.byref(agg), _p(r))
    assert rc == -7  # CF_E_UNSUPPORTED
    assert not r.any()
    eng.close()
