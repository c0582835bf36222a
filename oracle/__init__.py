"""ctypes bindings of the CPU restatement in oracle/oracle.cpp.

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()`` (as the
checker) and by ``bench.py``'s CPU-baseline leg.  The engine never imports this package.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")

_dp = ctypes.POINTER(ctypes.c_double)


class OrcModel(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("spot", ctypes.c_double), ("vol", ctypes.c_double),
                ("rate", ctypes.c_double), ("div", ctypes.c_double), ("spot_measure", ctypes.c_int),
                ("nS", ctypes.c_int), ("nT", ctypes.c_int), ("spots", _dp), ("times", _dp), ("vols", _dp),
                ("maxdt", ctypes.c_double)]


class OrcProduct(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("strike", ctypes.c_double), ("exercise", ctypes.c_double),
                ("settlement", ctypes.c_double), ("barrier", ctypes.c_double), ("maturity", ctypes.c_double),
                ("freq", ctypes.c_double), ("smooth", ctypes.c_double), ("callput", ctypes.c_int),
                ("n", ctypes.c_int), ("mats", _dp), ("strikes", _dp), ("coupon", ctypes.c_double)]


class OrcIvs(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("spot", ctypes.c_double), ("p", ctypes.c_double * 4)]


def build(force=False):
    """Compile liboracle.so with g++ (no fp-contraction, no fast-math)."""
    src = os.path.join(HERE, "oracle.cpp")
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(src):
        return LIB
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared",
                           src, "-o", LIB, "-lpthread"])
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = ctypes.CDLL(LIB)
        _lib.orc_inv_normal_cdf.restype = ctypes.c_double
        _lib.orc_normal_cdf.restype = ctypes.c_double
    return _lib


def _arr(x):
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float64))
    return a, a.ctypes.data_as(_dp)


class Model:
    """Holds the ctypes struct and keeps its arrays alive."""

    def __init__(self, spec):
        self.spec = spec
        self._keep = []
        m = OrcModel()
        m.spot = spec["spot"]
        if spec["kind"] == "bs":
            m.kind = 0
            m.vol, m.rate, m.div = spec["vol"], spec["rate"], spec["div"]
            m.spot_measure = int(spec.get("qspot", 0))
        else:
            m.kind = 1
            s, ps = _arr(spec["spots"])
            t, pt = _arr(spec["times"])
            v, pv = _arr(np.asarray(spec["vols"]).reshape(-1))
            self._keep += [s, t, v]
            m.nS, m.nT = len(s), len(t)
            m.spots, m.times, m.vols = ps, pt, pv
            m.maxdt = spec["maxdt"]
        self.c = m


class Product:
    def __init__(self, spec):
        self.spec = spec
        self._keep = []
        p = OrcProduct()
        if spec["kind"] == "european":
            p.kind = 0
            p.strike, p.exercise, p.settlement = spec["strike"], spec["exercise"], spec["settlement"]
        elif spec["kind"] == "uoc":
            p.kind = 1
            p.strike, p.barrier, p.maturity = spec["strike"], spec["barrier"], spec["maturity"]
            p.freq, p.smooth, p.callput = spec["freq"], spec["smooth"], int(spec.get("callput", 0))
        elif spec["kind"] == "contingent":
            p.kind = 3
            p.coupon, p.maturity, p.freq, p.smooth = spec["coupon"], spec["maturity"], spec["freq"], spec["smooth"]
        else:
            p.kind = 2
            m, pm = _arr(spec["mats"])
            k, pk = _arr(spec["strikes"])
            self._keep += [m, k]
            p.n, p.mats, p.strikes = len(m), pm, pk
        self.c = p


def shapes(model, product):
    a, b, c = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    lib().orc_shapes(ctypes.byref(model.c), ctypes.byref(product.c), ctypes.byref(a), ctypes.byref(b),
                     ctypes.byref(c))
    return a.value, b.value, c.value


def value(model, product, sobol, npath, seed1=12345, seed2=1234, threads=1):
    npay, _, _ = shapes(model, product)
    v, pv = _arr(np.zeros(npay))
    e, pe = _arr(np.zeros(npay))
    lib().orc_value(ctypes.byref(model.c), ctypes.byref(product.c), int(sobol), int(npath), seed1, seed2,
                    int(threads), pv, pe)
    return v, e


def paths(model, product, sobol, npath, seed1=12345, seed2=1234):
    npay, _, _ = shapes(model, product)
    out, po = _arr(np.zeros(npath * npay))
    lib().orc_paths(ctypes.byref(model.c), ctypes.byref(product.c), int(sobol), int(npath), seed1, seed2, po)
    return out.reshape(npath, npay)


def risk(model, product, sobol, npath, weights, seed1=12345, seed2=1234, fast=False, threads=1):
    npay, npar, _ = shapes(model, product)
    w, pw = _arr(weights)
    v, pv = _arr(np.zeros(npay))
    r, pr = _arr(np.zeros(npar))
    agg = ctypes.c_double()
    if fast:
        lib().orc_risk_fast(ctypes.byref(model.c), ctypes.byref(product.c), int(sobol), int(npath), seed1, seed2,
                            pw, int(threads), pv, ctypes.byref(agg), pr)
    else:
        lib().orc_risk(ctypes.byref(model.c), ctypes.byref(product.c), int(sobol), int(npath), seed1, seed2, pw,
                       pv, ctypes.byref(agg), pr)
    return v, agg.value, r


def risk_multi(model, product, sobol, npath, seed1=12345, seed2=1234, ref_quirk=False):
    npay, npar, _ = shapes(model, product)
    v, pv = _arr(np.zeros(npay))
    r, pr = _arr(np.zeros(npar * npay))
    lib().orc_risk_multi(ctypes.byref(model.c), ctypes.byref(product.c), int(sobol), int(npath), seed1, seed2,
                         int(ref_quirk), pv, pr)
    return v, r.reshape(npar, npay)


def sobol_ints(dim, first, n):
    out = np.zeros(n * dim, dtype=np.uint32)
    rc = lib().orc_sobol_ints(int(dim), ctypes.c_int64(first), int(n),
                              out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)))
    assert rc == 0
    return out.reshape(n, dim)


def sobol_gauss(dim, first, n):
    out, po = _arr(np.zeros(n * dim))
    lib().orc_sobol_gauss(int(dim), ctypes.c_int64(first), int(n), po)
    return out.reshape(n, dim)


def mrg_gauss(seed1, seed2, dim, first, n):
    out, po = _arr(np.zeros(n * dim))
    lib().orc_mrg_gauss(seed1, seed2, int(dim), ctypes.c_int64(first), int(n), po)
    return out.reshape(n, dim)


def mrg_state(seed1, seed2, dim, first):
    out, po = _arr(np.zeros(6))
    lib().orc_mrg_state(seed1, seed2, int(dim), ctypes.c_int64(first), po)
    return out.astype(np.int64)


def inv_normal_cdf(p):
    return lib().orc_inv_normal_cdf(ctypes.c_double(p))


def normal_cdf(x):
    return lib().orc_normal_cdf(ctypes.c_double(x))


def ivs(kind, spot, params):
    s = OrcIvs()
    s.kind = 0 if kind == "param" else 1
    s.spot = spot
    for i, x in enumerate(params):
        s.p[i] = x
    return s


def calib(iv, incl_spots, max_ds, incl_times, max_dt_vol):
    isp, pis = _arr(incl_spots)
    itm, pit = _arr(incl_times)
    nS, nT = ctypes.c_int(), ctypes.c_int()
    lib().orc_calib(ctypes.byref(iv), pis, len(isp), ctypes.c_double(max_ds), pit, len(itm),
                    ctypes.c_double(max_dt_vol), ctypes.byref(nS), ctypes.byref(nT), None, None, None)
    s, ps = _arr(np.zeros(nS.value))
    t, pt = _arr(np.zeros(nT.value))
    lv, pl = _arr(np.zeros(nS.value * nT.value))
    lib().orc_calib(ctypes.byref(iv), pis, len(isp), ctypes.c_double(max_ds), pit, len(itm),
                    ctypes.c_double(max_dt_vol), ctypes.byref(nS), ctypes.byref(nT), ps, pt, pl)
    return s, t, lv.reshape(nS.value, nT.value)


def calib_adjoint(iv, incl_spots, max_ds, incl_times, max_dt_vol, rv_strikes, rv_mats, micro, ref_quirk=False):
    isp, pis = _arr(incl_spots)
    itm, pit = _arr(incl_times)
    k, pk = _arr(rv_strikes)
    m, pm = _arr(rv_mats)
    mb, pmb = _arr(np.asarray(micro).reshape(-1))
    vega, pv = _arr(np.zeros(len(k) * len(m)))
    lib().orc_calib_adjoint(ctypes.byref(iv), pis, len(isp), ctypes.c_double(max_ds), pit, len(itm),
                            ctypes.c_double(max_dt_vol), pk, len(k), pm, len(m), pmb, int(ref_quirk), pv)
    return vega.reshape(len(k), len(m))


def calib_adjoint_given(iv, incl_spots, max_ds, incl_times, max_dt_vol, rv_strikes, rv_mats, micro, calls=None,
                        vegas=None, ref_quirk=False):
    """The calibration adjoint restated pointwise: each node's five calls enter the tape as one
    node of their implied vol, with the given values `calls` and partials `vegas` ([nT][nS][5],
    per node (K,T), (K,T-h), (K,T+h), (K-h,T), (K+h,T)); None: the oracle's own.  Returns a dict:
    vega [strike][mat]; calls, vegas (the oracle's own) and pointAdj (the adjoint of each point's
    implied vol), [nT][nS][5]; absTerms [strike][mat], the sum of |pointAdj| x interpolation
    weight over the points, the scale of the terms that cancel in vega."""
    isp, pis = _arr(incl_spots)
    itm, pit = _arr(incl_times)
    k, pk = _arr(rv_strikes)
    m, pm = _arr(rv_mats)
    mb, pmb = _arr(np.asarray(micro).reshape(-1))
    s, t, _lv = calib(iv, incl_spots, max_ds, incl_times, max_dt_vol)
    n5 = len(s) * len(t) * 5
    own, po = _arr(np.zeros(n5))
    ownv, pov = _arr(np.zeros(n5))
    padj, ppa = _arr(np.zeros(n5))
    pc = pvg = None
    if calls is not None:
        c, pc = _arr(np.asarray(calls).reshape(-1))
        assert c.size == n5
    if vegas is not None:
        vg, pvg = _arr(np.asarray(vegas).reshape(-1))
        assert vg.size == n5
    vega, pv = _arr(np.zeros(len(k) * len(m)))
    absT, pab = _arr(np.zeros(len(k) * len(m)))
    lib().orc_calib_adjoint_given(ctypes.byref(iv), pis, len(isp), ctypes.c_double(max_ds), pit, len(itm),
                                  ctypes.c_double(max_dt_vol), pk, len(k), pm, len(m), pmb, int(ref_quirk), pc, pvg,
                                  po, pov, ppa, pab, pv, 1)
    shape = (len(t), len(s), 5)
    return dict(vega=vega.reshape(len(k), len(m)), calls=own.reshape(shape), vegas=ownv.reshape(shape),
                pointAdj=padj.reshape(shape), absTerms=absT.reshape(len(k), len(m)))


def superbucket(iv, spot, maxdt, product, notionals, incl_spots, max_ds, incl_times, max_dt_vol,
                rv_strikes, rv_mats, sobol, npath, seed1=12345, seed2=1234, ref_quirk=False):
    isp, pis = _arr(incl_spots)
    itm, pit = _arr(incl_times)
    k, pk = _arr(rv_strikes)
    m, pm = _arr(rv_mats)
    nots, pn = _arr(notionals)
    s, _t, _lv = calib(iv, incl_spots, max_ds, incl_times, max_dt_vol)
    vega, pv = _arr(np.zeros(len(k) * len(m)))
    micro, pmb = _arr(np.zeros(len(s) * len(_t)))
    val, dl = ctypes.c_double(), ctypes.c_double()
    lib().orc_superbucket(ctypes.byref(iv), ctypes.c_double(spot), ctypes.c_double(maxdt), ctypes.byref(product.c),
                          pn, pis, len(isp), ctypes.c_double(max_ds), pit, len(itm), ctypes.c_double(max_dt_vol),
                          pk, len(k), pm, len(m), int(sobol), int(npath), seed1, seed2, int(ref_quirk),
                          ctypes.byref(val),
                          ctypes.byref(dl), pv, pmb)
    return val.value, dl.value, vega.reshape(len(k), len(m)), micro.reshape(len(s), len(_t))


def fill(x, maxdx, mindx, add=()):
    xa, px = _arr(x)
    aa, pa = _arr(add if len(add) else [0.0])
    n = lib().orc_fill(px, len(xa), ctypes.c_double(maxdx), ctypes.c_double(mindx), pa, len(add), None)
    out, po = _arr(np.zeros(n))
    lib().orc_fill(px, len(xa), ctypes.c_double(maxdx), ctypes.c_double(mindx), pa, len(add), po)
    return out


# ---- multi-asset displaced model and products (mcMdlMultiDisplaced.h, mcPrdMulti.h) ----
class OrcMModel(ctypes.Structure):
    _fields_ = [("nA", ctypes.c_int), ("disc", ctypes.c_double), ("spots", _dp), ("spreads", _dp),
                ("nDiv", ctypes.c_int), ("divDates", _dp), ("divs", _dp), ("atms", _dp), ("skews", _dp),
                ("correl", _dp), ("lambda_", ctypes.c_double)]


class OrcMProduct(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("nA", ctypes.c_int), ("weights", _dp), ("maturity", ctypes.c_double),
                ("nK", ctypes.c_int), ("strikes", _dp), ("refs", _dp), ("periods", ctypes.c_int),
                ("ko", ctypes.c_double), ("strike", ctypes.c_double), ("cpn", ctypes.c_double),
                ("smooth", ctypes.c_double)]


class MModel:
    """spec: assets, spots, atms, skews, disc, spreads, div_dates, divs [nDiv][nA], correl [nA][nA], lambda."""

    def __init__(self, spec):
        self.spec = spec
        n = len(spec["assets"])
        self._keep = []
        m = OrcMModel()
        m.nA, m.disc, m.lambda_ = n, spec["disc"], spec["lambda"]

        def arr(x):
            a, p = _arr(np.asarray(x, dtype=float).reshape(-1) if np.size(x) else [0.0])
            self._keep.append(a)
            return p
        m.spots, m.spreads = arr(spec["spots"]), arr(spec["spreads"])
        m.atms, m.skews = arr(spec["atms"]), arr(spec["skews"])
        m.nDiv = len(spec["div_dates"])
        m.divDates, m.divs = arr(spec["div_dates"]), arr(spec["divs"])
        m.correl = arr(spec["correl"])
        self.c = m


class MProduct:
    """spec kind 'baskets' (assets, weights, maturity, strikes) or 'autocall' (assets, refs,
    maturity, periods, ko, strike, cpn, smooth)."""

    def __init__(self, spec):
        self.spec = spec
        self._keep = []
        p = OrcMProduct()
        p.nA = len(spec["assets"])

        def arr(x):
            a, q = _arr(x)
            self._keep.append(a)
            return q
        if spec["kind"] == "baskets":
            p.kind = 0
            p.weights, p.maturity = arr(spec["weights"]), spec["maturity"]
            p.nK, p.strikes = len(spec["strikes"]), arr(spec["strikes"])
        else:
            p.kind = 1
            p.refs, p.maturity, p.periods = arr(spec["refs"]), spec["maturity"], int(spec["periods"])
            p.ko, p.strike, p.cpn, p.smooth = spec["ko"], spec["strike"], spec["cpn"], spec["smooth"]
        self.c = p


def m_shapes(model, product):
    a, b, c = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    lib().orc_m_shapes(ctypes.byref(model.c), ctypes.byref(product.c), ctypes.byref(a), ctypes.byref(b),
                       ctypes.byref(c))
    return a.value, b.value, c.value


def m_value(model, product, sobol, npath, seed1=12345, seed2=1234):
    npay, _, _ = m_shapes(model, product)
    v, pv = _arr(np.zeros(npay))
    e, pe = _arr(np.zeros(npay))
    assert lib().orc_m_value(ctypes.byref(model.c), ctypes.byref(product.c), int(sobol), int(npath), seed1, seed2,
                             pv, pe) == 0
    return v, e


def m_risk(model, product, sobol, npath, weights, seed1=12345, seed2=1234):
    npay, npar, _ = m_shapes(model, product)
    w, pw = _arr(weights)
    v, pv = _arr(np.zeros(npay))
    r, pr = _arr(np.zeros(npar))
    agg = ctypes.c_double()
    assert lib().orc_m_risk(ctypes.byref(model.c), ctypes.byref(product.c), int(sobol), int(npath), seed1, seed2,
                            pw, pv, ctypes.byref(agg), pr) == 0
    return v, agg.value, r


def m_risk_multi(model, product, sobol, npath, seed1=12345, seed2=1234):
    npay, npar, _ = m_shapes(model, product)
    v, pv = _arr(np.zeros(npay))
    r, pr = _arr(np.zeros(npar * npay))
    assert lib().orc_m_risk_multi(ctypes.byref(model.c), ctypes.byref(product.c), int(sobol), int(npath), seed1,
                                  seed2, pv, pr) == 0
    return v, r.reshape(npar, npay)


def m_init(model, product):
    """(chol, stds, drifts, ffs, alphas, dynamics, numeraires) after the model's init."""
    n = len(model.spec["assets"])
    _, _, dim = m_shapes(model, product)
    ns = dim // n
    nev = 1 if product.spec["kind"] == "baskets" else int(product.spec["periods"])
    out = [np.zeros(n * n), np.zeros(ns * n), np.zeros(ns * n), np.zeros(ns * n), np.zeros(n)]
    ptr = [o.ctypes.data_as(_dp) for o in out]
    dyn = np.zeros(n, dtype=np.int32)
    nums = np.zeros(nev)
    assert lib().orc_m_init(ctypes.byref(model.c), ctypes.byref(product.c), *ptr,
                            dyn.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), nums.ctypes.data_as(_dp)) == 0
    return out[0].reshape(n, n), out[1].reshape(ns, n), out[2].reshape(ns, n), out[3].reshape(ns, n), out[4], dyn, nums
