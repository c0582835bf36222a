"""ctypes binding of libcfgpu.so under the reference's entry-point names (main.h, store.h)."""
import ctypes
import os
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(HERE, "libcfgpu.so")
_dp = ctypes.POINTER(ctypes.c_double)
_lib = None


def library_path():
    return _LIB_PATH


class CfError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"cfgpu error {code}: {msg}")
        self.code = code


class CfNumParam(ctypes.Structure):
    _fields_ = [("parallel", ctypes.c_int), ("useSobol", ctypes.c_int), ("numPath", ctypes.c_int),
                ("seed1", ctypes.c_int), ("seed2", ctypes.c_int), ("precision", ctypes.c_int)]


class CfIvs(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("spot", ctypes.c_double), ("p", ctypes.c_double * 4)]


def lib():
    """Load libcfgpu.so; raises if it has not been built (there is no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            raise CfError(-7, f"{_LIB_PATH} missing: build it with __graft_entry__.build()")
        _lib = ctypes.CDLL(_LIB_PATH)
        _lib.cf_create.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]
    return _lib


def _check(rc):
    if rc != 0:
        buf = ctypes.create_string_buffer(4096)
        lib().cf_last_error(buf, ctypes.c_size_t(4096))
        raise CfError(rc, buf.value.decode(errors="replace"))


def _arr(x, dtype=np.float64):
    a = np.ascontiguousarray(np.asarray(x, dtype=dtype))
    return a


def _p(a):
    return a.ctypes.data_as(_dp)


@dataclass
class NumericalParam:
    """main.h:33-40, plus the precision of the path arithmetic ('fp64' or 'fp32')."""
    parallel: bool = True
    useSobol: bool = False
    numPath: int = 1 << 16
    seed1: int = 12345
    seed2: int = 1234
    precision: str = "fp64"

    def c(self):
        return CfNumParam(int(self.parallel), int(self.useSobol), int(self.numPath), int(self.seed1),
                          int(self.seed2), 1 if self.precision == "fp32" else 0)


class Engine:
    """One context on one GPU: the store plus the entry points of main.h."""

    def __init__(self, device=0):
        h = ctypes.c_void_p()
        _check(lib().cf_create(int(device), ctypes.byref(h)))
        self._h = h
        # labels of stored models and products, dropped when the id is stored again
        self._label_cache = {}

    def close(self):
        if self._h:
            lib().cf_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream_ptr):
        _check(lib().cf_set_stream(self._h, ctypes.c_void_p(stream_ptr)))

    def synchronize(self):
        _check(lib().cf_synchronize(self._h))

    def transfer_stats(self):
        h, d = ctypes.c_uint64(), ctypes.c_uint64()
        _check(lib().cf_transfer_stats(self._h, ctypes.byref(h), ctypes.byref(d)))
        return h.value, d.value

    # ---- store (store.h) ----------------------------------------------------------------
    def putBlackScholes(self, spot, vol, qSpot, rate, div, id):
        _check(lib().cf_put_black_scholes(self._h, ctypes.c_double(spot), ctypes.c_double(vol), int(bool(qSpot)),
                                          ctypes.c_double(rate), ctypes.c_double(div), id.encode()))
        self._label_cache.pop(("m", id), None)
        self._label_cache.pop(("mgrid", id), None)
        return id

    def putDupire(self, spot, spots, times, vols, maxDt, id):
        s, t = _arr(spots), _arr(times)
        v = _arr(vols).reshape(-1)
        if v.size != s.size * t.size:
            raise CfError(-1, "putDupire: vols must be len(spots) x len(times)")
        _check(lib().cf_put_dupire(self._h, ctypes.c_double(spot), _p(s), len(s), _p(t), len(t), _p(v),
                                   ctypes.c_double(maxDt), id.encode()))
        # a Dupire model's parameter labels depend on its spot and time grid only
        grid = (s.tobytes(), t.tobytes())
        if self._label_cache.get(("mgrid", id)) != grid:
            self._label_cache.pop(("m", id), None)
            self._label_cache[("mgrid", id)] = grid
        return id

    def putEuropean(self, strike, exerciseDate, settlementDate=None, id="european"):
        if settlementDate is None:
            settlementDate = exerciseDate
        _check(lib().cf_put_european(self._h, ctypes.c_double(strike), ctypes.c_double(exerciseDate),
                                     ctypes.c_double(settlementDate), id.encode()))
        self._label_cache.pop(("p", id), None)
        return id

    def putBarrier(self, strike, barrier, maturity, monitorFreq, smooth, callPut, id):
        _check(lib().cf_put_barrier(self._h, ctypes.c_double(strike), ctypes.c_double(barrier),
                                    ctypes.c_double(maturity), ctypes.c_double(monitorFreq), ctypes.c_double(smooth),
                                    int(bool(callPut)), id.encode()))
        self._label_cache.pop(("p", id), None)
        return id

    def putContingent(self, coupon, maturity, payFreq, smooth, id):
        """store.h:165-180: the contingent bond of mcPrd.h:404-574."""
        _check(lib().cf_put_contingent(self._h, ctypes.c_double(coupon), ctypes.c_double(maturity),
                                       ctypes.c_double(payFreq), ctypes.c_double(smooth), id.encode()))
        self._label_cache.pop(("p", id), None)

    def putEuropeans(self, maturities, strikes, id):
        m, k = _arr(maturities), _arr(strikes)
        _check(lib().cf_put_europeans(self._h, _p(m), _p(k), len(m), id.encode()))
        self._label_cache.pop(("p", id), None)
        return id

    # ---- multi-asset store (store.h:75-94, 224-255) --------------------------------------
    @staticmethod
    def _names(assets):
        arr = (ctypes.c_char_p * len(assets))(*[a.encode() for a in assets])
        return arr

    def putDisplaced(self, assets, spots, atms, skews, discRate, repoSpreads, divDates, divs, correl, lambda_, id):
        """MultiDisplaced (mcMdlMultiDisplaced.h): divs [len(divDates)][nA], correl [nA][nA] (the lower
        triangle is the model's)."""
        n = len(assets)
        sp, at, sk, rs = _arr(spots), _arr(atms), _arr(skews), _arr(repoSpreads)
        dd = _arr(divDates) if len(divDates) else _arr([0.0])
        dv = _arr(np.asarray(divs, dtype=float).reshape(-1)) if len(divDates) else _arr([0.0])
        co = _arr(np.asarray(correl, dtype=float).reshape(-1))
        if sp.size != n or at.size != n or sk.size != n or rs.size != n or co.size != n * n or \
                (len(divDates) and dv.size != n * len(divDates)):
            raise CfError(-1, "putDisplaced: inconsistent dimensions")
        _check(lib().cf_put_displaced(self._h, n, self._names(assets), _p(sp), _p(at), _p(sk),
                                      ctypes.c_double(discRate), _p(rs), len(divDates), _p(dd), _p(dv), _p(co),
                                      ctypes.c_double(lambda_), id.encode()))
        self._label_cache.pop(("m", id), None)
        self._label_cache.pop(("mgrid", id), None)
        return id

    def putBaskets(self, assets, weights, maturity, strikes, id):
        w, k = _arr(weights), _arr(strikes)
        if w.size != len(assets):
            raise CfError(-1, "putBaskets: one weight per asset")
        _check(lib().cf_put_baskets(self._h, len(assets), self._names(assets), _p(w), ctypes.c_double(maturity),
                                    len(k), _p(k), id.encode()))
        self._label_cache.pop(("p", id), None)
        return id

    def putAutocall(self, assets, refs, maturity, periods, ko, strike, cpn, smooth, id):
        r = _arr(refs)
        if r.size != len(assets):
            raise CfError(-1, "putAutocall: one reference per asset")
        _check(lib().cf_put_autocall(self._h, len(assets), self._names(assets), _p(r), ctypes.c_double(maturity),
                                     int(periods), ctypes.c_double(ko), ctypes.c_double(strike),
                                     ctypes.c_double(cpn), ctypes.c_double(smooth), id.encode()))
        self._label_cache.pop(("p", id), None)
        return id

    def mdState(self, modelId, productId):
        """Initialised multi-asset model: dict(s0, chol, stds, drifts, ffs, alphas, numeraires, dynamics)."""
        cnt = ctypes.c_int()
        _check(lib().cf_md_state(self._h, modelId.encode(), productId.encode(), None, 0, ctypes.byref(cnt), None))
        npay, npar, dim = self.shapes(modelId, productId)
        d = np.zeros(cnt.value)
        # the asset count: the model's "spot <asset>" parameters
        nA = sum(1 for l in self.parameterLabels(modelId) if l.startswith("spot "))
        dyn = np.zeros(nA, dtype=np.int32)
        _check(lib().cf_md_state(self._h, modelId.encode(), productId.encode(), _p(d), cnt.value, ctypes.byref(cnt),
                                 dyn.ctypes.data_as(ctypes.POINTER(ctypes.c_int))))
        ns = dim // nA
        o = [0, nA, nA + nA * nA, nA + nA * nA + ns * nA, nA + nA * nA + 2 * ns * nA, nA + nA * nA + 3 * ns * nA,
             2 * nA + nA * nA + 3 * ns * nA]
        return dict(s0=d[o[0]:o[1]], chol=d[o[1]:o[2]].reshape(nA, nA), stds=d[o[2]:o[3]].reshape(ns, nA),
                    drifts=d[o[3]:o[4]].reshape(ns, nA), ffs=d[o[4]:o[5]].reshape(ns, nA), alphas=d[o[5]:o[6]],
                    numeraires=d[o[6]:], dynamics=dyn)

    def _labels(self, fn, key, kind):
        got = self._label_cache.get((kind, key))
        if got is None:
            got = self._label_cache[(kind, key)] = self._fetch_labels(fn, key)
        return list(got)

    def _fetch_labels(self, fn, key):
        n, need = ctypes.c_int(), ctypes.c_size_t()
        _check(fn(self._h, key.encode(), None, ctypes.c_size_t(0), ctypes.byref(n), ctypes.byref(need)))
        buf = ctypes.create_string_buffer(need.value)
        _check(fn(self._h, key.encode(), buf, need, ctypes.byref(n), ctypes.byref(need)))
        s = buf.value.decode()
        return s.split("\n") if s else []

    def payoffLabels(self, productId):
        return self._labels(lib().cf_payoff_labels, productId, "p")

    def parameterLabels(self, modelId):
        return self._labels(lib().cf_parameter_labels, modelId, "m")

    def shapes(self, modelId, productId):
        a, b, c = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        _check(lib().cf_shapes(self._h, modelId.encode(), productId.encode(), ctypes.byref(a), ctypes.byref(b),
                               ctypes.byref(c)))
        return a.value, b.value, c.value

    # ---- entry points (main.h) -----------------------------------------------------------
    def value(self, modelId, productId, num):
        npay, _, _ = self.shapes(modelId, productId)
        v, e = np.zeros(npay), np.zeros(npay)
        nc = num.c()
        _check(lib().cf_value(self._h, modelId.encode(), productId.encode(), ctypes.byref(nc), _p(v), _p(e)))
        return dict(identifiers=self.payoffLabels(productId), values=v, stderrs=e)

    def simulatePaths(self, modelId, productId, num):
        """mcSimul (mcBase.h:267-308): every path's payoffs, [numPath][nPay]."""
        npay, _, _ = self.shapes(modelId, productId)
        out = np.zeros(num.numPath * npay)
        nc = num.c()
        _check(lib().cf_simulate_paths(self._h, modelId.encode(), productId.encode(), ctypes.byref(nc), _p(out)))
        return out.reshape(num.numPath, npay)

    def AADriskOne(self, modelId, productId, num, riskPayoff=""):
        npay, npar, _ = self.shapes(modelId, productId)
        v, r = np.zeros(npay), np.zeros(npar)
        rv = ctypes.c_double()
        nc = num.c()
        _check(lib().cf_aad_risk_one(self._h, modelId.encode(), productId.encode(), ctypes.byref(nc),
                                     riskPayoff.encode(), _p(v), ctypes.byref(rv), _p(r)))
        return dict(payoffIds=self.payoffLabels(productId), payoffValues=v, riskPayoffValue=rv.value,
                    paramIds=self.parameterLabels(modelId), risks=r)

    def AADriskAggregate(self, modelId, productId, notionals, num):
        npay, npar, _ = self.shapes(modelId, productId)
        labels = self.payoffLabels(productId)
        w = np.zeros(npay)
        if isinstance(notionals, dict):
            for lab, x in notionals.items():
                if lab not in labels:
                    raise CfError(-2, "AADriskAggregate() : payoff not found")
                w[labels.index(lab)] = x
        else:
            w[:] = notionals
        v, r = np.zeros(npay), np.zeros(npar)
        agg = ctypes.c_double()
        nc = num.c()
        _check(lib().cf_aad_risk_aggregate(self._h, modelId.encode(), productId.encode(), _p(w), ctypes.byref(nc),
                                           _p(v), ctypes.byref(agg), _p(r)))
        return dict(payoffIds=labels, payoffValues=v, riskPayoffValue=agg.value,
                    paramIds=self.parameterLabels(modelId), risks=r)

    def modelGrid(self, modelId):
        """(spots, times) of a Dupire model; raises for other models (cf_model_grid)."""
        ns, nt = ctypes.c_int(), ctypes.c_int()
        _check(lib().cf_model_grid(self._h, modelId.encode(), ctypes.byref(ns), ctypes.byref(nt), None, None))
        spots, times = np.zeros(ns.value), np.zeros(nt.value)
        _check(lib().cf_model_grid(self._h, modelId.encode(), ctypes.byref(ns), ctypes.byref(nt), _p(spots),
                                   _p(times)))
        return spots, times

    def dupireAADRisk(self, modelId, productId, notionals, num):
        """main.h:364-411: value, delta and the vega matrix [spots][times] of the aggregate."""
        spots, times = self.modelGrid(modelId)
        r = self.AADriskAggregate(modelId, productId, notionals, num)
        return dict(value=r["riskPayoffValue"], delta=r["risks"][0],
                    vega=np.asarray(r["risks"][1:]).reshape(len(spots), len(times)))

    BUMP_METHODS = {"auto": 0, "reprice": 1, "pathwise": 2}

    def bumpRisk(self, modelId, productId, num, method="auto"):
        """main.h:316-359: risks[nParam][nPay] by one-sided 1e-8 bumps, repriced on the same
        random numbers in FP64 ('reprice' revalues each bumped model; 'pathwise' re-simulates
        only the paths each bumped local-vol node touches)."""
        npay, npar, _ = self.shapes(modelId, productId)
        v, r = np.zeros(npay), np.zeros(npar * npay)
        nc = num.c()
        _check(lib().cf_bump_risk(self._h, modelId.encode(), productId.encode(), ctypes.byref(nc),
                                  int(self.BUMP_METHODS[method]), _p(v), _p(r)))
        return dict(payoffs=self.payoffLabels(productId), params=self.parameterLabels(modelId), values=v,
                    risks=r.reshape(npar, npay))

    def AADriskMulti(self, modelId, productId, num):
        npay, npar, _ = self.shapes(modelId, productId)
        v, r = np.empty(npay), np.empty(npar * npay)  # every entry is written
        nc = num.c()
        _check(lib().cf_aad_risk_multi(self._h, modelId.encode(), productId.encode(), ctypes.byref(nc), _p(v),
                                       _p(r)))
        return dict(payoffs=self.payoffLabels(productId), params=self.parameterLabels(modelId), values=v,
                    risks=r.reshape(npar, npay))

    @staticmethod
    def ivs(kind, spot, params):
        s = CfIvs()
        s.kind = 0 if kind in ("param", 0) else 1
        s.spot = spot
        for i, x in enumerate(params):
            s.p[i] = x
        return s

    def dupireCalib(self, ivs, inclSpots, maxDs, inclTimes, maxDtVol, riskView=None):
        """riskView = (strikes, mats, spreads[nK][nM]) shifts the implied vols (bump harness)."""
        if riskView is not None:
            a, b = _arr(inclSpots), _arr(inclTimes)
            k, m, sp = _arr(riskView[0]), _arr(riskView[1]), _arr(riskView[2]).reshape(-1)
            nS, nT = ctypes.c_int(), ctypes.c_int()
            _check(lib().cf_dupire_calib(self._h, ctypes.byref(ivs), _p(a), len(a), ctypes.c_double(maxDs), _p(b),
                                         len(b), ctypes.c_double(maxDtVol), ctypes.byref(nS), ctypes.byref(nT), None,
                                         None, None))
            s, t, lv = np.zeros(nS.value), np.zeros(nT.value), np.zeros(nS.value * nT.value)
            _check(lib().cf_dupire_calib_view(self._h, ctypes.byref(ivs), _p(a), len(a), ctypes.c_double(maxDs), _p(b),
                                              len(b), ctypes.c_double(maxDtVol), _p(k), len(k), _p(m), len(m), _p(sp),
                                              ctypes.byref(nS), ctypes.byref(nT), _p(s), _p(t), _p(lv)))
            return dict(spots=s, times=t, lVols=lv.reshape(nS.value, nT.value))
        a, b = _arr(inclSpots), _arr(inclTimes)
        nS, nT = ctypes.c_int(), ctypes.c_int()
        _check(lib().cf_dupire_calib(self._h, ctypes.byref(ivs), _p(a), len(a), ctypes.c_double(maxDs), _p(b), len(b),
                                     ctypes.c_double(maxDtVol), ctypes.byref(nS), ctypes.byref(nT), None, None, None))
        s, t, lv = np.zeros(nS.value), np.zeros(nT.value), np.zeros(nS.value * nT.value)
        _check(lib().cf_dupire_calib(self._h, ctypes.byref(ivs), _p(a), len(a), ctypes.c_double(maxDs), _p(b), len(b),
                                     ctypes.c_double(maxDtVol), ctypes.byref(nS), ctypes.byref(nT), _p(s), _p(t),
                                     _p(lv)))
        return dict(spots=s, times=t, lVols=lv.reshape(nS.value, nT.value))

    def dupireSuperbucket(self, ivs, spot, maxDt, productId, notionals, inclSpots, maxDs, inclTimes, maxDtVol,
                          strikes, mats, num, refSeeding=False):
        npay = len(self.payoffLabels(productId))
        labels = self.payoffLabels(productId)
        w = np.zeros(npay)
        if isinstance(notionals, dict):
            for lab, x in notionals.items():
                w[labels.index(lab)] = x
        else:
            w[:] = notionals
        a, b = _arr(inclSpots), _arr(inclTimes)
        k, m = _arr(strikes), _arr(mats)
        nS, nT = ctypes.c_int(), ctypes.c_int()
        _check(lib().cf_dupire_calib(self._h, ctypes.byref(ivs), _p(a), len(a), ctypes.c_double(maxDs), _p(b), len(b),
                                     ctypes.c_double(maxDtVol), ctypes.byref(nS), ctypes.byref(nT), None, None, None))
        vega = np.zeros(len(k) * len(m))
        micro = np.zeros(nS.value * nT.value)
        val, dl = ctypes.c_double(), ctypes.c_double()
        nc = num.c()
        _check(lib().cf_dupire_superbucket(self._h, ctypes.byref(ivs), ctypes.c_double(spot), ctypes.c_double(maxDt),
                                           productId.encode(), _p(w), _p(a), len(a), ctypes.c_double(maxDs), _p(b),
                                           len(b), ctypes.c_double(maxDtVol), _p(k), len(k), _p(m), len(m),
                                           ctypes.byref(nc), int(bool(refSeeding)), ctypes.byref(val),
                                           ctypes.byref(dl), _p(vega), _p(micro)))
        return dict(value=val.value, delta=dl.value, strikes=k, mats=m, vega=vega.reshape(len(k), len(m)),
                    microbucket=micro.reshape(nS.value, nT.value))

    def calibAdjoint(self, ivs, inclSpots, maxDs, inclTimes, maxDtVol, strikes, mats, micro, refSeeding=False):
        """The calibration's adjoint alone (test hook): local-vol adjoints micro[nS][nT] -> vega
        [strike][mat] of the risk view; with, per node and point ([nT][nS][5] each), the forward's
        call prices and their derivatives to the implied vol that it was taken at, and the adjoint
        of each point's implied vol."""
        a, b = _arr(inclSpots), _arr(inclTimes)
        k, m = _arr(strikes), _arr(mats)
        nS, nT = ctypes.c_int(), ctypes.c_int()
        _check(lib().cf_dupire_calib(self._h, ctypes.byref(ivs), _p(a), len(a), ctypes.c_double(maxDs), _p(b), len(b),
                                     ctypes.c_double(maxDtVol), ctypes.byref(nS), ctypes.byref(nT), None, None, None))
        mb = _arr(micro).reshape(-1)
        if mb.size != nS.value * nT.value:
            raise CfError(-1, "calibAdjoint: micro must hold nS x nT local-vol adjoints")
        vega = np.zeros(len(k) * len(m))
        calls = np.zeros(nT.value * nS.value * 5)
        cvegas = np.zeros(nT.value * nS.value * 5)
        padj = np.zeros(nT.value * nS.value * 5)
        _check(lib().cf_calib_adjoint(self._h, ctypes.byref(ivs), _p(a), len(a), ctypes.c_double(maxDs), _p(b), len(b),
                                      ctypes.c_double(maxDtVol), _p(k), len(k), _p(m), len(m), _p(mb),
                                      int(bool(refSeeding)), _p(vega), _p(calls), _p(cvegas), _p(padj)))
        shape = (nT.value, nS.value, 5)
        return dict(vega=vega.reshape(len(k), len(m)), calls=calls.reshape(shape), callVegas=cvegas.reshape(shape),
                    pointAdj=padj.reshape(shape))

    # ---- RNG access --------------------------------------------------------------------------
    def dupireSuperbucketBump(self, ivs, spot, maxDt, productId, notionals, inclSpots, maxDs, inclTimes, maxDtVol,
                              strikes, mats, num, vegaBump=0.0):
        """main.h:575-696: value, delta (spot +1e-8) and vega[strike][mat] (each risk-view implied
        vol +vegaBump, the reference's 1e-5 when 0, recalibrated and repriced), FP64 valuations on
        the same random numbers."""
        labels = self.payoffLabels(productId)
        w = np.zeros(len(labels))
        if isinstance(notionals, dict):
            for lab, x in notionals.items():
                if lab not in labels:
                    raise CfError(-2, "dupireSuperbucketBump() : payoff not found")
                w[labels.index(lab)] = x
        else:
            w[:] = notionals
        a, b = _arr(inclSpots), _arr(inclTimes)
        k, m = _arr(strikes), _arr(mats)
        vega = np.zeros(len(k) * len(m))
        val, dl = ctypes.c_double(), ctypes.c_double()
        nc = num.c()
        _check(lib().cf_dupire_superbucket_bump(self._h, ctypes.byref(ivs), ctypes.c_double(spot),
                                                ctypes.c_double(maxDt), productId.encode(), _p(w), _p(a), len(a),
                                                ctypes.c_double(maxDs), _p(b), len(b), ctypes.c_double(maxDtVol), _p(k),
                                                len(k), _p(m), len(m), ctypes.byref(nc), ctypes.c_double(vegaBump),
                                                ctypes.byref(val), ctypes.byref(dl), _p(vega)))
        return dict(value=val.value, delta=dl.value, strikes=k, mats=m, vega=vega.reshape(len(k), len(m)))

    def sobolPoints(self, dim, firstPath, nPaths):
        out = np.zeros(nPaths * dim, dtype=np.uint32)
        _check(lib().cf_sobol_points(self._h, int(dim), ctypes.c_int64(firstPath), int(nPaths),
                                     out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))))
        return out.reshape(nPaths, dim)

    def mrgState(self, seed1, seed2, dim, firstPath):
        out = np.zeros(6, dtype=np.uint32)
        _check(lib().cf_mrg_state(self._h, ctypes.c_uint(seed1), ctypes.c_uint(seed2), int(dim),
                                  ctypes.c_int64(firstPath), out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))))
        return out

    def gaussians(self, useSobol, seed1, seed2, dim, firstPath, nPaths):
        out = np.zeros(nPaths * dim)
        _check(lib().cf_gaussians(self._h, int(bool(useSobol)), ctypes.c_uint(seed1), ctypes.c_uint(seed2), int(dim),
                                  ctypes.c_int64(firstPath), int(nPaths), _p(out)))
        return out.reshape(nPaths, dim)

    # ---- device-resident launches ------------------------------------------------------------
    def enqueue(self, modelId, productId, num, risk=True, weights=None):
        w = None if weights is None else _arr(weights)
        n = ctypes.c_int()
        nc = num.c()
        _check(lib().cf_enqueue(self._h, modelId.encode(), productId.encode(), ctypes.byref(nc), int(bool(risk)),
                                None if w is None else _p(w), ctypes.byref(n)))
        return n.value

    def enqueue_shard(self, modelId, productId, num, firstPath, risk=True, weights=None):
        """cf_enqueue_shard: paths [firstPath, firstPath + num.numPath) of the run's sequence."""
        w = None if weights is None else _arr(weights)
        n = ctypes.c_int()
        nc = num.c()
        _check(lib().cf_enqueue_shard(self._h, modelId.encode(), productId.encode(), ctypes.byref(nc),
                                      ctypes.c_int64(int(firstPath)), int(bool(risk)), None if w is None else _p(w),
                                      ctypes.byref(n)))
        return n.value

    def fetch_raw(self):
        """The exact accumulators of the last enqueue (int64 words, hi/lo pairs)."""
        nw = ctypes.c_int()
        _check(lib().cf_fetch_raw(self._h, None, 0, ctypes.byref(nw)))
        acc = np.zeros(nw.value, dtype=np.int64)
        _check(lib().cf_fetch_raw(self._h, acc.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), nw.value,
                                  ctypes.byref(nw)))
        return acc

    def fetch(self, npay, nparam=0):
        v, e, r = np.zeros(npay), np.zeros(npay), np.zeros(max(nparam, 1))
        agg = ctypes.c_double()
        _check(lib().cf_fetch_result(self._h, _p(v), _p(e), ctypes.byref(agg), _p(r) if nparam else None))
        return v, e, agg.value, r[:nparam]


def results_from_raw(acc, nRisk, nPay, nPath):
    """cf_results_from_raw: (values, stderrs, aggregate, risks) of summed shard accumulators."""
    acc = np.ascontiguousarray(acc, dtype=np.int64)
    v, e, r = np.zeros(nPay), np.zeros(nPay), np.zeros(max(nRisk, 1))
    agg = ctypes.c_double()
    _check(lib().cf_results_from_raw(acc.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), int(nRisk), int(nPay),
                                     ctypes.c_int64(int(nPath)), _p(v), _p(e), ctypes.byref(agg), _p(r)))
    return v, e, agg.value, r[:nRisk]


class CfRequest(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("modelId", ctypes.c_char_p), ("productId", ctypes.c_char_p),
                ("num", CfNumParam), ("weights", _dp), ("nWeights", ctypes.c_int),
                ("queueTimeoutMs", ctypes.c_double)]


class CfServingStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_uint64), ("completed", ctypes.c_uint64), ("failed", ctypes.c_uint64),
                ("rejected", ctypes.c_uint64), ("cancelled", ctypes.c_uint64), ("timedOut", ctypes.c_uint64),
                ("p50Ms", ctypes.c_double), ("p99Ms", ctypes.c_double), ("meanMs", ctypes.c_double),
                ("pathStepsDone", ctypes.c_uint64), ("maxInFlight", ctypes.c_int),
                ("peakFootprint", ctypes.c_uint64), ("maxStartMs", ctypes.c_double), ("maxStepMs", ctypes.c_double),
                ("bufferGrowths", ctypes.c_uint64)]


STATUS = {0: "queued", 1: "running", 2: "done", 3: "failed", 4: "rejected", 5: "cancelled", 6: "timeout"}
KINDS = {"value": 0, "risk": 1, "multi": 2}


class Server:
    """Continuous-batching server over an Engine: `slots` concurrent CUDA streams, admission
    by device-memory footprint (hbm_budget bytes)."""

    def __init__(self, engine, slots=8, hbm_budget=64 << 30):
        self.eng = engine
        h = ctypes.c_void_p()
        _check(lib().cf_server_create(engine._h, int(slots), ctypes.c_uint64(hbm_budget), ctypes.byref(h)))
        self._h = h
        self._shape = {}

    def configure(self, short_slots, long_threshold, chunk_path_steps=0.0, long_blocks_per_sm=0):
        """cf_server_configure: short requests on short_slots high-priority slots, risks above
        long_threshold path-steps on the others, launched in chunks of chunk_path_steps with at
        most long_blocks_per_sm resident blocks per SM."""
        _check(lib().cf_server_configure(self._h, int(short_slots), ctypes.c_double(long_threshold),
                                         ctypes.c_double(chunk_path_steps), int(long_blocks_per_sm)))

    def close(self):
        if self._h:
            lib().cf_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, kind, modelId, productId, num, weights=None, queue_timeout_ms=0.0):
        w = None if weights is None else _arr(weights)
        r = CfRequest(KINDS[kind], modelId.encode(), productId.encode(), num.c(), None if w is None else _p(w),
                      0 if w is None else len(w), float(queue_timeout_ms))
        rid = ctypes.c_uint64()
        _check(lib().cf_server_submit(self._h, ctypes.byref(r), ctypes.byref(rid)))
        self._shape[rid.value] = (kind, modelId, productId)
        return rid.value

    def cancel(self, rid):
        _check(lib().cf_server_cancel(self._h, ctypes.c_uint64(rid)))

    def order(self, lane, order, aging_ms=0.0):
        """cf_server_order: admission order of a lane (0 arrival order, 1 least work first, with
        requests older than aging_ms first)."""
        _check(lib().cf_server_order(self._h, int(lane), int(order), ctypes.c_double(aging_ms)))

    def wait(self, rid, timeout_ms=-1):
        st = ctypes.c_int()
        _check(lib().cf_server_wait(self._h, ctypes.c_uint64(rid), int(timeout_ms), ctypes.byref(st)))
        return STATUS[st.value]

    def error(self):
        buf = ctypes.create_string_buffer(4096)
        lib().cf_last_error(buf, ctypes.c_size_t(4096))
        return buf.value.decode(errors="replace")

    def result(self, rid):
        kind, mid, pid = self._shape[rid]
        npay, npar, _ = self.eng.shapes(mid, pid)
        v, e = np.zeros(npay), np.zeros(npay)
        r = np.zeros(max(1, npar * (npay if kind == "multi" else 1)))
        agg, lat = ctypes.c_double(), ctypes.c_double()
        _check(lib().cf_server_result(self._h, ctypes.c_uint64(rid), _p(v), _p(e), ctypes.byref(agg),
                                      _p(r) if kind != "value" else None, ctypes.byref(lat)))
        out = dict(values=v, stderrs=e, aggregate=agg.value, latency_ms=lat.value)
        if kind == "risk":
            out["risks"] = r[:npar]
        elif kind == "multi":
            out["risks"] = r.reshape(npar, npay)
        return out

    def release(self, rid):
        _check(lib().cf_server_release(self._h, ctypes.c_uint64(rid)))
        self._shape.pop(rid, None)

    def stats(self):
        s = CfServingStats()
        _check(lib().cf_server_stats(self._h, ctypes.byref(s)))
        return {k: getattr(s, k) for k, _ in CfServingStats._fields_}

    def reset_stats(self):
        """Starts the statistics afresh; the slots keep their streams and device buffers."""
        _check(lib().cf_server_reset_stats(self._h))

    def inject_failures(self, n):
        _check(lib().cf_server_inject_failures(self._h, int(n)))
