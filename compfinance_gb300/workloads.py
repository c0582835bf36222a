"""Synthetic inputs of the Dupire / Black-Scholes Monte Carlo workloads.

No market data is involved: every surface is built from a closed formula plus seeded noise
so that the golden fixtures, the parity tests and the benchmark all see the same numbers.

* ``dupire_surface``  local-vol grid sigma(S,t) = max(0.05, 0.15 + 0.10 e^{-t} ln^2(S/100) + 0.005 z)
  on nS log-spaced spots over [50, 200] and nT evenly spaced times over [0.1, 3.0]; z are
  standard normals drawn from a splitmix64 counter stream (Box-Muller), so the grid depends
  only on (nS, nT, seed).
* ``uoc_barrier``     the up-and-out call of the reference's barrier workload (K=120, B=150,
  T=3y, weekly monitoring, 1% smoothing).
* ``superbucket_*``   the implied-vol surface iv(K,T) = 0.18 + 0.08 ln^2(K/100)/sqrt(T) - 0.02 ln(K/100),
  its 30x12 risk view and the 10x20 European portfolio.
"""
import math

import numpy as np

_MASK = (1 << 64) - 1


def _splitmix64(x):
    x = (x + 0x9E3779B97F4A7C15) & _MASK
    z = x
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & _MASK
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & _MASK
    return z ^ (z >> 31)


def seeded_normals(n, seed):
    """n standard normals from a counter-based splitmix64 stream (Box-Muller)."""
    out = np.empty(n)
    for i in range(0, n, 2):
        a = _splitmix64(seed * 1000003 + i)
        b = _splitmix64(seed * 1000003 + i + 1)
        u1 = ((a >> 11) + 1) * (1.0 / 9007199254740993.0)
        u2 = (b >> 11) * (1.0 / 9007199254740992.0)
        r = math.sqrt(-2.0 * math.log(u1))
        out[i] = r * math.cos(2.0 * math.pi * u2)
        if i + 1 < n:
            out[i + 1] = r * math.sin(2.0 * math.pi * u2)
    return out


def dupire_surface(nS=60, nT=30, seed=20181, noise=0.005):
    """(spots[nS], times[nT], vols[nS][nT]) of the synthetic local-vol surface, spot-major."""
    spots = np.array([50.0 * 4.0 ** (i / (nS - 1)) for i in range(nS)])
    times = np.array([0.1 + 2.9 * j / (nT - 1) for j in range(nT)])
    z = seeded_normals(nS * nT, seed).reshape(nS, nT)
    vols = np.empty((nS, nT))
    for i in range(nS):
        l2 = math.log(spots[i] / 100.0) ** 2
        for j in range(nT):
            vols[i, j] = max(0.05, 0.15 + 0.10 * math.exp(-times[j]) * l2 + noise * z[i, j])
    return spots, times, vols


# Barrier product of the Dupire workload: strike 120, barrier 150, 3y, weekly monitoring.
UOC_BARRIER = dict(strike=120.0, barrier=150.0, maturity=3.0, monitor_freq=3.0 / 156.0,
                   smooth=0.01, callput=0)
DUPIRE_SPOT = 100.0
DUPIRE_MAXDT = 0.25          # no refinement of the weekly product timeline: 156 steps
MRG_SEEDS = (12345, 1234)    # NumericalParam defaults of the reference

# Black-Scholes European workload.
BS_EUROPEAN = dict(spot=100.0, vol=0.20, rate=0.02, div=0.0, strike=100.0, maturity=1.0)

# Superbucket workload.
SB_IVS = dict(a=0.18, b=0.08, c=-0.02, sref=100.0)


def superbucket_grid(nS=60, nT=30):
    incl_spots = [50.0 * 4.0 ** (i / (nS - 1)) for i in range(nS)]
    incl_times = [0.1 + 2.9 * j / (nT - 1) for j in range(nT)]
    return incl_spots, 1000.0, incl_times, 3.0   # maxDs, maxDtVol: no refinement


def superbucket_riskview(nK=30, nM=12):
    strikes = [50.0 + 150.0 * i / (nK - 1) for i in range(nK)]
    mats = [0.25 + 2.75 * j / (nM - 1) for j in range(nM)]
    return strikes, mats


def superbucket_portfolio(nM=10, nK=20):
    """Europeans portfolio as the reference's putEuropeans wants it: parallel lists."""
    mats, strikes = [], []
    for j in range(nM):
        t = 0.3 + 2.7 * j / (nM - 1)
        for i in range(nK):
            mats.append(t)
            strikes.append(70.0 + 90.0 * i / (nK - 1))
    return mats, strikes


# ---------------------------------------------------------------------------------------
# Mixed serving stream: 40% Black-Scholes European values (2^14 Sobol paths), 40% Dupire
# barrier full risk (paths log-uniform 2^16..2^20, grid 20x10 / 60x30 / 120x60, 12 / 52 /
# 156 / 520 steps), 20% Dupire European-portfolio AADriskMulti (50-200 payoffs, 36 monthly
# steps, 2^16 Sobol paths).  Spot 80-120, strike 0.8-1.2 x spot, barrier 1.2-1.6 x spot
# (drawn from small sets so that models and products are stored once and reused).
# ---------------------------------------------------------------------------------------
SERVE_SPOTS = (80.0, 90.0, 100.0, 110.0, 120.0)
SERVE_KR = (0.8, 0.9, 1.0, 1.1, 1.2)
SERVE_KR_BARRIER = (0.9, 1.0, 1.1)
SERVE_BR = (1.2, 1.4, 1.6)
SERVE_GRIDS = ((20, 10), (60, 30), (120, 60))
SERVE_STEPS = (12, 52, 156, 520)
SERVE_NPAY = (50, 100, 150, 200)


def serving_store():
    """(models, products): id -> spec, everything the stream refers to."""
    models, products = {}, {}
    surf = {g: dupire_surface(*g) for g in SERVE_GRIDS}
    for s0 in SERVE_SPOTS:
        models[f"bs{s0:g}"] = dict(kind="bs", spot=s0, vol=0.2, rate=0.02, div=0.0, qspot=0)
        for g in SERVE_GRIDS:
            sp, tm, vv = surf[g]
            for tag, mdt in (("w", 0.25), ("m", 1.0 / 12.0)):
                models[f"dup{s0:g}_{g[0]}x{g[1]}{tag}"] = dict(kind="dupire", spot=s0, spots=sp, times=tm, vols=vv,
                                                              maxdt=mdt)
        for kr in SERVE_KR:
            products[f"eu{s0:g}_{kr:g}"] = dict(kind="european", strike=kr * s0, exercise=1.0, settlement=1.0)
        for kr in SERVE_KR_BARRIER:
            for br in SERVE_BR:
                for st in SERVE_STEPS:
                    products[f"uoc{s0:g}_{kr:g}_{br:g}_{st}"] = dict(kind="uoc", strike=kr * s0, barrier=br * s0,
                                                                      maturity=3.0, freq=3.0 / st, smooth=0.01,
                                                                      callput=0)
        for npay in SERVE_NPAY:
            nk = npay // 10
            mats, strikes = [], []
            for j in range(10):
                for i in range(nk):
                    mats.append(0.3 + 0.3 * j)
                    strikes.append(s0 * (0.8 + 0.4 * i / max(1, nk - 1)))
            products[f"port{s0:g}_{npay}"] = dict(kind="europeans", mats=mats, strikes=strikes)
    return models, products


def serving_stream(n=10000, rate=2000.0, seed=2026):
    """Seeded Poisson arrivals: list of dicts (t, kind, model, product, paths, sobol)."""
    rs = np.random.RandomState(seed)
    t = np.cumsum(rs.exponential(1.0 / rate, n))
    out = []
    for i in range(n):
        u = rs.uniform()
        s0 = SERVE_SPOTS[rs.randint(len(SERVE_SPOTS))]
        if u < 0.4:
            kr = SERVE_KR[rs.randint(len(SERVE_KR))]
            out.append(dict(t=t[i], kind="value", model=f"bs{s0:g}", product=f"eu{s0:g}_{kr:g}", paths=1 << 14,
                            sobol=True))
        elif u < 0.8:
            g = SERVE_GRIDS[rs.randint(3)]
            st = SERVE_STEPS[rs.randint(4)]
            kr = SERVE_KR_BARRIER[rs.randint(3)]
            br = SERVE_BR[rs.randint(3)]
            paths = int(round(2.0 ** rs.uniform(16, 20) / 256)) * 256
            out.append(dict(t=t[i], kind="risk", model=f"dup{s0:g}_{g[0]}x{g[1]}w",
                            product=f"uoc{s0:g}_{kr:g}_{br:g}_{st}", paths=paths, sobol=False))
        else:
            g = SERVE_GRIDS[rs.randint(3)]
            npay = SERVE_NPAY[rs.randint(4)]
            out.append(dict(t=t[i], kind="multi", model=f"dup{s0:g}_{g[0]}x{g[1]}m", product=f"port{s0:g}_{npay}",
                            paths=1 << 16, sobol=True))
    return out


# ---------------------------------------------------------------------------------------
# Portfolio risk run (AADriskMulti of the superbucket portfolio on a synthetic Dupire surface)
# for timing and profiling (bench.py --case multi)
# ---------------------------------------------------------------------------------------
def run_multi(grid=(60, 30), paths=1 << 20, reps=1, precision="fp32", device=0):
    """Times `reps` AADriskMulti calls (200 payoffs x (1 + nS nT) parameters, 36 monthly steps,
    Sobol paths) after one warm-up call; returns seconds per call."""
    import time
    from compfinance_gb300 import Engine, NumericalParam
    eng = Engine(device)
    mats, strikes = superbucket_portfolio(10, 20)
    eng.putEuropeans(mats, strikes, "port")
    s, t, v = dupire_surface(*grid)
    eng.putDupire(100.0, s, t, v, 1.0 / 12.0, "dup")
    num = NumericalParam(useSobol=True, numPath=int(paths), precision=precision)
    eng.AADriskMulti("dup", "port", num)
    t0 = time.perf_counter()
    for _ in range(reps):
        eng.AADriskMulti("dup", "port", num)
    dt = (time.perf_counter() - t0) / max(1, reps)
    eng.close()
    return dt


def run_superbucket(paths=1 << 20, reps=1, precision="fp32", device=0):
    """Times `reps` dupireSuperbucket calls of the portfolio (parametric implied surface calibrated
    to 60x30 local vols, 200 Europeans, 36 monthly steps, Sobol paths, 30x12 risk view) after one
    warm-up call; returns seconds per call."""
    import time
    from compfinance_gb300 import Engine, NumericalParam
    eng = Engine(device)
    iv = Engine.ivs("param", 100.0, [SB_IVS["a"], SB_IVS["b"], SB_IVS["c"], SB_IVS["sref"]])
    isp, mds, itm, mdt = superbucket_grid(60, 30)
    rk, rm = superbucket_riskview(30, 12)
    mats, strikes = superbucket_portfolio(10, 20)
    eng.putEuropeans(mats, strikes, "port")
    num = NumericalParam(useSobol=True, numPath=int(paths), precision=precision)
    w = [1.0] * len(mats)
    eng.dupireSuperbucket(iv, 100.0, 1.0 / 12.0, "port", w, isp, mds, itm, mdt, rk, rm, num)
    t0 = time.perf_counter()
    for _ in range(reps):
        eng.dupireSuperbucket(iv, 100.0, 1.0 / 12.0, "port", w, isp, mds, itm, mdt, rk, rm, num)
    dt = (time.perf_counter() - t0) / max(1, reps)
    eng.close()
    return dt


# ---------------------------------------------------------------------------------------
# Multi-asset workload (mcMdlMultiDisplaced.h, mcPrdMulti.h): four correlated assets, one per
# dynamics of the displacement rule (lognormal, surnormal, subnormal, normal), with dividends;
# a 6-period autocall and a 5-strike basket on them.
# ---------------------------------------------------------------------------------------
MD4 = dict(assets=["A", "B", "C", "D"], spots=[100.0, 50.0, 80.0, 120.0], atms=[0.2, 0.25, 0.15, 0.2],
           skews=[0.0, -0.05, -0.1, -0.1], disc=0.03, spreads=[0.01, 0.0, 0.02, -0.01], div_dates=[0.4, 1.2, 2.5],
           divs=[[0.02, 0.0, 0.01, 0.03], [0.01, 0.02, 0.0, 0.0], [0.02, 0.01, 0.01, 0.01]],
           correl=[[1.0, 0.5, 0.3, 0.2], [0.5, 1.0, 0.4, 0.1], [0.3, 0.4, 1.0, 0.25], [0.2, 0.1, 0.25, 1.0]],
           lam=0.1)
MD4_AUTOCALL = dict(refs=[100.0, 50.0, 80.0, 120.0], maturity=3.0, periods=6, ko=1.0, strike=0.7, cpn=0.06,
                    smooth=0.05)
MD4_BASKET = dict(weights=[0.25, 0.3, 0.2, 0.25], maturity=2.0, strikes=[70.0, 80.0, 86.0, 95.0, 105.0])


def put_md4(eng, mid="md4", ac="md4_ac", bk="md4_bk"):
    m = MD4
    eng.putDisplaced(m["assets"], m["spots"], m["atms"], m["skews"], m["disc"], m["spreads"], m["div_dates"],
                     m["divs"], m["correl"], m["lam"], mid)
    a = MD4_AUTOCALL
    eng.putAutocall(m["assets"], a["refs"], a["maturity"], a["periods"], a["ko"], a["strike"], a["cpn"], a["smooth"],
                    ac)
    b = MD4_BASKET
    eng.putBaskets(m["assets"], b["weights"], b["maturity"], b["strikes"], bk)
    return mid, ac, bk


def run_md(product="autocall", paths=1 << 20, reps=1, precision="fp32", risk=True, device=0):
    """Times `reps` AADriskOne (risk) or value calls of the four-asset autocall or basket after one
    warm-up call (Sobol paths); returns seconds per call."""
    import time
    from compfinance_gb300 import Engine, NumericalParam
    eng = Engine(device)
    mid, ac, bk = put_md4(eng)
    pid = ac if product == "autocall" else bk
    num = NumericalParam(useSobol=True, numPath=int(paths), precision=precision)
    call = (lambda: eng.AADriskOne(mid, pid, num)) if risk else (lambda: eng.value(mid, pid, num))
    call()
    t0 = time.perf_counter()
    for _ in range(reps):
        call()
    dt = (time.perf_counter() - t0) / max(1, reps)
    eng.close()
    return dt

