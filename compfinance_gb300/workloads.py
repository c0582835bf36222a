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
