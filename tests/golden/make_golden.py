#!/usr/bin/env python3
"""Write the golden fixtures of tests/golden/ by running the reference itself.

The reference's C++ (compiled in this container by oracle/build_ref.py into
oracle/_ref/ref_driver) is driven through its own entry points (value, AADriskOne,
AADriskAggregate, AADriskMulti, bumpRisk, dupireCalib, dupireSuperbucket, the RNG classes).
Every case records its inputs next to its outputs, so the fixtures are self-contained:
the tests never need the reference.

    python3 tests/golden/make_golden.py [rng host mc calib bump products multi_asset baseline]   # all when none named;
                                                                   # rebuilds the driver when missing
                                                                   # (from CF_REFERENCE_DIR)
"""
import json
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from compfinance_gb300 import workloads as W  # noqa: E402

DRIVER = os.path.join(ROOT, "oracle", "_ref", "ref_driver")
ONEOVER2POW32 = 2.3283064365387e-10
M1P1 = 4294967088.0


def run(cmds):
    if not os.path.exists(DRIVER):
        ref = os.environ.get("CF_REFERENCE_DIR")
        if not ref:
            raise SystemExit("oracle/_ref/ref_driver is missing: set CF_REFERENCE_DIR to the reference checkout")
        subprocess.check_call([sys.executable, os.path.join(ROOT, "oracle", "build_ref.py"), "--reference", ref])
    out = subprocess.run([DRIVER], input="\n".join(cmds) + "\n", capture_output=True, text=True,
                         check=True).stdout
    res = []
    for line in out.splitlines():
        tag, rest = line.split(" ", 1)
        if "|" in rest:
            res.append((tag, rest.split("|")[1:]))
        else:
            parts = rest.split()
            res.append((tag, [float.fromhex(x) for x in parts[1:]]))
    return res


def f(x):
    return float(x).hex()


def fl(xs):
    return " ".join(f(x) for x in xs)


def num(sobol, n, s1=12345, s2=1234, par=0):
    return f"{int(sobol)} {n} {s1} {s2} {par}"


def cmd_bs(mid, spot, vol, rate, div, qspot=0):
    return f"bs {mid} {f(spot)} {f(vol)} {qspot} {f(rate)} {f(div)}"


def cmd_dupire(mid, spot, maxdt, spots, times, vols):
    return (f"dupire {mid} {f(spot)} {f(maxdt)} {len(spots)} {fl(spots)} {len(times)} {fl(times)} "
            + fl(vols.reshape(-1)))


def cmd_uoc(pid, K, B, T, freq, smooth, cp=0):
    return f"uoc {pid} {f(K)} {f(B)} {f(T)} {f(freq)} {f(smooth)} {cp}"


def cmd_europeans(pid, mats, strikes):
    return f"europeans {pid} {len(mats)} {fl(mats)} {fl(strikes)}"


def models_products():
    """Model and product definitions shared by the MC cases (name -> spec, command)."""
    models, products = {}, {}
    b = W.BS_EUROPEAN
    models["bs"] = dict(kind="bs", spot=b["spot"], vol=b["vol"], rate=b["rate"], div=b["div"], qspot=0)
    models["bs_spotmeasure"] = dict(kind="bs", spot=100.0, vol=0.25, rate=0.03, div=0.01, qspot=1)
    models["bs_rates"] = dict(kind="bs", spot=100.0, vol=0.3, rate=0.05, div=0.02, qspot=0)
    for (nS, nT) in [(20, 10), (60, 30), (120, 60)]:
        s, t, v = W.dupire_surface(nS, nT)
        models[f"dup{nS}x{nT}"] = dict(kind="dupire", spot=W.DUPIRE_SPOT, maxdt=W.DUPIRE_MAXDT,
                                       spots=s.tolist(), times=t.tolist(), vols=v.tolist())
    s, t, v = W.dupire_surface(60, 30)
    models["dup60x30_fine"] = dict(kind="dupire", spot=W.DUPIRE_SPOT, maxdt=1.0 / 52.0,
                                   spots=s.tolist(), times=t.tolist(), vols=v.tolist())
    models["dup60x30_monthly"] = dict(kind="dupire", spot=W.DUPIRE_SPOT, maxdt=1.0 / 12.0,
                                      spots=s.tolist(), times=t.tolist(), vols=v.tolist())
    u = W.UOC_BARRIER
    products["euro"] = dict(kind="european", strike=100.0, exercise=1.0, settlement=1.0)
    products["euro_settle"] = dict(kind="european", strike=105.0, exercise=1.0, settlement=1.25)
    products["uoc"] = dict(kind="uoc", strike=u["strike"], barrier=u["barrier"], maturity=u["maturity"],
                           freq=u["monitor_freq"], smooth=u["smooth"], callput=0)
    products["uoc_put"] = dict(kind="uoc", strike=110.0, barrier=130.0, maturity=1.0, freq=1.0 / 12.0,
                               smooth=0.02, callput=1)
    products["uoc_monthly"] = dict(kind="uoc", strike=100.0, barrier=140.0, maturity=2.0, freq=1.0 / 12.0,
                                   smooth=0.0, callput=0)
    mats, strikes = [], []
    for t in (0.5, 1.0, 2.0, 3.0):
        for k in (80.0, 95.0, 110.0):
            mats.append(t)
            strikes.append(k)
    products["europeans"] = dict(kind="europeans", mats=mats, strikes=strikes)
    return models, products


def model_cmd(mid, m):
    import numpy as np
    if m["kind"] == "bs":
        return cmd_bs(mid, m["spot"], m["vol"], m["rate"], m["div"], m["qspot"])
    return cmd_dupire(mid, m["spot"], m["maxdt"], m["spots"], m["times"], np.array(m["vols"]))


def product_cmd(pid, p):
    if p["kind"] == "contingent":
        return f"contingent {pid} {f(p['coupon'])} {f(p['maturity'])} {f(p['freq'])} {f(p['smooth'])}"
    if p["kind"] == "european":
        return f"european {pid} {f(p['strike'])} {f(p['exercise'])} {f(p['settlement'])}"
    if p["kind"] == "uoc":
        return cmd_uoc(pid, p["strike"], p["barrier"], p["maturity"], p["freq"], p["smooth"], p["callput"])
    return cmd_europeans(pid, p["mats"], p["strikes"])


def rng_cases():
    out = {}
    cmds = ["sobol_dirhash", "sobol_u 1101 3", "sobol_u 8 300"]
    skips = [1, 2, 3, 31, 32, 63, 64, 1000, 65535, 524287, 1048575]
    cmds += [f"sobol_skip 36 {b}" for b in skips]
    cmds += ["mrg_u 12345 1234 3 6", "mrg_u 12345 12346 5 4", "mrg_g 12345 1234 156 3"]
    mskips = [0, 64, 128, 1000, 131072, 2097088, 4194240]
    cmds += [f"mrg_skip 12345 1234 156 {b}" for b in mskips]
    r = run(cmds)
    it = iter(r)
    out["sobol_dirhash"] = [int(x) for x in next(it)[1]]

    def ints(u):
        return [int(round(x / ONEOVER2POW32)) for x in u]
    out["sobol_1101"] = [ints(next(it)[1]) for _ in range(3)]
    out["sobol_8"] = [ints(next(it)[1]) for _ in range(300)]
    out["sobol_skip"] = []
    for b in skips:
        u = next(it)[1]
        g = next(it)[1]
        out["sobol_skip"].append(dict(dim=36, b=b, ints=ints(u), u=u, g=g))
    out["mrg_seq"] = []
    for (s1, s2, d, n, kind) in [(12345, 1234, 3, 6, "u"), (12345, 12346, 5, 4, "u"), (12345, 1234, 156, 3, "g")]:
        seq = []
        for _ in range(n):
            v = next(it)[1]
            st = next(it)[1]
            seq.append(dict(v=v, state=[int(x) for x in st[:6]], anti=int(st[6])))
        out["mrg_seq"].append(dict(seed1=s1, seed2=s2, dim=d, kind=kind, seq=seq))
    out["mrg_skip"] = []
    for b in mskips:
        st = next(it)[1]
        u = next(it)[1]
        out["mrg_skip"].append(dict(seed1=12345, seed2=1234, dim=156, b=b, state=[int(x) for x in st[:6]],
                                    anti=int(st[6]), u=u, diff=[int(round(x * M1P1)) for x in u]))
    # Gaussian functions on a grid that covers both branches of invNormalCdf and the cut-offs.
    import numpy as np
    rs = np.random.RandomState(7)
    ps = [1e-300, 1e-12, 2.3283064365387e-10, 1e-6, 0.02, 0.0799, 0.08, 0.0801, 0.25, 0.5,
          0.5000000000000008, 0.75, 0.9199, 0.92, 0.9201, 0.98, 1 - 1e-9, 1 - 2.3283064365387e-10]
    ps += rs.uniform(0, 1, 200).tolist()
    xs = [-12.0, -10.0, -9.99, -3.0, -1e-3, 0.0, 1e-3, 0.7, 3.0, 9.99, 10.0, 12.0]
    xs += rs.normal(0, 2, 100).tolist()
    r = run([f"invnorm {len(ps)} {fl(ps)}", f"normcdf {len(xs)} {fl(xs)}", f"normdens {len(xs)} {fl(xs)}"])
    out["invnorm"] = dict(p=ps, y=r[0][1])
    out["normcdf"] = dict(x=xs, y=r[1][1])
    out["normdens"] = dict(x=xs, y=r[2][1])
    return out


def host_cases(models, products):
    out = {}
    fills = [([0.0, 1.0, 3.0], 0.25, 0.0, []), ([0.0, 0.5, 0.51, 2.0], 0.1, 0.00136986301369863, [0.0]),
             ([0.1, 0.2, 3.0], 0.3, 0.000114469, [3.0]), ([1.0, 2.0], 0.3, 0.01, [])]
    cmds = []
    for (x, mx, mn, add) in fills:
        cmds.append(f"fill {len(x)} {fl(x)} {f(mx)} {f(mn)} {len(add)} {fl(add)}")
    pairs = [("bs", "euro"), ("bs_rates", "euro_settle"), ("bs", "uoc"), ("bs_spotmeasure", "europeans"),
             ("dup20x10", "uoc"), ("dup60x30", "uoc"), ("dup60x30_fine", "uoc_monthly"),
             ("dup60x30_monthly", "europeans"), ("dup20x10", "euro_settle"), ("dup20x10", "uoc_put")]
    for mid, m in models.items():
        cmds.append(model_cmd(mid, m))
    for pid, p in products.items():
        cmds.append(product_cmd(pid, p))
    for (mid, pid) in pairs:
        cmds.append(f"labels {mid} {pid}")
    r = run(cmds)
    it = iter(r)
    out["fill"] = [dict(x=x, maxdx=mx, mindx=mn, add=add, out=next(it)[1]) for (x, mx, mn, add) in fills]
    out["timelines"] = []
    for (mid, pid) in pairs:
        rec = dict(model=mid, product=pid)
        rec["payoff_labels"] = next(it)[1]
        rec["param_labels"] = next(it)[1]
        next(it)
        rec["product_timeline"] = next(it)[1]
        if models[mid]["kind"] == "dupire":
            rec["sim_timeline"] = next(it)[1]
            rec["common_steps"] = [int(x) for x in next(it)[1]]
            iv = next(it)[1]
            if mid == "dup20x10":
                rec["interp_vols"] = iv
        else:
            rec["sim_timeline"] = next(it)[1]
            rec["bs_stds"] = next(it)[1]
            rec["bs_drifts"] = next(it)[1]
            rec["bs_numeraires"] = next(it)[1]
        out["timelines"].append(rec)
    return out


def mc_cases(models, products):
    """(name, model, product, mode, sobol, nPath, extra)."""
    cases = [
        ("c1_bs_european_sobol", "bs", "euro", "risk", 1, 65536, 0),
        ("bs_european_mrg", "bs", "euro", "risk", 0, 4096, 0),
        ("bs_european_settle", "bs_rates", "euro_settle", "risk", 1, 4096, 0),
        ("bs_spotmeasure_european", "bs_spotmeasure", "euro", "risk", 1, 4096, 0),
        ("bs_uoc_mrg", "bs", "uoc", "risk", 0, 1024, 0),
        ("bs_uoc_mrg_p1", "bs", "uoc", "risk", 0, 1024, 1),
        ("bs_europeans_multi", "bs_spotmeasure", "europeans", "multi", 1, 1024, None),
    ] + [(f"bs_europeans_each_{k}", "bs_spotmeasure", "europeans", "risk", 1, 1024, k) for k in range(12)] + [
        ("dup20x10_uoc", "dup20x10", "uoc", "risk", 0, 2048, 0),
        ("c2_dup60x30_uoc", "dup60x30", "uoc", "risk", 0, 4096, 0),
        ("c2_dup60x30_uoc_p1", "dup60x30", "uoc", "risk", 0, 2048, 1),
        ("c2_dup60x30_uoc_value", "dup60x30", "uoc", "value", 0, 65536, None),
        ("dup120x60_uoc", "dup120x60", "uoc", "risk", 0, 1024, 0),
        ("dup60x30_uoc_sobol", "dup60x30", "uoc", "risk", 1, 1024, 0),
        ("dup20x10_uoc_put", "dup20x10", "uoc_put", "risk", 0, 2048, 0),
        ("dup60x30_fine_uoc_monthly", "dup60x30_fine", "uoc_monthly", "risk", 0, 1024, 0),
        ("dup20x10_european_settle", "dup20x10", "euro_settle", "risk", 1, 4096, 0),
        ("dup60x30_europeans_multi", "dup60x30_monthly", "europeans", "multi", 1, 1024, None),
        ("dup60x30_europeans_agg", "dup60x30_monthly", "europeans", "agg", 1, 1024,
         [(0, 1.0), (4, -2.0), (7, 0.5), (11, 3.0)]),
    ]
    cmds = [model_cmd(mid, m) for mid, m in models.items()] + \
           [product_cmd(pid, p) for pid, p in products.items()]
    n_setup = 0
    for (name, mid, pid, mode, sob, n, extra) in cases:
        nm = num(sob, n)
        if mode == "value":
            cmds.append(f"value {mid} {pid} {nm}")
        elif mode == "risk":
            cmds.append(f"risk {mid} {pid} {nm} {extra}")
        elif mode == "multi":
            cmds.append(f"riskmulti {mid} {pid} {nm}")
        else:
            cmds.append(f"riskagg {mid} {pid} {nm} {len(extra)} " + " ".join(f"{k} {f(w)}" for k, w in extra))
    r = run(cmds)
    it = iter(r[n_setup:])
    out = {"models": models, "products": products, "cases": []}
    for (name, mid, pid, mode, sob, n, extra) in cases:
        rec = dict(name=name, model=mid, product=pid, mode=mode, sobol=sob, npath=n, seed1=12345, seed2=1234)
        if mode == "value":
            rec["values"] = next(it)[1]
            next(it)
        elif mode == "risk":
            rec["payoff"] = extra
            rec["values"] = next(it)[1]
            rec["risk_value"] = next(it)[1][0]
            rec["risks"] = next(it)[1]
            next(it)
        elif mode == "multi":
            rec["values"] = next(it)[1]
            rec["risks"] = next(it)[1]
            rec["shape"] = [int(x) for x in next(it)[1]]
            next(it)
        else:
            rec["notionals"] = extra
            rec["values"] = next(it)[1]
            rec["risk_value"] = next(it)[1][0]
            rec["risks"] = next(it)[1]
        out["cases"].append(rec)
    return out


def bump_cases(models, products):
    """bumpRisk (main.h:316-359): every model parameter bumped by 1e-8 and the product repriced on
    the same random numbers; risks[nParam][nPay] = 1e8 (bumped - base)."""
    cases = [
        ("bs_european_mrg", "bs", "euro", 0, 4096),
        ("bs_europeans_sobol", "bs_spotmeasure", "europeans", 1, 1024),
        ("bs_uoc_mrg", "bs", "uoc", 0, 1024),
        ("dup20x10_uoc_mrg", "dup20x10", "uoc", 0, 1024),
        ("dup20x10_uoc_sobol", "dup20x10", "uoc", 1, 512),
        ("dup20x10_european_settle_sobol", "dup20x10", "euro_settle", 1, 1024),
        ("dup60x30_uoc_mrg", "dup60x30", "uoc", 0, 256),
        ("dup60x30_monthly_europeans_sobol", "dup60x30_monthly", "europeans", 1, 256),
    ]
    cmds = [model_cmd(mid, m) for mid, m in models.items()] + \
           [product_cmd(pid, p) for pid, p in products.items()]
    cmds += [f"bump {mid} {pid} {num(sob, n)}" for (_, mid, pid, sob, n) in cases]
    it = iter(run(cmds))
    out = {"models": models, "products": products, "cases": []}
    for (name, mid, pid, sob, n) in cases:
        rec = dict(name=name, model=mid, product=pid, sobol=sob, npath=n, seed1=12345, seed2=1234)
        rec["values"] = next(it)[1]
        rec["risks"] = next(it)[1]
        rec["shape"] = [int(x) for x in next(it)[1]]
        next(it)
        out["cases"].append(rec)
    # dupireSuperbucketBump (main.h:575-696): Merton surface, a reduced portfolio and risk view
    mats, strikes = [], []
    for t in (0.5, 1.0, 2.0):
        for k in (90.0, 100.0, 115.0):
            mats.append(t)
            strikes.append(k)
    small_s = [60.0, 80.0, 90.0, 100.0, 110.0, 125.0, 150.0]
    small_t = [0.25, 0.5, 1.0, 2.0]
    rv_k, rv_m = W.superbucket_riskview(8, 5)
    nots = [(0, 1.0), (1, 2.0), (4, -1.0), (8, 0.5)]
    mert = [0.15, 0.5, -0.1, 0.15]
    ivs = "merton " + " ".join(f(x) for x in [100.0] + mert)
    r = run([cmd_europeans("sbp", mats, strikes),
             f"superbucket_bump {ivs} {len(small_s)} {fl(small_s)} {f(10.0)} {len(small_t)} {fl(small_t)} {f(0.25)} "
             f"{f(1.0 / 12.0)} sbp {len(nots)} " + " ".join(f"{k} {f(w)}" for k, w in nots) +
             f" {len(rv_k)} {fl(rv_k)} {len(rv_m)} {fl(rv_m)} {num(1, 1024)}"])
    d = {tag: v for tag, v in r}
    out["superbucket_bump"] = dict(ivs="merton", ivs_params=[100.0] + mert, incl_spots=small_s, max_ds=10.0,
                                   incl_times=small_t, max_dt_vol=0.25, maxdt=1.0 / 12.0,
                                   portfolio=dict(mats=mats, strikes=strikes), notionals=nots, rv_strikes=rv_k,
                                   rv_mats=rv_m, sobol=1, npath=1024, value=d["sb_value"][0], delta=d["sb_delta"][0],
                                   vega=d["sb_vega"])
    return out


def product_cases(models):
    """The contingent bond (mcPrd.h:404-574): pays (libor + coupon) x coverage at the end of each
    period whose spot rose (a smoothed digital), plus the redemption; on Black-Scholes (risk-
    neutral and spot measure: libors and numeraires) and Dupire (no rates).  value, AADriskOne
    and bumpRisk through the reference."""
    products = {"cbond": dict(kind="contingent", coupon=0.02, maturity=3.0, freq=0.25, smooth=0.05),
                "cbond_sharp": dict(kind="contingent", coupon=0.035, maturity=2.0, freq=0.5, smooth=0.0),
                "cbond_monthly": dict(kind="contingent", coupon=0.01, maturity=1.0, freq=1.0 / 12.0, smooth=0.02)}
    cases = [("bs_cbond_mrg", "bs", "cbond", 0, 4096), ("bs_cbond_sobol", "bs", "cbond", 1, 2048),
             ("bs_rates_cbond_monthly", "bs_rates", "cbond_monthly", 0, 2048),
             ("bs_spotmeasure_cbond", "bs_spotmeasure", "cbond", 1, 2048),
             ("bs_cbond_sharp", "bs_rates", "cbond_sharp", 0, 2048),
             ("dup20x10_cbond", "dup20x10", "cbond", 0, 2048), ("dup60x30_monthly_cbond", "dup60x30_monthly",
                                                                 "cbond_monthly", 1, 1024)]
    used = {c[1] for c in cases}
    cmds = [model_cmd(mid, m) for mid, m in models.items() if mid in used] + \
           [product_cmd(pid, p) for pid, p in products.items()]
    for (_, mid, pid, sob, n) in cases:
        cmds += [f"value {mid} {pid} {num(sob, n)}", f"risk {mid} {pid} {num(sob, n)} 0",
                 f"bump {mid} {pid} {num(sob, min(n, 512))}"]
    it = iter(run(cmds))
    out = {"models": {k: v for k, v in models.items() if k in used}, "products": products, "cases": []}
    for (name, mid, pid, sob, n) in cases:
        rec = dict(name=name, model=mid, product=pid, sobol=sob, npath=n, bump_npath=min(n, 512),
                   seed1=12345, seed2=1234)
        rec["values"] = next(it)[1]
        next(it)
        next(it)  # risk: values
        rec["risk_value"] = next(it)[1][0]
        rec["risks"] = next(it)[1]
        next(it)
        next(it)  # bump: values
        rec["bump_risks"] = next(it)[1]
        next(it)
        next(it)
        out["cases"].append(rec)
    return out


def md_models_products():
    """Multi-asset displaced model (mcMdlMultiDisplaced.h) and products (mcPrdMulti.h).  The four
    assets of md4 take the four dynamics of the displacement rule: skew 0 (lognormal),
    atm + 2 skew > 0 (surnormal), < 0 (subnormal), = 0 (normal)."""
    models = {
        "md4": dict(assets=["A", "B", "C", "D"], spots=[100.0, 50.0, 80.0, 120.0], atms=[0.2, 0.25, 0.15, 0.2],
                    skews=[0.0, -0.05, -0.1, -0.1], disc=0.03, spreads=[0.01, 0.0, 0.02, -0.01],
                    div_dates=[0.4, 1.2, 2.5],
                    divs=[[0.02, 0.0, 0.01, 0.03], [0.01, 0.02, 0.0, 0.0], [0.02, 0.01, 0.01, 0.01]],
                    correl=[[1.0, 0.5, 0.3, 0.2], [0.5, 1.0, 0.4, 0.1], [0.3, 0.4, 1.0, 0.25], [0.2, 0.1, 0.25, 1.0]],
                    **{"lambda": 0.1}),
        "md2": dict(assets=["X", "Y"], spots=[100.0, 100.0], atms=[0.2, 0.3], skews=[0.0, -0.05], disc=0.02,
                    spreads=[0.0, 0.005], div_dates=[0.5], divs=[[0.02, 0.0]], correl=[[1.0, 0.6], [0.6, 1.0]],
                    **{"lambda": 0.0}),
    }
    products = {
        "bask4": dict(kind="baskets", assets=["A", "B", "C", "D"], weights=[0.25, 0.3, 0.2, 0.25], maturity=2.0,
                      strikes=[70.0, 80.0, 86.0, 95.0, 105.0]),
        "ac4": dict(kind="autocall", assets=["A", "B", "C", "D"], refs=[100.0, 50.0, 80.0, 120.0], maturity=3.0,
                    periods=6, ko=1.0, strike=0.7, cpn=0.06, smooth=0.05),
        "ac4_sharp": dict(kind="autocall", assets=["A", "B", "C", "D"], refs=[100.0, 50.0, 80.0, 120.0],
                          maturity=2.0, periods=4, ko=1.05, strike=0.8, cpn=0.04, smooth=0.0),
        "bask2": dict(kind="baskets", assets=["X", "Y"], weights=[0.5, 0.5], maturity=1.0, strikes=[100.0, 108.0]),
        "ac2": dict(kind="autocall", assets=["X", "Y"], refs=[100.0, 100.0], maturity=1.0, periods=12, ko=1.02,
                    strike=0.75, cpn=0.03, smooth=0.02),
    }
    return models, products


def md_model_cmd(mid, m):
    n = len(m["assets"])
    divs = [x for row in m["divs"] for x in row]
    corr = [x for row in m["correl"] for x in row]
    return (f"displaced {mid} {n} {' '.join(m['assets'])} {fl(m['spots'])} {fl(m['atms'])} {fl(m['skews'])} "
            f"{f(m['disc'])} {fl(m['spreads'])} {len(m['div_dates'])} {fl(m['div_dates'])} {fl(divs)} {fl(corr)} "
            f"{f(m['lambda'])}")


def md_product_cmd(pid, p):
    n = len(p["assets"])
    if p["kind"] == "baskets":
        return (f"baskets {pid} {n} {' '.join(p['assets'])} {fl(p['weights'])} {f(p['maturity'])} "
                f"{len(p['strikes'])} {fl(p['strikes'])}")
    return (f"autocall {pid} {n} {' '.join(p['assets'])} {fl(p['refs'])} {f(p['maturity'])} {p['periods']} "
            f"{f(p['ko'])} {f(p['strike'])} {f(p['cpn'])} {f(p['smooth'])}")


def multi_asset_cases():
    """value, AADriskOne, AADriskAggregate, AADriskMulti and bumpRisk of the multi-asset products
    through the reference, with the model's initialised quantities (Cholesky factor, per-step
    stds, drifts and dividend-adjusted forward factors, displacements, numeraires)."""
    models, products = md_models_products()
    cases = [("md4_bask4_sobol", "md4", "bask4", 1, 4096), ("md4_bask4_mrg", "md4", "bask4", 0, 4096),
             ("md4_ac4_sobol", "md4", "ac4", 1, 2048), ("md4_ac4_mrg", "md4", "ac4", 0, 2048),
             ("md4_ac4_sharp", "md4", "ac4_sharp", 1, 2048), ("md2_bask2_sobol", "md2", "bask2", 1, 2048),
             ("md2_ac2_mrg", "md2", "ac2", 0, 2048)]
    cmds = [md_model_cmd(mid, m) for mid, m in models.items()] + \
           [md_product_cmd(pid, p) for pid, p in products.items()]
    for (_, mid, pid, sob, n) in cases:
        npay = len(products[pid]["strikes"]) if products[pid]["kind"] == "baskets" else 1
        agg = [(k, 1.0 + 0.5 * k) for k in range(npay)]
        cmds += [f"labels {mid} {pid}", f"value {mid} {pid} {num(sob, n)}", f"risk {mid} {pid} {num(sob, n)} 0",
                 f"riskagg {mid} {pid} {num(sob, n)} {len(agg)} " + " ".join(f"{k} {f(w)}" for k, w in agg),
                 f"riskmulti {mid} {pid} {num(sob, n)}", f"bump {mid} {pid} {num(sob, min(n, 512))}"]
    res = run(cmds)
    it = iter(res)
    out = {"models": models, "products": products, "cases": []}
    for (name, mid, pid, sob, n) in cases:
        npay = len(products[pid]["strikes"]) if products[pid]["kind"] == "baskets" else 1
        rec = dict(name=name, model=mid, product=pid, sobol=sob, npath=n, bump_npath=min(n, 512), seed1=12345,
                   seed2=1234, agg_weights=[1.0 + 0.5 * k for k in range(npay)])
        d = {}
        while True:  # labels block: tags until md_dynamics
            tag, v = next(it)
            d[tag] = v
            if tag == "md_dynamics":
                break
        rec["payoff_labels"], rec["param_labels"] = d["payoff_labels"], d["param_labels"]
        for k in ("sim_timeline", "md_chol", "md_stds", "md_drifts", "md_ffs", "md_numeraires", "md_alphas",
                  "md_dynamics"):
            rec[k] = d[k]
        rec["values"] = next(it)[1]
        next(it)
        next(it)
        rec["risk_value"] = next(it)[1][0]
        rec["risks"] = next(it)[1]
        next(it)
        next(it)
        rec["agg_value"] = next(it)[1][0]
        rec["agg_risks"] = next(it)[1]
        next(it)
        rec["multi_risks"] = next(it)[1]
        next(it)
        next(it)
        next(it)
        rec["bump_risks"] = next(it)[1]
        next(it)
        next(it)
        out["cases"].append(rec)
    return out


def calib_cases():
    out = {}
    incl_spots, maxds, incl_times, maxdtv = W.superbucket_grid(60, 30)
    iv = W.SB_IVS
    small_s = [60.0, 80.0, 90.0, 100.0, 110.0, 125.0, 150.0]
    small_t = [0.25, 0.5, 1.0, 2.0]
    specs = [
        ("param_60x30", f"param {f(100.0)} {f(iv['a'])} {f(iv['b'])} {f(iv['c'])} {f(iv['sref'])}",
         incl_spots, maxds, incl_times, maxdtv),
        ("param_refined", f"param {f(100.0)} {f(iv['a'])} {f(iv['b'])} {f(iv['c'])} {f(iv['sref'])}",
         small_s, 7.5, small_t, 0.2),
        ("merton_small", f"merton {f(100.0)} {f(0.15)} {f(0.5)} {f(-0.1)} {f(0.15)}",
         small_s, 10.0, small_t, 0.25),
    ]
    cmds = []
    for (name, ivs, s, mds, t, mdt) in specs:
        cmds.append(f"calib {ivs} {len(s)} {fl(s)} {f(mds)} {len(t)} {fl(t)} {f(mdt)}")
    r = run(cmds)
    out["calib"] = []
    for k, (name, ivs, s, mds, t, mdt) in enumerate(specs):
        out["calib"].append(dict(name=name, ivs=ivs.split()[0], ivs_params=[float.fromhex(x) for x in ivs.split()[1:]],
                                 incl_spots=s, max_ds=mds, incl_times=t, max_dt_vol=mdt,
                                 spots=r[3 * k][1], times=r[3 * k + 1][1], lvols=r[3 * k + 2][1]))
    # Superbucket on a reduced portfolio, both surfaces.
    mats, strikes = [], []
    for t in (0.5, 1.0, 2.0):
        for k in (90.0, 100.0, 115.0):
            mats.append(t)
            strikes.append(k)
    rv_k, rv_m = W.superbucket_riskview(8, 5)
    nots = [(0, 1.0), (1, 2.0), (4, -1.0), (8, 0.5)]
    sbs = []
    for (name, ivs, s, mds, t, mdt, npath) in [
            ("sb_param", specs[0][1], incl_spots[::3], maxds, incl_times[::3], 3.0, 2048),
            ("sb_merton", specs[2][1], small_s, 10.0, small_t, 0.25, 1024)]:
        cmds = [cmd_europeans("sbp", mats, strikes),
                f"superbucket {ivs} {len(s)} {fl(s)} {f(mds)} {len(t)} {fl(t)} {f(mdt)} {f(1.0 / 12.0)} sbp "
                f"{len(nots)} " + " ".join(f"{k} {f(w)}" for k, w in nots) +
                f" {len(rv_k)} {fl(rv_k)} {len(rv_m)} {fl(rv_m)} {num(1, npath)}"]
        r = run(cmds)
        d = {tag: v for tag, v in r}
        rec = dict(name=name, ivs=ivs.split()[0], ivs_params=[float.fromhex(x) for x in ivs.split()[1:]],
                   incl_spots=s, max_ds=mds, incl_times=t, max_dt_vol=mdt, maxdt=1.0 / 12.0,
                   portfolio=dict(mats=mats, strikes=strikes), notionals=nots, rv_strikes=rv_k, rv_mats=rv_m,
                   sobol=1, npath=npath, value=d["sb_value"][0], delta=d["sb_delta"][0], vega=d["sb_vega"])
        if "sb_microbucket" in d:
            rec["microbucket"] = d["sb_microbucket"]
            rec["lvol_spots"], rec["lvol_times"], rec["lvols"] = d["sb_spots"], d["sb_times"], d["sb_lvols"]
        sbs.append(rec)
    out["superbucket"] = sbs
    r = run([f"analytics {f(100.0)} {f(110.0)} {f(0.2)} {f(1.5)} {f(0.03)} {f(0.01)} {f(140.0)}"])
    out["analytics"] = dict(inputs=[100.0, 110.0, 0.2, 1.5, 0.03, 0.01, 140.0], out=r[0][1])
    return out


def baseline_cases(models, products):
    """The benchmark's own configurations through the reference: the 60x30 Dupire barrier's
    AADriskOne at 2^18 mrg32k3a paths (1801 risks), and the superbucket of the 200-European
    portfolio (parametric implied surface, 60x30 local vols, 30x12 risk view, 36 monthly steps)
    at 2^20 Sobol paths, with the reference's calibrated local vols and microbucket."""
    out = {}
    m = models["dup60x30"]
    cmds = [model_cmd("dup60x30", m), product_cmd("uoc", products["uoc"]),
            f"risk dup60x30 uoc {num(0, 1 << 18, par=1)} 0"]
    r = run(cmds)
    out["c2"] = dict(model="dup60x30", product="uoc", mode="risk", sobol=0, npath=1 << 18, seed1=12345, seed2=1234,
                     payoff=0, values=r[0][1], risk_value=r[1][1][0], risks=r[2][1])
    iv = W.SB_IVS
    ivs = f"param {f(100.0)} {f(iv['a'])} {f(iv['b'])} {f(iv['c'])} {f(iv['sref'])}"
    isp, mds, itm, mdt = W.superbucket_grid(60, 30)
    rk, rm = W.superbucket_riskview(30, 12)
    mats, strikes = W.superbucket_portfolio(10, 20)
    nots = [(k, 1.0) for k in range(len(mats))]
    cmds = [cmd_europeans("c4port", mats, strikes),
            f"superbucket {ivs} {len(isp)} {fl(isp)} {f(mds)} {len(itm)} {fl(itm)} {f(mdt)} {f(1.0 / 12.0)} c4port "
            f"{len(nots)} " + " ".join(f"{k} {f(w)}" for k, w in nots) +
            f" {len(rk)} {fl(rk)} {len(rm)} {fl(rm)} {num(1, 1 << 20, par=1)}"]
    d = {tag: v for tag, v in run(cmds)}
    out["c4"] = dict(ivs="param", ivs_params=[100.0, iv["a"], iv["b"], iv["c"], iv["sref"]], incl_spots=isp,
                     max_ds=mds, incl_times=itm, max_dt_vol=mdt, maxdt=1.0 / 12.0,
                     portfolio=dict(mats=mats, strikes=strikes), notionals=nots, rv_strikes=rk, rv_mats=rm,
                     sobol=1, npath=1 << 20, value=d["sb_value"][0], delta=d["sb_delta"][0], vega=d["sb_vega"],
                     microbucket=d["sb_microbucket"], lvol_spots=d["sb_spots"], lvol_times=d["sb_times"],
                     lvols=d["sb_lvols"])
    return out


def main():
    models, products = models_products()
    only = set(sys.argv[1:])
    for name, fn in [("rng", rng_cases), ("host", lambda: host_cases(models, products)),
                     ("mc", lambda: mc_cases(models, products)), ("calib", calib_cases),
                     ("bump", lambda: bump_cases(models, products)), ("products", lambda: product_cases(models)),
                     ("multi_asset", multi_asset_cases),
                     ("baseline", lambda: baseline_cases(models, products))]:
        if only and name not in only:
            continue
        obj = fn()
        path = os.path.join(HERE, f"{name}.json")
        with open(path, "w") as fh:
            json.dump(obj, fh, separators=(",", ":"))
        print(path, os.path.getsize(path))


if __name__ == "__main__":
    main()
