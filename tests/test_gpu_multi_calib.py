"""AADriskMulti of a European portfolio, Dupire calibration, the superbucket, and
finite-difference checks of the adjoints, on the GPU."""
import numpy as np
import pytest

import oracle as O
from compfinance_gb300 import Engine
from compfinance_gb300 import workloads as W
from calib_util import support as _support
from gpu_util import num, rel_to_max

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng():
    e = Engine(0)
    yield e
    e.close()


@pytest.fixture(scope="module")
def portfolio(eng):
    mats, strikes = W.superbucket_portfolio(10, 20)
    s, t, v = W.dupire_surface(60, 30)
    eng.putDupire(100.0, s, t, v, 1.0 / 12.0, "c4dup")
    eng.putEuropeans(mats, strikes, "c4port")
    m = O.Model(dict(kind="dupire", spot=100.0, spots=s, times=t, vols=v, maxdt=1.0 / 12.0))
    p = O.Product(dict(kind="europeans", mats=mats, strikes=strikes))
    return m, p


@pytest.mark.parametrize("sob", [1, 0])
def test_aggregate_fp32_through_the_portfolio_kernels(eng, portfolio, monkeypatch, sob):
    """FP32 AADriskAggregate (and AADriskOne) of a European portfolio on Dupire runs the portfolio
    kernels and weighs the payoffs' risks on the device: it equals the weighted sum of AADriskMulti's
    risks on the same paths (to the rounding of the sum), and agrees with the generic kernel's aggregated adjoint
    (CF_FAST32=0) within 0.1 Monte Carlo standard error of each risk."""
    n = 1 << 16
    rs = np.random.RandomState(5)
    w = rs.uniform(-1.0, 2.0, 200)
    a = eng.AADriskAggregate("c4dup", "c4port", w, num(sob, n, "fp32"))
    m = eng.AADriskMulti("c4dup", "c4port", num(sob, n, "fp32"))
    assert rel_to_max(a["risks"], m["risks"] @ w) < 1e-12
    assert rel_to_max(np.array([a["riskPayoffValue"]]), np.array([m["values"] @ w])) < 1e-12
    assert rel_to_max(a["payoffValues"], m["values"]) == 0.0
    k = 37
    one = eng.AADriskOne("c4dup", "c4port", num(sob, n, "fp32"), eng.payoffLabels("c4port")[k])
    assert rel_to_max(one["risks"], m["risks"][:, k]) < 1e-12
    monkeypatch.setenv("CF_FAST32", "0")
    g = eng.AADriskAggregate("c4dup", "c4port", w, num(sob, n, "fp32"))
    monkeypatch.delenv("CF_FAST32")
    # standard error of each risk from 8 independent FP32 runs at a quarter of the paths
    se = np.std([eng.AADriskAggregate("c4dup", "c4port", w, num(0, n // 4, "fp32", seed1=900 + k, seed2=31 + k))["risks"]
                 for k in range(8)], axis=0, ddof=1) / 2.0
    mask = se > 1e-3 * np.abs(g["risks"]).max()
    assert np.max(np.abs(a["risks"] - g["risks"])[mask] / se[mask]) < 0.1
    assert abs(a["riskPayoffValue"] - g["riskPayoffValue"]) < 1e-4 * abs(g["riskPayoffValue"])


def test_multi_c4_shape_fp64_vs_oracle(eng, portfolio):
    """200 payoffs x 1801 parameters, 36 monthly steps: exact per-payoff path averages."""
    m, p = portfolio
    for sob in (1, 0):
        r = eng.AADriskMulti("c4dup", "c4port", num(sob, 2048))
        v, ref = O.risk_multi(m, p, sob, 2048)
        assert r["risks"].shape == (1801, 200)
        assert rel_to_max(r["values"], v) < 1e-12
        assert rel_to_max(r["risks"], ref) < 1e-12


def test_multi_fp32_vs_fp64(eng, portfolio):
    """FP32 paths vs FP64 on the same mrg32k3a paths: within 0.1 Monte Carlo standard error."""
    n = 1 << 16
    runs = np.array([eng.AADriskMulti("c4dup", "c4port", num(0, n // 4, "fp64", 3000 + k, 11 + k))["risks"]
                     for k in range(8)])
    se = runs.std(axis=0, ddof=1) / 2.0
    r64 = eng.AADriskMulti("c4dup", "c4port", num(0, n))
    r32 = eng.AADriskMulti("c4dup", "c4port", num(0, n, "fp32"))
    vse = eng.value("c4dup", "c4port", num(0, n))["stderrs"]
    assert np.all(np.abs(r32["values"] - r64["values"]) <= 0.1 * vse)
    mask = se > 1e-6 * np.abs(r64["risks"]).max()
    assert np.all(np.abs(r32["risks"] - r64["risks"])[mask] <= 0.1 * se[mask])
    assert np.all(np.abs(r32["risks"] - r64["risks"])[~mask] <= 1e-6 * np.abs(r64["risks"]).max())


def test_multi_fp32_sobol_vs_fp64(eng, portfolio):
    """FP32 Sobol paths (bucket-grouped kernels) vs FP64 on the same Sobol points: within 0.1
    Monte Carlo standard error (estimated from independent mrg32k3a runs of the same size)."""
    n = 1 << 16
    runs = np.array([eng.AADriskMulti("c4dup", "c4port", num(0, n // 4, "fp64", 5000 + k, 17 + k))["risks"]
                     for k in range(8)])
    se = runs.std(axis=0, ddof=1) / 2.0
    r64 = eng.AADriskMulti("c4dup", "c4port", num(1, n))
    r32 = eng.AADriskMulti("c4dup", "c4port", num(1, n, "fp32"))
    vse = eng.value("c4dup", "c4port", num(0, n))["stderrs"]
    assert np.all(np.abs(r32["values"] - r64["values"]) <= 0.1 * vse)
    mask = se > 1e-6 * np.abs(r64["risks"]).max()
    z = np.where(mask, np.abs(r32["risks"] - r64["risks"]) / np.where(mask, se, 1.0), 0.0)
    # A path whose spot at a maturity sits within FP32 rounding of a strike can land on the
    # other side of it: that payoff's column then differs by the path's own adjoint / n
    # (measured: 2 of 200 columns, 0.15 standard error at most, identical for the
    # generic FP32 kernel).  All other columns stay within 0.1 standard error.
    flipped = (z > 0.1).any(axis=0)
    assert flipped.sum() <= 3
    assert z.max() <= 0.3
    assert np.all(np.abs(r32["risks"] - r64["risks"])[~mask] <= 1e-6 * np.abs(r64["risks"]).max())


@pytest.mark.parametrize("sob", [1, 0])
def test_multi_fp32_deterministic(eng, portfolio, sob):
    """Each node contribution is rounded once to a fixed-point integer and the sums are integer
    sums, so repeated FP32 runs agree bit for bit whatever the order of the atomic adds."""
    a = eng.AADriskMulti("c4dup", "c4port", num(sob, 50000, "fp32"))
    b = eng.AADriskMulti("c4dup", "c4port", num(sob, 50000, "fp32"))
    assert np.array_equal(a["risks"], b["risks"]) and np.array_equal(a["values"], b["values"])


@pytest.mark.parametrize("sob,n", [(0, 1), (0, 777), (1, 1), (1, 31), (1, 1000)])
def test_multi_fp32_small_and_odd(eng, portfolio, sob, n):
    """Path counts that leave antithetic pairs and Sobol warp batches partly filled: FP32 within
    1e-3 of FP64 on the same paths (relative to the largest entry)."""
    r64 = eng.AADriskMulti("c4dup", "c4port", num(sob, n))
    r32 = eng.AADriskMulti("c4dup", "c4port", num(sob, n, "fp32"))
    assert rel_to_max(r32["values"], r64["values"]) < 1e-3
    # a path whose spot sits next to a strike may fall on the other side of it in FP32: compare
    # the risks column by column where the buckets agree, i.e. with a bound per flipped payoff
    bad = np.abs(r32["risks"] - r64["risks"]) > 1e-3 * np.abs(r64["risks"]).max()
    assert bad.any(axis=0).sum() <= max(1, r64["risks"].shape[1] // 100)


def test_multi_matches_risk_one(eng, portfolio):
    """Each column of AADriskMulti equals AADriskOne of that payoff on the same paths."""
    labels = eng.payoffLabels("c4port")
    r = eng.AADriskMulti("c4dup", "c4port", num(1, 4096))
    for k in (0, 7, 55, 199):
        one = eng.AADriskOne("c4dup", "c4port", num(1, 4096), labels[k])
        assert rel_to_max(r["risks"][:, k], one["risks"]) < 1e-12


def test_calibration_vs_reference(eng, golden):
    """Local vols from Dupire's formula on Black-Scholes prices (ivs.h:119-138).

    The formula divides a second strike difference of prices (step 1e-4) by 1e-8, so the
    reference's own local vols carry rounding noise (~1e-4 relative near the money, ~1e-3 at
    the +-2.5 std cut-off): ulp-level differences between CUDA's and glibc's exp/log show up
    at that level.
    """
    for c in golden("calib")["calib"]:
        iv = Engine.ivs(c["ivs"], c["ivs_params"][0], c["ivs_params"][1:])
        r = eng.dupireCalib(iv, c["incl_spots"], c["max_ds"], c["incl_times"], c["max_dt_vol"])
        assert list(r["spots"]) == c["spots"] and list(r["times"]) == c["times"]
        ref = np.array(c["lvols"]).reshape(r["lVols"].shape)
        rel = np.abs(r["lVols"] - ref) / np.abs(ref)
        print(c["name"], "max", rel.max(), "median", np.median(rel))
        assert rel.max() < 1e-2, c["name"]
        assert np.median(rel) < 1e-3, c["name"]


@pytest.mark.parametrize("which", ["sb_param", "sb_merton"])
def test_superbucket_vs_reference_and_oracle(eng, golden, which):
    c = [x for x in golden("calib")["superbucket"] if x["name"] == which][0]
    iv = Engine.ivs(c["ivs"], c["ivs_params"][0], c["ivs_params"][1:])
    eng.putEuropeans(c["portfolio"]["mats"], c["portfolio"]["strikes"], "sbport")
    w = np.zeros(len(c["portfolio"]["mats"]))
    for k, x in c["notionals"]:
        w[k] = x
    args = (iv, 100.0, c["maxdt"], "sbport", w, c["incl_spots"], c["max_ds"], c["incl_times"], c["max_dt_vol"],
            c["rv_strikes"], c["rv_mats"], num(1, c["npath"]))
    r = eng.dupireSuperbucket(*args, refSeeding=True)
    # the local vols differ from the reference's by their rounding noise (see above)
    print(which, r["value"] - c["value"], r["delta"] - c["delta"], rel_to_max(r["vega"], c["vega"]))
    assert abs(r["value"] - c["value"]) < 1e-4 * abs(c["value"])
    assert abs(r["delta"] - c["delta"]) < 1e-3 * abs(c["delta"])
    assert rel_to_max(r["vega"], c["vega"]) < 5e-2
    # the calibration adjoint alone, on the same microbucket, against the oracle's tape
    ex = eng.dupireSuperbucket(*args, refSeeding=False)
    oiv = O.ivs(c["ivs"], c["ivs_params"][0], c["ivs_params"][1:])
    ovega = O.calib_adjoint(oiv, c["incl_spots"], c["max_ds"], c["incl_times"], c["max_dt_vol"], c["rv_strikes"],
                            c["rv_mats"], ex["microbucket"])
    print(which, "adjoint vs oracle", rel_to_max(ex["vega"], ovega))
    assert rel_to_max(ex["vega"], ovega) < 1e-2


def _sb_case(golden, which):
    if which == "c4":
        return golden("baseline")["c4"]
    return [x for x in golden("calib")["superbucket"] if x["name"] == which][0]


@pytest.mark.parametrize("which", ["sb_param", "sb_merton", "c4"])
@pytest.mark.parametrize("ref_seeding", [True, False])
def test_calibration_adjoint_tight_vs_oracle_tape(eng, golden, which, ref_seeding):
    """The calibration adjoint alone (main.h:519-562), pinned tightly against the oracle's tape.

    Per node, Dupire's formula takes a second difference of 5 Black-Scholes prices divided by
    1e-8.  In the adjoint, the 5 points' terms, spread onto the risk view with nearly equal
    smoothstep weights, cancel: each vega entry is a sum of terms up to ~5e10 times the largest
    entry.  So the adjoint moves by ~3e-3 of its largest entry under a 1e-15 relative change of
    the prices, and two evaluation orders of the same sum agree only to a few ulps of its terms.
    The check is therefore split:
      * the forward values the adjoint is taken at (the 5 prices per node and their derivatives
        to the implied vol), where nothing cancels: GPU against oracle to 1e-13;
      * the adjoint of each point's implied vol (Dupire's partials, the seeding of the
        extrapolated nodes, at the GPU's forward values), where nothing cancels either: 1e-12;
      * each vega entry (the risk view's interpolation and the sums): to rounding, i.e. within
        1e-13 of the sum of the absolute values of its terms plus 1e-15 of the absolute point
        adjoints of the interpolation cells it is a corner of (see _support).
    Seeds: the reference's own microbucket where the fixture has one (param surface, C4), else
    seeded random adjoints (Merton surface)."""
    c = _sb_case(golden, which)
    iv = Engine.ivs(c["ivs"], c["ivs_params"][0], c["ivs_params"][1:])
    oiv = O.ivs(c["ivs"], c["ivs_params"][0], c["ivs_params"][1:])
    grid = (c["incl_spots"], c["max_ds"], c["incl_times"], c["max_dt_vol"])
    s, t, _ = O.calib(oiv, *grid)
    if "microbucket" in c:
        micro = np.array(c["microbucket"])
    else:
        micro = np.random.RandomState(41).standard_normal(len(s) * len(t))
    g = eng.calibAdjoint(iv, *grid, c["rv_strikes"], c["rv_mats"], micro, refSeeding=ref_seeding)
    o = O.calib_adjoint_given(oiv, *grid, c["rv_strikes"], c["rv_mats"], micro, calls=g["calls"],
                              vegas=g["callVegas"], ref_quirk=ref_seeding)
    assert np.array_equal(g["calls"] == 0.0, o["calls"] == 0.0)
    assert rel_to_max(g["calls"], o["calls"]) < 1e-13
    assert rel_to_max(g["callVegas"], o["vegas"]) < 1e-13
    assert np.abs(o["pointAdj"]).max() > 0
    assert rel_to_max(g["pointAdj"], o["pointAdj"]) < 1e-12
    bound = 1e-13 * o["absTerms"] + 1e-15 * _support(s, t, c["rv_strikes"], c["rv_mats"], o["pointAdj"])
    diff = np.abs(g["vega"] - o["vega"])
    print(which, ref_seeding, "point adjoints", rel_to_max(g["pointAdj"], o["pointAdj"]), "vega diff / bound",
          (diff / np.maximum(bound, 1e-300)).max(), "vega rel to max", rel_to_max(g["vega"], o["vega"]))
    assert np.all(diff <= bound)
    assert np.abs(o["vega"]).max() > 0


@pytest.mark.parametrize("which", ["sb_param", "c4"])
def test_microbucket_on_reference_local_vols(eng, golden, which):
    """The Monte Carlo half of the superbucket on the reference's own calibrated local vols: the
    book value, delta and microbucket (adjoints to every local vol) of the reference's
    dupireAADRisk on the same Sobol paths, to 1e-12 (C4: 200 Europeans, 36 monthly steps,
    60x30 local vols, 2^20 paths).  With the microbucket equal, the calibration adjoint of it
    is pinned by the test above: the remaining differences of the end-to-end vega from the
    reference's come from the local vols' own rounding noise."""
    c = _sb_case(golden, which)
    s, t = np.array(c["lvol_spots"]), np.array(c["lvol_times"])
    lv = np.array(c["lvols"]).reshape(len(s), len(t))
    eng.putDupire(100.0, s, t, lv, c["maxdt"], f"reflv_{which}")
    eng.putEuropeans(c["portfolio"]["mats"], c["portfolio"]["strikes"], f"refport_{which}")
    w = np.zeros(len(c["portfolio"]["mats"]))
    for k, x in c["notionals"]:
        w[k] = x
    r = eng.AADriskAggregate(f"reflv_{which}", f"refport_{which}", w, num(1, c["npath"]))
    assert abs(r["riskPayoffValue"] - c["value"]) <= 1e-12 * abs(c["value"])
    assert abs(r["risks"][0] - c["delta"]) <= 1e-12 * abs(c["delta"])
    assert rel_to_max(r["risks"][1:], c["microbucket"]) < 1e-12


def test_c4_superbucket_end_to_end_vs_reference(eng, golden):
    """The whole C4 chain on the GPU (calibration, 2^20 Sobol paths of Monte Carlo adjoints,
    calibration adjoint) against the reference's: value and delta to the local vols' rounding
    noise; vega within the loose end-to-end bound of that noise (the tight checks are above)."""
    c = golden("baseline")["c4"]
    iv = Engine.ivs(c["ivs"], c["ivs_params"][0], c["ivs_params"][1:])
    eng.putEuropeans(c["portfolio"]["mats"], c["portfolio"]["strikes"], "c4e2e")
    w = np.ones(len(c["portfolio"]["mats"]))
    r = eng.dupireSuperbucket(iv, 100.0, c["maxdt"], "c4e2e", w, c["incl_spots"], c["max_ds"], c["incl_times"],
                              c["max_dt_vol"], c["rv_strikes"], c["rv_mats"], num(1, c["npath"]), refSeeding=True)
    print("c4", r["value"] - c["value"], r["delta"] - c["delta"], rel_to_max(r["vega"], c["vega"]))
    assert abs(r["value"] - c["value"]) < 1e-4 * abs(c["value"])
    assert abs(r["delta"] - c["delta"]) < 1e-3 * abs(c["delta"])
    assert rel_to_max(r["vega"], c["vega"]) < 5e-2


def test_superbucket_finite_differences(eng):
    """Superbucket vega against bump / recalibrate / reprice of 20 seeded risk-view nodes
    (the reference's dupireSuperbucketBump, main.h:575-696), common random numbers."""
    iv = Engine.ivs("param", 100.0, [W.SB_IVS["a"], W.SB_IVS["b"], W.SB_IVS["c"], W.SB_IVS["sref"]])
    isp, mds, itm, mdt = W.superbucket_grid(30, 12)
    rk, rm = W.superbucket_riskview(15, 6)
    mats, strikes = W.superbucket_portfolio(5, 8)
    eng.putEuropeans(mats, strikes, "fdport")
    w = np.ones(len(mats))
    nm = num(1, 1 << 14)
    sb = eng.dupireSuperbucket(iv, 100.0, 1.0 / 12.0, "fdport", w, isp, mds, itm, mdt, rk, rm, nm)
    rs = np.random.RandomState(2018)
    nodes = [(rs.randint(len(rk)), rs.randint(len(rm))) for _ in range(20)]
    # The local vols carry the rounding noise of Dupire's formula (a second price difference
    # divided by 1e-8), so the calibrated value is a rough function of a spread: single
    # difference quotients of the calibration alone scatter by ~1 (0.5% of the largest vega)
    # for bumps of 1e-4..1e-3, and bumps above ~1e-3 leave the linear range (larger single-node
    # bumps of a coarse risk view admit butterfly arbitrage: NaN local vols).  The slope of a
    # least-squares line through +-1..5e-4 bumps averages that scatter.  The calibration
    # adjoint itself matches the oracle's tape to ~1e-3 (test above).
    scale = np.abs(sb["vega"]).max()
    hs = np.array([1e-4, 2e-4, 3e-4, 4e-4, 5e-4])
    checked = 0
    for (i, j) in nodes:
        xs, ys = [0.0], [sb["value"]]
        for h in np.concatenate([hs, -hs]):
            sp = np.zeros((len(rk), len(rm)))
            sp[i, j] = h
            cal = eng.dupireCalib(iv, isp, mds, itm, mdt, riskView=(rk, rm, sp))
            if not np.isfinite(cal["lVols"]).all():
                continue
            eng.putDupire(100.0, cal["spots"], cal["times"], cal["lVols"], 1.0 / 12.0, "fdmodel")
            xs.append(h)
            ys.append(eng.value("fdmodel", "fdport", nm)["values"] @ w)
        assert len(xs) >= 6, (i, j)
        fd = np.polyfit(np.array(xs), np.array(ys), 1)[0]
        v = sb["vega"][i, j]
        print(f"node ({i},{j}) fd {fd:.6f} vega {v:.6f}")
        assert abs(fd - v) <= 3e-2 * abs(v) + 1e-2 * scale, (i, j, fd, v)
        checked += 1
    assert checked == 20


def test_risk_finite_differences(eng):
    """AAD risks against central bumps on the same paths (common random numbers): spot on a
    European call, 8 seeded local vols on the barrier.  (The barrier's smoothing width is
    frozen at S0 * smooth, mcPrd.h:247, so its AAD spot risk deliberately omits
    d smooth / d spot, which a bumped spot would include.)"""
    s, t, v = W.dupire_surface(20, 10)
    u = W.UOC_BARRIER
    eng.putBarrier(u["strike"], u["barrier"], u["maturity"], u["monitor_freq"], u["smooth"], 0, "fduoc")
    eng.putEuropean(110.0, 2.0, 2.0, "fdcall")
    eng.putDupire(100.0, s, t, v, 0.25, "fdbase")
    nm = num(0, 1 << 14)
    rs = np.random.RandomState(7)
    cases = [("fdcall", -1, -1)] + [("fduoc", rs.randint(4, 16), rs.randint(10)) for _ in range(8)]
    for (prd, i, j) in cases:
        r = eng.AADriskOne("fdbase", prd, nm)["risks"]
        scale = np.abs(r).max()
        vals = []
        for sgn in (1.0, -1.0):
            if i < 0:
                h = 1e-4
                eng.putDupire(100.0 + sgn * h, s, t, v, 0.25, "fdbump")
            else:
                h = 1e-5
                vb = v.copy()
                vb[i, j] += sgn * h
                eng.putDupire(100.0, s, t, vb, 0.25, "fdbump")
            vals.append(eng.value("fdbump", prd, nm)["values"][0])
        fd = (vals[0] - vals[1]) / (2 * h)
        aad = r[0] if i < 0 else r[1 + i * 10 + j]
        # paths that straddle a payoff kink (strike, barrier breach) within the bump make the
        # difference quotient differ from the path derivative: an absolute error of order
        # 1e-4 of the largest risk at 2^14 paths
        assert abs(fd - aad) <= 2e-3 * abs(aad) + 1e-4 * scale, (prd, i, j, fd, aad)


def test_superbucket_c4_shape(eng):
    """C4 shape: 30x12 implied vols -> 60x30 local vols -> 200 Europeans, 36 monthly steps."""
    iv = Engine.ivs("param", 100.0, [W.SB_IVS["a"], W.SB_IVS["b"], W.SB_IVS["c"], W.SB_IVS["sref"]])
    isp, mds, itm, mdt = W.superbucket_grid(60, 30)
    rk, rm = W.superbucket_riskview(30, 12)
    mats, strikes = W.superbucket_portfolio(10, 20)
    eng.putEuropeans(mats, strikes, "c4port2")
    w = np.ones(len(mats))
    r = eng.dupireSuperbucket(iv, 100.0, 1.0 / 12.0, "c4port2", w, isp, mds, itm, mdt, rk, rm, num(1, 1 << 16))
    assert r["vega"].shape == (30, 12) and r["microbucket"].shape == (60, 30)
    assert np.isfinite(r["vega"]).all() and r["value"] > 0
