"""Parity of the CUDA engine (through the C ABI) with the reference.

* RNG: Sobol integer points and mrg32k3a states bit-exact; Gaussians within 1 ulp-level.
* FP64 form: prices and risks of every golden case within 1e-12 (relative to the largest
  entry) of the reference's own mcSimul / mcSimulAAD results on the same RNG sequence.
"""
import numpy as np
import pytest

import oracle as O
from compfinance_gb300 import Engine
from gpu_util import num, put_model, put_product, rel_to_max

pytestmark = pytest.mark.gpu

TOL = 1e-12


@pytest.fixture(scope="module")
def eng():
    e = Engine(0)
    yield e
    e.close()


def test_sobol_points_bit_exact(eng, golden):
    g = golden("rng")
    assert (eng.sobolPoints(1101, 0, 3) == np.array(g["sobol_1101"], dtype=np.uint32)).all()
    assert (eng.sobolPoints(8, 0, 300) == np.array(g["sobol_8"], dtype=np.uint32)).all()
    for c in g["sobol_skip"]:
        assert (eng.sobolPoints(c["dim"], c["b"], 1)[0] == np.array(c["ints"], dtype=np.uint32)).all(), c["b"]
    # large indices against the oracle (skip-ahead by gray code)
    for first in (123456789, (1 << 30) + 12345):
        assert (eng.sobolPoints(64, first, 40) == O.sobol_ints(64, first, 40)).all()


def test_mrg_states_bit_exact(eng, golden):
    for c in golden("rng")["mrg_skip"]:
        st = eng.mrgState(c["seed1"], c["seed2"], c["dim"], c["b"])
        assert list(st) == c["state"], c["b"]
    for first in (0, 2, 1 << 21, (1 << 40) + 6):
        assert list(eng.mrgState(12345, 1234, 156, first)) == list(O.mrg_state(12345, 1234, 156, first))


def test_gaussians(eng, golden):
    seq = [s for s in golden("rng")["mrg_seq"] if s["kind"] == "g"][0]
    got = eng.gaussians(False, seq["seed1"], seq["seed2"], seq["dim"], 0, len(seq["seq"]))
    ref = np.array([r["v"] for r in seq["seq"]])
    # The uniforms are bit-exact; the inverse normal differs from glibc's by a few ulps
    # (CUDA's double log, and FMA contraction of the Beasley-Springer-Moro polynomials).
    assert (np.abs(got - ref) <= 16 * np.spacing(np.abs(ref))).all()
    for sob in (0, 1):
        got = eng.gaussians(sob, 12345, 1234, 36, 1000, 200)
        ref = O.sobol_gauss(36, 1000, 200) if sob else O.mrg_gauss(12345, 1234, 36, 1000, 200)
        assert (np.abs(got - ref) <= 16 * np.spacing(np.abs(ref))).all()
        assert (got == ref).mean() > 0.5


@pytest.fixture(scope="module")
def mc_eng(eng, golden):
    d = golden("mc")
    for mid, spec in d["models"].items():
        put_model(eng, mid, spec)
    for pid, spec in d["products"].items():
        put_product(eng, pid, spec)
    return eng, d


def test_labels(mc_eng, golden):
    eng, _ = mc_eng
    for t in golden("host")["timelines"]:
        assert eng.payoffLabels(t["product"]) == t["payoff_labels"]
        assert eng.parameterLabels(t["model"]) == t["param_labels"]
        _, _, dim = eng.shapes(t["model"], t["product"])
        assert dim == len(t["sim_timeline"]) - 1


def test_label_cache_follows_the_model(eng):
    """Parameter labels stay cached while a Dupire model is re-put on the same grid, and follow it
    when the grid or the model kind changes."""
    from compfinance_gb300 import workloads as W
    s, t, v = W.dupire_surface(20, 10)
    eng.putDupire(W.DUPIRE_SPOT, s, t, v, W.DUPIRE_MAXDT, "lab")
    first = eng.parameterLabels("lab")
    assert len(first) == 1 + 20 * 10 and first[0] == "spot"
    eng.putDupire(W.DUPIRE_SPOT, s, t, v * 1.1, W.DUPIRE_MAXDT, "lab")  # new vols, same grid
    assert eng.parameterLabels("lab") == first
    eng.putBlackScholes(100.0, 0.2, 0, 0.0, 0.0, "lab")
    assert eng.parameterLabels("lab") == ["spot", "vol", "rate", "div"]
    eng.putDupire(W.DUPIRE_SPOT, s, t, v, W.DUPIRE_MAXDT, "lab")  # back on the first grid
    assert eng.parameterLabels("lab") == first
    s2, t2, v2 = W.dupire_surface(12, 6)
    eng.putDupire(W.DUPIRE_SPOT, s2, t2, v2, W.DUPIRE_MAXDT, "lab")
    assert len(eng.parameterLabels("lab")) == 1 + 12 * 6


def _weights(c, npay):
    w = np.zeros(npay)
    if c["mode"] == "risk":
        w[c["payoff"]] = 1.0
    else:
        for k, x in c["notionals"]:
            w[k] = x
    return w


def test_fp64_parity_with_reference(mc_eng):
    eng, d = mc_eng
    worst = {}
    for c in d["cases"]:
        nm = num(c["sobol"], c["npath"])
        mid, pid = c["model"], c["product"]
        npay, npar, _ = eng.shapes(mid, pid)
        if c["mode"] == "value":
            r = eng.value(mid, pid, nm)
            err = rel_to_max(r["values"], c["values"])
        elif c["mode"] in ("risk", "agg"):
            labels = eng.payoffLabels(pid)
            if c["mode"] == "risk":
                r = eng.AADriskOne(mid, pid, nm, labels[c["payoff"]])
            else:
                r = eng.AADriskAggregate(mid, pid, _weights(c, npay), nm)
            err = max(rel_to_max(r["payoffValues"], c["values"]),
                      abs(r["riskPayoffValue"] - c["risk_value"]) / abs(c["risk_value"]),
                      rel_to_max(r["risks"], c["risks"]))
        else:
            r = eng.AADriskMulti(mid, pid, nm)
            m, p = O.Model(d["models"][mid]), O.Product(d["products"][pid])
            _, ref = O.risk_multi(m, p, c["sobol"], c["npath"])  # exact path average
            err = max(rel_to_max(r["values"], c["values"]), rel_to_max(r["risks"], ref))
        worst[c["name"]] = err
    bad = {k: v for k, v in worst.items() if not v < TOL}
    assert not bad, bad


def test_fp64_parity_large_vs_oracle(mc_eng):
    # C2 shape (Dupire 60x30 UOC, 156 weekly steps, mrg32k3a) at 2^16 paths vs the oracle
    eng, d = mc_eng
    m, p = O.Model(d["models"]["dup60x30"]), O.Product(d["products"]["uoc"])
    v, agg, ref = O.risk(m, p, 0, 1 << 16, np.array([1.0, 0.0]), fast=True, threads=8)
    r = eng.AADriskOne("dup60x30", "uoc", num(0, 1 << 16))
    assert rel_to_max(r["payoffValues"], v) < TOL
    assert rel_to_max(r["risks"], ref) < TOL


def test_determinism(mc_eng):
    eng, _ = mc_eng
    a = eng.AADriskOne("dup60x30", "uoc", num(0, 50000, "fp32"))
    b = eng.AADriskOne("dup60x30", "uoc", num(0, 50000, "fp32"))
    assert (a["risks"] == b["risks"]).all() and (a["payoffValues"] == b["payoffValues"]).all()


def test_odd_and_tiny_path_counts(mc_eng):
    eng, d = mc_eng
    m, p = O.Model(d["models"]["dup20x10"]), O.Product(d["products"]["uoc"])
    for n in (1, 2, 3, 31, 33, 1001):
        for sob in (0, 1):
            v, agg, ref = O.risk(m, p, sob, n, np.array([1.0, 0.0]))
            r = eng.AADriskOne("dup20x10", "uoc", num(sob, n))
            assert rel_to_max(r["payoffValues"], v) < TOL, (n, sob)
            assert rel_to_max(r["risks"], ref) < TOL, (n, sob)


@pytest.mark.parametrize("grid", [(20, 10), (60, 30), (120, 60)])
def test_fp32_form_within_tenth_of_stderr(eng, grid):
    """FP32 path arithmetic with exact accumulation vs the FP64 form on the same paths: every
    price and every risk within 0.1 Monte Carlo standard error (spec tolerance)."""
    from compfinance_gb300 import workloads as W
    s, t, v = W.dupire_surface(*grid)
    u = W.UOC_BARRIER
    mid = f"eq{grid[0]}"
    eng.putDupire(W.DUPIRE_SPOT, s, t, v, W.DUPIRE_MAXDT, mid)
    eng.putBarrier(u["strike"], u["barrier"], u["maturity"], u["monitor_freq"], u["smooth"], 0, "equoc")
    n = 1 << 18
    # standard error of each risk at n paths, from 8 independent seed pairs at n/4 paths
    rs = np.array([eng.AADriskOne(mid, "equoc", num(0, n // 4, "fp64", 1000 + k, 77 + k))["risks"]
                   for k in range(8)])
    se = rs.std(axis=0, ddof=1) / 2.0
    for seeds in ((12345, 1234), (1001, 78), (4242, 99)):
        r64 = eng.AADriskOne(mid, "equoc", num(0, n, "fp64", *seeds))
        r32 = eng.AADriskOne(mid, "equoc", num(0, n, "fp32", *seeds))
        v64 = eng.value(mid, "equoc", num(0, n, "fp64", *seeds))
        assert np.all(np.abs(r32["payoffValues"] - r64["payoffValues"]) <= 0.1 * v64["stderrs"])
        mask = se > 1e-6 * np.abs(r64["risks"]).max()
        assert np.all(np.abs(r32["risks"] - r64["risks"])[mask] <= 0.1 * se[mask])
        # nodes with no measurable variance must agree to FP32 rounding
        assert np.all(np.abs(r32["risks"] - r64["risks"])[~mask] <= 1e-6 * np.abs(r64["risks"]).max())


def _se_fp64(eng, mid, pid, n):
    """Standard error of each risk at n paths, from 8 independent mrg32k3a seed pairs at n/4."""
    rs = np.array([eng.AADriskOne(mid, pid, num(0, n // 4, "fp64", 1000 + k, 77 + k))["risks"] for k in range(8)])
    return rs.std(axis=0, ddof=1) / 2.0


@pytest.mark.parametrize("prod", ["uoc", "european"])
@pytest.mark.parametrize("sobol", [0, 1])
def test_fp32_risk_kernel_variants_within_tenth_of_stderr(eng, prod, sobol):
    """Every variant of the FP32 Dupire risk kernel (barrier or European payoff, mrg32k3a or
    Sobol draws) against the FP64 form on the same paths: prices and risks within 0.1 Monte
    Carlo standard error."""
    from compfinance_gb300 import workloads as W
    s, t, v = W.dupire_surface(60, 30)
    u = W.UOC_BARRIER
    eng.putDupire(W.DUPIRE_SPOT, s, t, v, W.DUPIRE_MAXDT, "var60")
    if prod == "uoc":
        eng.putBarrier(u["strike"], u["barrier"], u["maturity"], u["monitor_freq"], u["smooth"], 0, "var_p")
    else:
        eng.putEuropean(110.0, 2.0, 2.0, "var_p")
    n = 1 << 17
    se = _se_fp64(eng, "var60", "var_p", n)
    r64 = eng.AADriskOne("var60", "var_p", num(sobol, n, "fp64"))
    r32 = eng.AADriskOne("var60", "var_p", num(sobol, n, "fp32"))
    v64 = eng.value("var60", "var_p", num(0, n, "fp64"))
    assert np.all(np.abs(r32["payoffValues"] - r64["payoffValues"]) <= 0.1 * v64["stderrs"])
    mask = se > 1e-6 * np.abs(r64["risks"]).max()
    assert mask.sum() > 50
    assert np.all(np.abs(r32["risks"] - r64["risks"])[mask] <= 0.1 * se[mask])
    assert np.all(np.abs(r32["risks"] - r64["risks"])[~mask] <= 1e-6 * np.abs(r64["risks"]).max())


def test_fp32_risk_kernel_agrees_with_generic_kernel(eng, monkeypatch):
    """The specialised FP32 Dupire risk kernel and the generic FP32 kernel (CF_FAST32=0)
    compute the same paths with different roundings: both within 0.1 standard error."""
    from compfinance_gb300 import workloads as W
    s, t, v = W.dupire_surface(60, 30)
    u = W.UOC_BARRIER
    eng.putDupire(W.DUPIRE_SPOT, s, t, v, W.DUPIRE_MAXDT, "gen60")
    eng.putBarrier(u["strike"], u["barrier"], u["maturity"], u["monitor_freq"], u["smooth"], 0, "gen_uoc")
    n = 1 << 17
    se = _se_fp64(eng, "gen60", "gen_uoc", n)
    fast = eng.AADriskOne("gen60", "gen_uoc", num(0, n, "fp32"))
    monkeypatch.setenv("CF_FAST32", "0")
    generic = eng.AADriskOne("gen60", "gen_uoc", num(0, n, "fp32"))
    monkeypatch.delenv("CF_FAST32")
    mask = se > 1e-6 * np.abs(generic["risks"]).max()
    assert np.all(np.abs(fast["risks"] - generic["risks"])[mask] <= 0.1 * se[mask])
    assert abs(fast["payoffValues"][0] - generic["payoffValues"][0]) <= 1e-5 * abs(generic["payoffValues"][0])


def test_fp32_risk_kernel_small_and_odd_path_counts(mc_eng):
    """Partial units, partial warps and partial blocks of the FP32 risk kernel: FP32 against
    FP64 on the same few paths, within FP32 rounding of the path arithmetic."""
    eng, d = mc_eng
    for n in (1, 2, 3, 31, 33, 257, 1001):
        for sob in (0, 1):
            r64 = eng.AADriskOne("dup60x30", "uoc", num(sob, n, "fp64"))
            r32 = eng.AADriskOne("dup60x30", "uoc", num(sob, n, "fp32"))
            scale = max(np.abs(r64["risks"]).max(), 1e-3)
            assert np.abs(r32["risks"] - r64["risks"]).max() <= 5e-3 * scale, (n, sob)
            assert abs(r32["payoffValues"][0] - r64["payoffValues"][0]) <= 1e-3 * max(abs(r64["payoffValues"][0]), 1e-3)


@pytest.mark.parametrize("steps", [1, 2, 3])
@pytest.mark.parametrize("prod", ["uoc", "european"])
def test_fp32_risk_kernel_short_timelines(eng, steps, prod):
    """Timelines of one to three steps (the reverse sweep's loads run ahead of the step it
    computes): FP32 against FP64 on the same paths, within FP32 rounding of the path
    arithmetic."""
    from compfinance_gb300 import workloads as W
    s, t, v = W.dupire_surface(60, 30)
    eng.putDupire(W.DUPIRE_SPOT, s, t, v, W.DUPIRE_MAXDT, "short60")
    T = (steps - 0.5) * W.DUPIRE_MAXDT
    if prod == "uoc":
        eng.putBarrier(100.0, 104.0, T, T / steps, 0.01, 0, "short_p")
    else:
        eng.putEuropean(100.0, T, T, "short_p")
    assert eng.shapes("short60", "short_p")[2] == steps
    for sob in (0, 1):
        r64 = eng.AADriskOne("short60", "short_p", num(sob, 4096, "fp64"))
        r32 = eng.AADriskOne("short60", "short_p", num(sob, 4096, "fp32"))
        scale = max(np.abs(r64["risks"]).max(), 1e-3)
        assert np.abs(r64["risks"]).max() > 0
        assert np.abs(r32["risks"] - r64["risks"]).max() <= 5e-3 * scale, (steps, prod, sob)
        assert abs(r32["payoffValues"][0] - r64["payoffValues"][0]) <= 1e-3 * max(abs(r64["payoffValues"][0]), 1e-3)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_tma_staged_local_vols_bit_identical(eng, monkeypatch, precision):
    """The generic kernel's local-vol table staged into shared memory by a TMA bulk copy
    (cp.async.bulk with an mbarrier, forced by CF_STAGE_Y=1) and read through L1 instead
    (CF_STAGE_Y=0): the same numbers bit for bit, and no device error flag (the bounded wait
    on the copy did not run out).  CF_FAST32=0 keeps FP32 risk on the generic kernel."""
    from compfinance_gb300 import workloads as W
    s, t, v = W.dupire_surface(60, 30)
    u = W.UOC_BARRIER
    eng.putDupire(W.DUPIRE_SPOT, s, t, v, W.DUPIRE_MAXDT, "tma60")
    eng.putBarrier(u["strike"], u["barrier"], u["maturity"], u["monitor_freq"], u["smooth"], 0, "tma_p")
    monkeypatch.setenv("CF_FAST32", "0")
    out = {}
    for stage in ("1", "0"):
        monkeypatch.setenv("CF_STAGE_Y", stage)
        out[stage] = eng.AADriskOne("tma60", "tma_p", num(0, 1 << 15, precision))
    assert np.array_equal(out["1"]["payoffValues"], out["0"]["payoffValues"])
    assert np.array_equal(out["1"]["risks"], out["0"]["risks"])
    assert np.abs(out["1"]["risks"]).max() > 0


@pytest.mark.parametrize("case", [("bs", "euro", 1), ("bs_rates", "euro_settle", 0), ("dup20x10", "uoc", 0),
                                  ("dup20x10", "uoc", 1), ("dup60x30_monthly", "europeans", 1),
                                  ("bs", "uoc", 0)])
def test_simulate_paths_vs_oracle(mc_eng, case):
    """mcSimul's payoff matrix (every path's payoffs, mcBase.h:267-308) against the oracle's
    per-path payoffs on the same random numbers: FP64 to 1e-12 of the largest payoff, path by
    path; the path averages equal the valuation entry point's; the FP32 form within FP32
    rounding of the path arithmetic, path by path."""
    eng, d = mc_eng
    mid, pid, sob = case
    n = 2049  # an odd count: the last antithetic pair has one path
    got = eng.simulatePaths(mid, pid, num(sob, n))
    ref = O.paths(O.Model(d["models"][mid]), O.Product(d["products"][pid]), sob, n).reshape(got.shape)
    assert got.shape == (n, eng.shapes(mid, pid)[0])
    assert rel_to_max(got, ref) < TOL
    v = eng.value(mid, pid, num(sob, n))["values"]
    assert np.abs(got.mean(axis=0) - v).max() <= 1e-13 * np.abs(v).max()
    g32 = eng.simulatePaths(mid, pid, num(sob, n, "fp32"))
    assert np.abs(g32 - ref).max() <= 5e-4 * np.abs(ref).max()


def test_c2_risk_at_full_size_vs_reference(eng, golden):
    """The 60x30 barrier's AADriskOne at its configured 2^18 mrg32k3a paths against the
    reference's own run (value and all 1801 risks): FP64 to 1e-12; the FP32 form within 0.1
    Monte Carlo standard error of the reference (standard errors from 8 independent runs of a
    quarter of the paths)."""
    d = golden("mc")
    c = golden("baseline")["c2"]
    put_model(eng, "c2full", d["models"][c["model"]])
    put_product(eng, "c2uoc", d["products"][c["product"]])
    r64 = eng.AADriskOne("c2full", "c2uoc", num(0, c["npath"]))
    assert rel_to_max(r64["payoffValues"], c["values"]) < TOL
    assert abs(r64["riskPayoffValue"] - c["risk_value"]) <= TOL * abs(c["risk_value"])
    assert rel_to_max(r64["risks"], c["risks"]) < TOL
    runs = np.array([eng.AADriskOne("c2full", "c2uoc", num(0, c["npath"] // 4, "fp64", 500 + k, 60 + k))["risks"]
                     for k in range(8)])
    se = runs.std(axis=0, ddof=1) / 2.0
    vse = eng.value("c2full", "c2uoc", num(0, c["npath"]))["stderrs"][0]
    r32 = eng.AADriskOne("c2full", "c2uoc", num(0, c["npath"], "fp32"))
    assert abs(r32["payoffValues"][0] - c["values"][0]) <= 0.1 * vse
    ref = np.array(c["risks"])
    mask = se > 1e-6 * np.abs(ref).max()
    assert np.all(np.abs(r32["risks"] - ref)[mask] <= 0.1 * se[mask])
    assert np.all(np.abs(r32["risks"] - ref)[~mask] <= 1e-6 * np.abs(ref).max())


@pytest.mark.parametrize("grid", [(20, 10), (60, 30), (120, 60)])
def test_fp32_risk_rows_staged_bit_identical(eng, monkeypatch, grid):
    """The FP32 risk kernel with its forward's local-vol rows staged into shared memory by bulk
    copies (CF_ROW_CHUNK = 2, 4, 8 steps per copy, two buffers) and read through L1 (0): the same
    numbers bit for bit, for the barrier (156 weekly steps, a multiple of every chunk, and 155,
    whose last chunk is short) and the European, both generators, with a partial last round of
    units; no device error flag (every bounded wait on a copy completed)."""
    from compfinance_gb300 import workloads as W
    s, t, v = W.dupire_surface(*grid)
    u = W.UOC_BARRIER
    name = f"rows{grid[0]}"
    eng.putDupire(W.DUPIRE_SPOT, s, t, v, W.DUPIRE_MAXDT, name)
    eng.putBarrier(u["strike"], u["barrier"], u["maturity"], u["monitor_freq"], u["smooth"], 0, "rows_uoc156")
    T155 = 155 * u["monitor_freq"]
    eng.putBarrier(u["strike"], u["barrier"], T155, u["monitor_freq"], u["smooth"], 0, "rows_uoc155")
    eng.putEuropean(110.0, 3.0, 3.0, "rows_eu")
    assert eng.shapes(name, "rows_uoc155")[2] == 155
    for prod in ("rows_uoc156", "rows_uoc155", "rows_eu"):
        for sob in (0, 1):
            out = {}
            for k in ("0", "2", "4", "8"):
                monkeypatch.setenv("CF_ROW_CHUNK", k)
                out[k] = eng.AADriskOne(name, prod, num(sob, (1 << 16) + 4001, "fp32"))
            assert np.abs(out["0"]["risks"]).max() > 0
            for k in ("2", "4", "8"):
                assert np.array_equal(out[k]["payoffValues"], out["0"]["payoffValues"]), (prod, sob, k)
                assert np.array_equal(out[k]["risks"], out["0"]["risks"]), (prod, sob, k)


@pytest.mark.parametrize("prod", ["uoc", "european"])
def test_fp32_risk_kernel_one_spot_knot(eng, prod):
    """A local vol flat in spot (one spot knot, 30 times): the FP32 risk kernel against FP64 on
    the same paths, within FP32 rounding of the path arithmetic."""
    from compfinance_gb300 import workloads as W
    s, t, v = W.dupire_surface(60, 30)
    vols = np.asarray(v).reshape(len(s), len(t))[30:31, :]  # the row of spot ~100, [1][nT]
    eng.putDupire(W.DUPIRE_SPOT, np.array([100.0]), t, vols, W.DUPIRE_MAXDT, "flat1")
    u = W.UOC_BARRIER
    if prod == "uoc":
        eng.putBarrier(u["strike"], u["barrier"], u["maturity"], u["monitor_freq"], u["smooth"], 0, "flat_p")
    else:
        eng.putEuropean(110.0, 2.0, 2.0, "flat_p")
    assert eng.shapes("flat1", "flat_p")[1] == 1 + len(t)
    for sob in (0, 1):
        r64 = eng.AADriskOne("flat1", "flat_p", num(sob, 1 << 14, "fp64"))
        r32 = eng.AADriskOne("flat1", "flat_p", num(sob, 1 << 14, "fp32"))
        scale = np.abs(r64["risks"]).max()
        assert scale > 0
        assert np.abs(r32["risks"] - r64["risks"]).max() <= 5e-3 * scale, (prod, sob)
        assert abs(r32["payoffValues"][0] - r64["payoffValues"][0]) <= 1e-3 * max(abs(r64["payoffValues"][0]), 1e-3)
