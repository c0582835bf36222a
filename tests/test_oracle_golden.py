"""The CPU restatement (oracle/) against golden vectors written by the reference itself.

These pin the oracle before it is trusted as the checker of the CUDA engine.
"""
import numpy as np
import pytest

import oracle as O
from calib_util import support


def rel(a, b):
    a = np.asarray(a, dtype=float).ravel()
    b = np.asarray(b, dtype=float).ravel()
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def test_sobol_direction_table(golden):
    # Per-dimension FNV-1a hash of the 32 direction numbers (sobol.cpp), regenerated here
    # from the Joe-Kuo initialisation data.
    g = golden("rng")
    dims = len(g["sobol_dirhash"])
    ints = O.sobol_ints(dims, 0, 1)  # smoke: first point is 2^31 everywhere
    assert (ints[0] == 1 << 31).all()
    # The point of index b = 2^(i+1) - 1 has gray(b) = 2^i, so its state is direction number i.
    tab = np.zeros((32, dims), dtype=np.uint64)
    for i in range(32):
        b = (1 << (i + 1)) - 1
        tab[i] = O.sobol_ints(dims, b - 1, 1)[0]
    h = np.full(dims, 1469598103934665603, dtype=np.uint64)
    prime = np.uint64(1099511628211)
    with np.errstate(over="ignore"):
        for i in range(32):
            for k in range(4):
                h ^= (tab[i] >> np.uint64(8 * k)) & np.uint64(0xFF)
                h *= prime
    assert ((h & np.uint64(0xFFFFFFFFFFFF)).astype(np.int64) == np.array(g["sobol_dirhash"])).all()


def test_sobol_points(golden):
    g = golden("rng")
    got = O.sobol_ints(1101, 0, 3)
    assert (got == np.array(g["sobol_1101"], dtype=np.uint32)).all()
    got = O.sobol_ints(8, 0, 300)
    assert (got == np.array(g["sobol_8"], dtype=np.uint32)).all()
    for c in g["sobol_skip"]:
        got = O.sobol_ints(c["dim"], c["b"], 1)[0]
        assert (got == np.array(c["ints"], dtype=np.uint32)).all(), c["b"]
        gg = O.sobol_gauss(c["dim"], c["b"], 1)[0]
        assert (gg == np.array(c["g"])).all(), c["b"]


def test_mrg_states_and_gaussians(golden):
    g = golden("rng")
    for c in g["mrg_skip"]:
        st = O.mrg_state(c["seed1"], c["seed2"], c["dim"], c["b"])
        assert list(st) == c["state"], c["b"]
    seq = [s for s in g["mrg_seq"] if s["kind"] == "g"][0]
    got = O.mrg_gauss(seq["seed1"], seq["seed2"], seq["dim"], 0, len(seq["seq"]))
    for i, rec in enumerate(seq["seq"]):
        assert (got[i] == np.array(rec["v"])).all()


def test_gaussian_functions(golden):
    g = golden("rng")
    for p, y in zip(g["invnorm"]["p"], g["invnorm"]["y"]):
        assert O.inv_normal_cdf(p) == y
    for x, y in zip(g["normcdf"]["x"], g["normcdf"]["y"]):
        assert O.normal_cdf(x) == y


def test_fill_data(golden):
    for c in golden("host")["fill"]:
        got = O.fill(c["x"], c["maxdx"], c["mindx"], c["add"])
        assert list(got) == c["out"]


@pytest.fixture(scope="module")
def mc(golden):
    d = golden("mc")
    models = {k: O.Model(v) for k, v in d["models"].items()}
    prods = {k: O.Product(v) for k, v in d["products"].items()}
    return d, models, prods


def _weights(c, npay):
    w = np.zeros(npay)
    if c["mode"] == "risk":
        w[c["payoff"]] = 1.0
    else:
        for k, x in c["notionals"]:
            w[k] = x
    return w


def test_mc_cases(mc):
    d, models, prods = mc
    for c in d["cases"]:
        m, p = models[c["model"]], prods[c["product"]]
        npay, npar, _ = O.shapes(m, p)
        if c["mode"] == "value":
            if c["npath"] > 20000:
                continue  # covered by the threaded test below
            v, _ = O.value(m, p, c["sobol"], c["npath"])
            assert rel(v, c["values"]) == 0.0, c["name"]
        elif c["mode"] in ("risk", "agg"):
            v, agg, r = O.risk(m, p, c["sobol"], c["npath"], _weights(c, npay))
            assert rel(v, c["values"]) == 0.0, c["name"]
            assert agg == pytest.approx(c["risk_value"], rel=1e-15, abs=0), c["name"]
            assert rel(r, c["risks"]) < 1e-14, c["name"]
            if m.spec["kind"] == "dupire":
                v2, agg2, r2 = O.risk(m, p, c["sobol"], c["npath"], _weights(c, npay), fast=True, threads=3)
                assert rel(v2, c["values"]) < 1e-14 and rel(r2, c["risks"]) < 1e-13, c["name"]
        else:
            quirk = m.spec["kind"] == "dupire"
            v, r = O.risk_multi(m, p, c["sobol"], c["npath"], ref_quirk=quirk)
            assert rel(v, c["values"]) == 0.0, c["name"]
            if quirk:
                assert rel(r, c["risks"]) < 1e-14, c["name"]


def test_mc_value_threaded(mc):
    d, models, prods = mc
    c = [c for c in d["cases"] if c["name"] == "c2_dup60x30_uoc_value"][0]
    v, e = O.value(models[c["model"]], prods[c["product"]], c["sobol"], c["npath"], threads=4)
    assert rel(v, c["values"]) < 1e-13


def test_multi_equals_per_payoff_risk(mc):
    # AADriskMulti of the reference re-propagates one tape node of its last path; the exact
    # path average must equal the per-payoff AADriskOne results of the reference.
    d, models, prods = mc
    cs = {c["name"]: c for c in d["cases"]}
    m, p = models["bs_spotmeasure"], prods["europeans"]
    v, r = O.risk_multi(m, p, 1, 1024)
    each = np.array([cs[f"bs_europeans_each_{k}"]["risks"] for k in range(12)]).T
    assert rel(r, each) < 1e-14


def test_calibration(golden):
    for c in golden("calib")["calib"]:
        iv = O.ivs(c["ivs"], c["ivs_params"][0], c["ivs_params"][1:])
        s, t, lv = O.calib(iv, c["incl_spots"], c["max_ds"], c["incl_times"], c["max_dt_vol"])
        assert list(s) == c["spots"] and list(t) == c["times"]
        assert rel(lv, c["lvols"]) == 0.0, c["name"]


def test_superbucket(golden):
    # Vega passes through the calibration's second strike difference (/1e-8), which
    # amplifies 1e-16 differences in the order of the Black-Scholes derivative chain:
    # agreement with the reference's tape is ~1e-6 of the largest vega.
    for c in golden("calib")["superbucket"]:
        iv = O.ivs(c["ivs"], c["ivs_params"][0], c["ivs_params"][1:])
        p = O.Product(dict(kind="europeans", mats=c["portfolio"]["mats"], strikes=c["portfolio"]["strikes"]))
        w = np.zeros(len(c["portfolio"]["mats"]))
        for k, x in c["notionals"]:
            w[k] = x
        v, dlt, vega, mb = O.superbucket(iv, 100.0, c["maxdt"], p, w, c["incl_spots"], c["max_ds"],
                                         c["incl_times"], c["max_dt_vol"], c["rv_strikes"], c["rv_mats"],
                                         1, c["npath"], ref_quirk=True)
        assert v == pytest.approx(c["value"], rel=1e-14) and dlt == pytest.approx(c["delta"], rel=1e-13)
        if "microbucket" in c:
            assert rel(mb, c["microbucket"]) < 1e-13
        assert rel(vega, c["vega"]) < 2e-5, c["name"]


def test_calibration_adjoint_pointwise(golden):
    """The pointwise restatement of the calibration adjoint (each call one tape node of its implied
    vol, with value and partial): at given values equal to its own, bit for bit what it computes
    alone; against the full tape adjoint, to rounding of the terms it sums (each vega entry is a
    sum of terms up to ~5e10 times the largest entry, which cancel); against the reference's
    superbucket vega on the reference's microbucket, within the same rounding."""
    for c in golden("calib")["superbucket"]:
        iv = O.ivs(c["ivs"], c["ivs_params"][0], c["ivs_params"][1:])
        grid = (c["incl_spots"], c["max_ds"], c["incl_times"], c["max_dt_vol"])
        s, t, _ = O.calib(iv, *grid)
        micro = np.random.RandomState(3).standard_normal(len(s) * len(t))
        for q in (False, True):
            v0 = O.calib_adjoint(iv, *grid, c["rv_strikes"], c["rv_mats"], micro, ref_quirk=q)
            r1 = O.calib_adjoint_given(iv, *grid, c["rv_strikes"], c["rv_mats"], micro, ref_quirk=q)
            r2 = O.calib_adjoint_given(iv, *grid, c["rv_strikes"], c["rv_mats"], micro, calls=r1["calls"],
                                       vegas=r1["vegas"], ref_quirk=q)
            assert np.array_equal(r1["vega"], r2["vega"]), c["name"]
            assert np.all(np.abs(r1["vega"] - v0) <= 1e-13 * r1["absTerms"]), c["name"]
            assert (r1["calls"] > 0).any() and (r1["vegas"] > 0).any()
        if "microbucket" in c:
            r = O.calib_adjoint_given(iv, *grid, c["rv_strikes"], c["rv_mats"], c["microbucket"], ref_quirk=True)
            ref = np.array(c["vega"]).reshape(r["vega"].shape)
            assert np.all(np.abs(r["vega"] - ref) <= 1e-13 * r["absTerms"]), c["name"]


def test_calibration_adjoint_pointwise_c4(golden):
    """The same restatement on the superbucket workload (60x30 local vols, 30x12 risk view), seeded
    with the reference's microbucket at 2^20 paths, against the reference's vega: within rounding
    of the terms and of the risk view's interpolation weights (a calibration time one ulp below a
    risk-view maturity gives a corner weight of 0 exactly or ~1e-16, on point adjoints ~1e11)."""
    c = golden("baseline")["c4"]
    iv = O.ivs(c["ivs"], c["ivs_params"][0], c["ivs_params"][1:])
    grid = (c["incl_spots"], c["max_ds"], c["incl_times"], c["max_dt_vol"])
    s, t, _ = O.calib(iv, *grid)
    r = O.calib_adjoint_given(iv, *grid, c["rv_strikes"], c["rv_mats"], c["microbucket"], ref_quirk=True)
    ref = np.array(c["vega"]).reshape(r["vega"].shape)
    bound = 1e-13 * r["absTerms"] + 1e-15 * support(s, t, c["rv_strikes"], c["rv_mats"], r["pointAdj"])
    assert np.all(np.abs(r["vega"] - ref) <= bound)
    assert rel(r["vega"], ref) < 1e-5


def test_contingent_bond(golden):
    """The contingent bond (mcPrd.h:404-574) in the restatement against the reference: values
    and tape risks (rates through the libors and numeraires on Black-Scholes)."""
    d = golden("products")
    for c in d["cases"]:
        m, p = O.Model(d["models"][c["model"]]), O.Product(d["products"][c["product"]])
        v, _ = O.value(m, p, c["sobol"], c["npath"])
        assert rel(v, c["values"]) < 1e-13, c["name"]
        vv, agg, r = O.risk(m, p, c["sobol"], c["npath"], np.array([1.0]))
        assert rel(r, c["risks"]) < 1e-12, c["name"]


def _md(golden, name):
    d = golden("multi_asset")
    c = [x for x in d["cases"] if x["name"] == name][0]
    return c, O.MModel(d["models"][c["model"]]), O.MProduct(d["products"][c["product"]])


@pytest.mark.parametrize("name", ["md4_bask4_sobol", "md4_bask4_mrg", "md4_ac4_sobol", "md4_ac4_mrg",
                                  "md4_ac4_sharp", "md2_bask2_sobol", "md2_ac2_mrg"])
def test_multi_asset(golden, name):
    """Multi-asset displaced model with Baskets / Autocall (mcMdlMultiDisplaced.h, mcPrdMulti.h):
    the initialised model (Cholesky factor, stds, drifts, dividend-adjusted forward factors,
    displacements, numeraires) and the values bit for bit; AADriskOne, AADriskAggregate and
    AADriskMulti within 1e-12 of the largest risk (the tape orders the same operations
    differently)."""
    c, m, p = _md(golden, name)
    chol, stds, drifts, ffs, alphas, dyn, nums = O.m_init(m, p)
    assert list(chol.ravel()) == c["md_chol"]
    assert list(stds.ravel()) == c["md_stds"] and list(drifts.ravel()) == c["md_drifts"]
    assert list(ffs.ravel()) == c["md_ffs"] and list(alphas) == c["md_alphas"]
    assert list(dyn) == [int(x) for x in c["md_dynamics"]] and list(nums) == c["md_numeraires"]
    npay, npar, dim = O.m_shapes(m, p)
    assert npay == len(c["payoff_labels"]) and npar == len(c["param_labels"])
    assert dim == (len(c["sim_timeline"]) - 1) * len(m.spec["assets"])
    v, _ = O.m_value(m, p, c["sobol"], c["npath"])
    assert list(v) == c["values"]
    w = np.zeros(npay)
    w[0] = 1.0
    _, agg, r = O.m_risk(m, p, c["sobol"], c["npath"], w)
    assert agg == c["risk_value"]
    ref = np.array(c["risks"])
    assert np.abs(r - ref).max() <= 1e-12 * np.abs(ref).max()
    _, agg, r = O.m_risk(m, p, c["sobol"], c["npath"], c["agg_weights"])
    assert abs(agg - c["agg_value"]) <= 1e-13 * abs(c["agg_value"])
    ref = np.array(c["agg_risks"])
    assert np.abs(r - ref).max() <= 1e-12 * np.abs(ref).max()
    _, r = O.m_risk_multi(m, p, c["sobol"], c["npath"])
    ref = np.array(c["multi_risks"]).reshape(npar, npay)
    assert np.abs(r - ref).max() <= 1e-12 * np.abs(ref).max()
