"""Multi-asset displaced model with Baskets and Autocall on the GPU (mcMdlMultiDisplaced.h,
mcPrdMulti.h) against fixtures written by the reference and against the oracle."""
import numpy as np
import pytest

import oracle as O
from compfinance_gb300 import CfError, Engine
from gpu_util import num, rel_to_max

pytestmark = pytest.mark.gpu

CASES = ["md4_bask4_sobol", "md4_bask4_mrg", "md4_ac4_sobol", "md4_ac4_mrg", "md4_ac4_sharp", "md2_bask2_sobol",
         "md2_ac2_mrg"]


@pytest.fixture(scope="module")
def eng():
    e = Engine(0)
    yield e
    e.close()


def put(eng, d, c):
    m = d["models"][c["model"]]
    eng.putDisplaced(m["assets"], m["spots"], m["atms"], m["skews"], m["disc"], m["spreads"], m["div_dates"],
                     m["divs"], m["correl"], m["lambda"], c["model"])
    p = d["products"][c["product"]]
    if p["kind"] == "baskets":
        eng.putBaskets(p["assets"], p["weights"], p["maturity"], p["strikes"], c["product"])
    else:
        eng.putAutocall(p["assets"], p["refs"], p["maturity"], p["periods"], p["ko"], p["strike"], p["cpn"],
                        p["smooth"], c["product"])


@pytest.fixture(scope="module")
def md(golden, eng):
    d = golden("multi_asset")
    for c in d["cases"]:
        put(eng, d, c)
    return d


def case(md, name):
    return [c for c in md["cases"] if c["name"] == name][0]


@pytest.mark.parametrize("name", CASES)
def test_labels_and_model_state(eng, md, name):
    """Labels, and the model after its initialisation (Cholesky factor, stds, drifts, dividend-
    adjusted forward factors, displacements, numeraires, dynamics) bit for bit."""
    c = case(md, name)
    assert eng.payoffLabels(c["product"]) == c["payoff_labels"]
    assert eng.parameterLabels(c["model"]) == c["param_labels"]
    s = eng.mdState(c["model"], c["product"])
    assert list(s["chol"].ravel()) == c["md_chol"]
    assert list(s["stds"].ravel()) == c["md_stds"] and list(s["drifts"].ravel()) == c["md_drifts"]
    assert list(s["ffs"].ravel()) == c["md_ffs"] and list(s["alphas"]) == c["md_alphas"]
    assert list(s["numeraires"]) == c["md_numeraires"] and list(s["dynamics"]) == [int(x) for x in c["md_dynamics"]]
    _, _, dim = eng.shapes(c["model"], c["product"])
    assert dim == (len(c["sim_timeline"]) - 1) * len(md["models"][c["model"]]["assets"])


@pytest.mark.parametrize("name", CASES)
def test_value_and_risks_vs_reference(eng, md, name):
    """FP64: values within 1e-13, AADriskOne / AADriskAggregate / AADriskMulti within 1e-12 of
    the largest risk of the reference's own run (same paths, exact path sums)."""
    c = case(md, name)
    n = num(c["sobol"], c["npath"])
    v = eng.value(c["model"], c["product"], n)["values"]
    assert rel_to_max(v, c["values"]) < 1e-13
    labels = eng.payoffLabels(c["product"])
    r = eng.AADriskOne(c["model"], c["product"], n, labels[0])
    assert abs(r["riskPayoffValue"] - c["risk_value"]) <= 1e-13 * abs(c["risk_value"])
    assert rel_to_max(r["risks"], c["risks"]) < 1e-12
    a = eng.AADriskAggregate(c["model"], c["product"], dict(zip(labels, c["agg_weights"])), n)
    assert abs(a["riskPayoffValue"] - c["agg_value"]) <= 1e-13 * abs(c["agg_value"])
    assert rel_to_max(a["risks"], c["agg_risks"]) < 1e-12
    m = eng.AADriskMulti(c["model"], c["product"], n)
    ref = np.array(c["multi_risks"]).reshape(m["risks"].shape)
    assert rel_to_max(m["risks"], ref) < 1e-12


@pytest.mark.parametrize("name", ["md4_bask4_sobol", "md4_ac4_mrg", "md2_ac2_mrg"])
def test_bump_risk_vs_reference(eng, md, name):
    """bumpRisk (main.h:316-359): one-sided 1e-8 bumps repriced on the same paths; the difference
    of two exact path sums is scaled by 1e8, so rounding of the sums (~1e-16 of the value) shows
    at ~1e-8 of the value."""
    c = case(md, name)
    r = eng.bumpRisk(c["model"], c["product"], num(c["sobol"], c["bump_npath"]))
    ref = np.array(c["bump_risks"]).reshape(r["risks"].shape)
    v = np.abs(np.array(c["values"])).max()
    assert np.abs(r["risks"] - ref).max() <= 1e-5 * np.abs(ref).max() + 1e-6 * v


@pytest.mark.parametrize("name", ["md4_bask4_mrg", "md4_ac4_sobol"])
def test_fp32_vs_fp64(eng, md, name):
    """FP32 paths vs FP64 on the same random numbers: values and risks within 0.1 Monte Carlo
    standard error (standard errors from 8 independent mrg32k3a runs of a quarter size)."""
    c = case(md, name)
    n = 1 << 16
    labels = eng.payoffLabels(c["product"])
    runs = np.array([eng.AADriskOne(c["model"], c["product"], num(0, n // 4, "fp64", 7000 + k, 31 + k), labels[0])
                     ["risks"] for k in range(8)])
    se = runs.std(axis=0, ddof=1) / 2.0
    r64 = eng.AADriskOne(c["model"], c["product"], num(c["sobol"], n), labels[0])
    r32 = eng.AADriskOne(c["model"], c["product"], num(c["sobol"], n, "fp32"), labels[0])
    vse = eng.value(c["model"], c["product"], num(0, n))["stderrs"]
    assert np.all(np.abs(r32["payoffValues"] - r64["payoffValues"]) <= 0.1 * vse)
    mask = se > 1e-6 * np.abs(r64["risks"]).max()
    assert np.all(np.abs(r32["risks"] - r64["risks"])[mask] <= 0.1 * se[mask])


@pytest.mark.parametrize("sob,npath", [(0, 1), (0, 333), (1, 1), (1, 95), (1, 4096)])
def test_vs_oracle_odd_sizes(eng, md, sob, npath):
    """Partly filled antithetic pairs and Sobol warp batches: values and risks of the oracle."""
    c = case(md, "md4_ac4_sobol")
    m, p = O.MModel(md["models"][c["model"]]), O.MProduct(md["products"][c["product"]])
    v, _ = O.m_value(m, p, sob, npath)
    assert rel_to_max(eng.value(c["model"], c["product"], num(sob, npath))["values"], v) < 1e-13
    _, agg, r = O.m_risk(m, p, sob, npath, [1.0])
    g = eng.AADriskOne(c["model"], c["product"], num(sob, npath))
    assert abs(g["riskPayoffValue"] - agg) <= 1e-13 * max(abs(agg), 1e-300)
    assert rel_to_max(g["risks"], r) < 1e-12


def test_incompatible_model_and_product(eng, md):
    """checkCompatiblity (mcBase.h:253-259): the asset names must agree."""
    with pytest.raises(CfError, match="not compatible"):
        eng.value("md2", "bask4", num(1, 64))
    eng.putBlackScholes(100.0, 0.2, 0, 0.02, 0.0, "bs_single")
    with pytest.raises(CfError, match="not compatible"):
        eng.value("bs_single", "ac2", num(1, 64))
