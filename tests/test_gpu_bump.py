"""bumpRisk (main.h:316-359) on the GPU against the reference's own bumpRisk (tests/golden/
bump.json, made by running the reference): every model parameter bumped by 1e-8 and repriced
on the same random numbers.  The reference's finite differences amplify the last-bit rounding
of two path averages by 1e8, so the parity bound is 1e-5 of the largest risk.  Both procedures
of the engine (full repricing of each bumped model, and pathwise re-simulation of the paths a
bumped local-vol node touches) give the same numbers."""
import numpy as np
import pytest

from compfinance_gb300 import Engine
from gpu_util import num, put_model, put_product, rel_to_max

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def bump_eng(golden):
    d = golden("bump")
    e = Engine(0)
    for mid, spec in d["models"].items():
        put_model(e, mid, spec)
    for pid, spec in d["products"].items():
        put_product(e, pid, spec)
    yield e, d
    e.close()


def test_bump_risk_reprice_matches_reference(bump_eng):
    eng, d = bump_eng
    worst = {}
    for c in d["cases"]:
        r = eng.bumpRisk(c["model"], c["product"], num(c["sobol"], c["npath"]), method="reprice")
        ref = np.array(c["risks"]).reshape(c["shape"])
        assert r["risks"].shape == tuple(c["shape"])
        assert rel_to_max(r["values"], c["values"]) < 1e-12, c["name"]
        worst[c["name"]] = rel_to_max(r["risks"], ref)
    print(worst)
    assert max(worst.values()) < 1e-5, worst


def test_bump_risk_pathwise_matches_reference(bump_eng):
    """The pathwise procedure (re-simulating only the paths a bumped local-vol node touches)
    against the reference's bumpRisk on every Dupire case."""
    eng, d = bump_eng
    worst = {}
    for c in d["cases"]:
        if d["models"][c["model"]]["kind"] != "dupire":
            continue
        r = eng.bumpRisk(c["model"], c["product"], num(c["sobol"], c["npath"]), method="pathwise")
        ref = np.array(c["risks"]).reshape(c["shape"])
        assert rel_to_max(r["values"], c["values"]) < 1e-12, c["name"]
        worst[c["name"]] = rel_to_max(r["risks"], ref)
    print(worst)
    assert max(worst.values()) < 1e-5, worst


@pytest.mark.parametrize("case", [("dup60x30", "uoc", 0, 1 << 12), ("dup60x30_monthly", "europeans", 1, 1 << 11),
                                  ("dup20x10", "euro_settle", 0, 1 << 12)])
def test_bump_risk_pathwise_equals_reprice(bump_eng, case):
    """Both procedures compute the same finite differences on the same paths (they differ only
    in the last-bit rounding of the repriced averages, amplified by 1e8)."""
    import time
    eng, d = bump_eng
    mid, pid, sob, n = case
    t0 = time.perf_counter()
    a = eng.bumpRisk(mid, pid, num(sob, n), method="reprice")
    t1 = time.perf_counter()
    b = eng.bumpRisk(mid, pid, num(sob, n), method="pathwise")
    t2 = time.perf_counter()
    print(case, "reprice", t1 - t0, "s, pathwise", t2 - t1, "s", rel_to_max(b["risks"], a["risks"]))
    assert np.array_equal(a["values"], b["values"]) or rel_to_max(b["values"], a["values"]) < 1e-15
    assert rel_to_max(b["risks"], a["risks"]) < 1e-5
    # the default procedure is the pathwise one for Dupire models
    auto = eng.bumpRisk(mid, pid, num(sob, n))
    assert np.array_equal(auto["risks"], b["risks"])


def test_superbucket_bump_matches_reference(bump_eng, golden):
    """dupireSuperbucketBump (main.h:575-696) against the reference's own.

    * value and delta: on the same calibrated local vols, like the reference's;
    * vega by the reference's 1e-5 bumps: such a bump moves the local vols less than the rounding
      noise of Dupire's formula (a second price difference divided by 1e-8), so the reference's
      numbers are that noise and only their structure is reproducible: risk-view nodes that
      cannot reach the calibrated grid give exactly zero in both;
    * the bumping itself, with 5e-4 bumps (above the noise floor): against the reference's AAD
      superbucket of the same case (tests/golden/calib.json, sb_merton)."""
    eng, _ = bump_eng
    c = golden("bump")["superbucket_bump"]
    iv = Engine.ivs("merton", c["ivs_params"][0], c["ivs_params"][1:])
    eng.putEuropeans(c["portfolio"]["mats"], c["portfolio"]["strikes"], "sbbport")
    w = np.zeros(len(c["portfolio"]["mats"]))
    for k, x in c["notionals"]:
        w[k] = x
    args = (iv, c["ivs_params"][0], c["maxdt"], "sbbport", w, c["incl_spots"], c["max_ds"], c["incl_times"],
            c["max_dt_vol"], c["rv_strikes"], c["rv_mats"], num(1, c["npath"]))
    r = eng.dupireSuperbucketBump(*args)
    ref = np.array(c["vega"]).reshape(len(c["rv_strikes"]), len(c["rv_mats"]))
    print("value", r["value"] - c["value"], "delta", r["delta"] - c["delta"])
    assert abs(r["value"] - c["value"]) < 1e-4 * abs(c["value"])
    assert abs(r["delta"] - c["delta"]) < 1e-3 * abs(c["delta"])
    assert np.array_equal(r["vega"] == 0.0, ref == 0.0)
    aad = [s for s in golden("calib")["superbucket"] if s["name"] == "sb_merton"][0]
    assert aad["incl_spots"] == c["incl_spots"] and aad["notionals"] == c["notionals"]
    ref_aad = np.array(aad["vega"]).reshape(ref.shape)
    wide = eng.dupireSuperbucketBump(*args, vegaBump=5e-4)
    print("5e-4 bumps vs the reference's AAD vega", rel_to_max(wide["vega"], ref_aad))
    assert rel_to_max(wide["vega"], ref_aad) < 0.1
