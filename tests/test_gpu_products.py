"""The contingent bond (mcPrd.h:404-574) on the GPU against the reference's own value,
AADriskOne and bumpRisk (tests/golden/products.json, made by running the reference): Black-
Scholes under the risk-neutral and the spot measure (libors, numeraires, rate risk through
them) and Dupire (no rates); a sharp digital (smooth 0); the FP32 form within 0.1 Monte Carlo
standard error of the FP64 form."""
import numpy as np
import pytest

from compfinance_gb300 import Engine
from gpu_util import num, put_model, put_product, rel_to_max

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def peng(golden):
    d = golden("products")
    e = Engine(0)
    for mid, spec in d["models"].items():
        put_model(e, mid, spec)
    for pid, spec in d["products"].items():
        put_product(e, pid, spec)
    yield e, d
    e.close()


def test_contingent_labels(peng):
    eng, d = peng
    assert eng.payoffLabels("cbond") == ["contingent bond 3.00 0.02"]


def test_contingent_fp64_parity(peng):
    eng, d = peng
    worst = {}
    for c in d["cases"]:
        v = eng.value(c["model"], c["product"], num(c["sobol"], c["npath"]))
        r = eng.AADriskOne(c["model"], c["product"], num(c["sobol"], c["npath"]))
        assert rel_to_max(v["values"], c["values"]) < 1e-12, c["name"]
        assert abs(r["riskPayoffValue"] - c["risk_value"]) < 1e-12 * abs(c["risk_value"]), c["name"]
        worst[c["name"]] = rel_to_max(r["risks"], c["risks"])
    print(worst)
    assert max(worst.values()) < 1e-12, worst


def test_contingent_bump_risk(peng):
    # One-sided 1e-8 differences of a value near 1 carry about 1e8 x its last-bit rounding
    # (~1e-7) whatever the risk: the bound has that absolute part beside 1e-5 of the largest risk.
    eng, d = peng
    for c in d["cases"]:
        b = eng.bumpRisk(c["model"], c["product"], num(c["sobol"], c["bump_npath"]))
        ref = np.array(c["bump_risks"])
        tol = 1e-5 * np.abs(ref).max() + 2e-7 * abs(c["values"][0])
        assert np.abs(b["risks"][:, 0] - ref).max() <= tol, (c["name"], np.abs(b["risks"][:, 0] - ref).max(), tol)


def test_contingent_fp32_within_tenth_of_stderr(peng):
    eng, d = peng
    for mid in ("bs_rates", "dup20x10"):
        n = 1 << 16
        rs = np.array([eng.AADriskOne(mid, "cbond", num(0, n // 4, "fp64", 1000 + k, 77 + k))["risks"]
                       for k in range(8)])
        se = rs.std(axis=0, ddof=1) / 2.0
        r64 = eng.AADriskOne(mid, "cbond", num(0, n, "fp64"))
        r32 = eng.AADriskOne(mid, "cbond", num(0, n, "fp32"))
        v64 = eng.value(mid, "cbond", num(0, n, "fp64"))
        assert np.all(np.abs(r32["payoffValues"] - r64["payoffValues"]) <= 0.1 * v64["stderrs"] + 1e-6)
        mask = se > 1e-6 * np.abs(r64["risks"]).max()
        assert np.all(np.abs(r32["risks"] - r64["risks"])[mask] <= 0.1 * se[mask]), mid
