"""The C++ drop-in (include/cfgpu.hpp) driving the engine exactly like a caller of the
reference's main.h; results equal the Python binding's on the same inputs."""
import json
import os
import subprocess

import numpy as np
import pytest

from compfinance_gb300 import Engine, NumericalParam, library_path

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_cpp_dropin_program(tmp_path):
    exe = str(tmp_path / "dropin")
    lib = library_path()
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                           os.path.join(ROOT, "tests", "cpp", "dropin_main.cpp"), lib, "-o", exe,
                           "-Wl,-rpath," + os.path.dirname(lib)])
    out = json.loads(subprocess.check_output([exe]).decode())
    assert out["threw"] == 1 and out["nparams"] == 201 and out["multi_shape"] == [201, 3]
    eng = Engine(0)
    spots = [50.0 * 4.0 ** (i / 19.0) for i in range(20)]
    times = [0.1 + 2.9 * j / 9.0 for j in range(10)]
    vols = np.array([[0.15 + 0.10 * np.exp(-t) * np.log(s / 100.0) ** 2 for t in times] for s in spots])
    eng.putDupire(100.0, spots, times, vols, 0.25, "d")
    eng.putBarrier(120.0, 150.0, 3.0, 3.0 / 156.0, 0.01, 0, "u")
    r = eng.AADriskOne("d", "u", NumericalParam(numPath=1 << 14))
    assert out["label0"] == r["payoffIds"][0]
    assert out["risk_value"] == r["riskPayoffValue"]
    assert out["risk0"] == r["risks"][0] and out["risk5"] == r["risks"][5]
    # dupireAADRisk (main.h:364-411): the aggregate's value, spot risk and local-vol risks as a
    # [spots][times] matrix; a Black-Scholes model is refused like the reference refuses it
    agg = eng.AADriskAggregate("d", "u", {r["payoffIds"][0]: 1.0}, NumericalParam(numPath=1 << 14))
    assert out["dupire"] == [agg["riskPayoffValue"], agg["risks"][0], agg["risks"][1 + 3 * 10 + 4]]
    assert out["vega_shape"] == [20, 10] and out["not_dupire"] == 1
    dr = eng.dupireAADRisk("d", "u", {r["payoffIds"][0]: 1.0}, NumericalParam(numPath=1 << 14))
    assert dr["vega"].shape == (20, 10) and dr["vega"][3, 4] == agg["risks"][1 + 3 * 10 + 4]
    # bumpRisk (main.h:316-359) in the RiskReports layout
    br = eng.bumpRisk("d", "u", NumericalParam(numPath=1 << 14))
    assert out["bump_shape"] == [201, 2] and out["bump50"] == br["risks"][50, 0]
    # multi-asset store entries (store.h:75-94, 224-255) and the compatibility check
    md = out["md"]
    eng.putDisplaced(["X", "Y"], [100.0, 100.0], [0.2, 0.3], [0.0, -0.05], 0.02, [0.0, 0.005], [0.5], [[0.02, 0.0]],
                     [[1.0, 0.6], [0.6, 1.0]], 0.0, "md")
    eng.putAutocall(["X", "Y"], [100.0, 100.0], 1.0, 12, 1.02, 0.75, 0.03, 0.02, "ac")
    eng.putBaskets(["X", "Y"], [0.5, 0.5], 1.0, [100.0, 108.0], "bk")
    a = eng.AADriskOne("md", "ac", NumericalParam(useSobol=True, numPath=1 << 14))
    assert md["ac_value"] == a["riskPayoffValue"] and md["ac_nparams"] == 13
    assert md["ac_risks"] == [a["risks"][0], a["risks"][1], a["risks"][11]]
    assert md["ac_label"] == a["payoffIds"][0] and md["param12"] == "correl Y X"
    b = eng.AADriskMulti("md", "bk", NumericalParam(numPath=1 << 14))
    assert md["bk_shape"] == [13, 2] and md["bk_00"] == b["risks"][0, 0] and md["incompatible"] == 1
    eng.close()


def test_cpp_object_dropin_program(tmp_path):
    """A caller of the reference's object interfaces (Model<T>, Product<T>, RNG, mcSimul,
    mcSimulAAD, mcSimulAADMulti; include/cfgpu_mc.hpp): every number equals the store API's on
    the same inputs, bit for bit."""
    exe = str(tmp_path / "objects")
    lib = library_path()
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                           os.path.join(ROOT, "tests", "cpp", "objects_main.cpp"), lib, "-o", exe,
                           "-Wl,-rpath," + os.path.dirname(lib)])
    out = json.loads(subprocess.check_output([exe]).decode())
    n = out["n"]
    assert n == 4096 and out["npay"] == 2
    eng = Engine(0)
    spots = [50.0 * 4.0 ** (i / 19.0) for i in range(20)]
    times = [0.1 + 2.9 * j / 9.0 for j in range(10)]
    vols = np.array([[0.15 + 0.10 * np.exp(-t) * np.log(s / 100.0) ** 2 for t in times] for s in spots])
    eng.putDupire(100.0, spots, times, vols, 0.25, "d")
    eng.putDupire(101.0, spots, times, vols, 0.25, "d_up")
    eng.putBarrier(120.0, 150.0, 3.0, 3.0 / 156.0, 0.01, 0, "u")
    mrg = NumericalParam(numPath=n)
    # mcSimul: the payoff matrix
    paths = eng.simulatePaths("d", "u", mrg)
    assert out["path0"] == list(paths[0]) and out["path1"] == list(paths[1]) and out["path_last"] == list(paths[-1])
    seq = lambda x: float(np.cumsum(x)[-1])  # the caller's sequential sum
    assert out["mean0"] == seq(paths[:, 0]) / n
    assert out["mean0_up"] == seq(eng.simulatePaths("d_up", "u", mrg)[:, 0]) / n != out["mean0"]
    assert out["mean0_again"] == out["mean0"]
    # mcSimulAAD: default aggregator (the first payoff) and 1 x payoff0 + 0.5 x payoff1
    r = eng.AADriskOne("d", "u", mrg)
    assert out["aad_nparams"] == 201
    assert out["aad_risks"] == [r["risks"][0], r["risks"][5], r["risks"][1 + 3 * 10 + 4]]
    assert out["aad_aggregated"] == [paths[0, 0], paths[1, 0], paths[-1, 0]]
    w = eng.AADriskAggregate("d", "u", np.array([1.0, 0.5]), mrg)
    assert out["aadw_risks"] == [w["risks"][0], w["risks"][5], w["risks"][1 + 3 * 10 + 4]]
    assert out["aadw_aggregated"] == [paths[0, 0] + 0.5 * paths[0, 1], paths[1, 0] + 0.5 * paths[1, 1]]
    assert out["non_affine_threw"] == 1
    # Black-Scholes European, Sobol, FP32 path arithmetic
    eng.putBlackScholes(100.0, 0.2, 0, 0.02, 0.0, "bs")
    eng.putEuropean(100.0, 1.0, 1.0, "call")
    b = eng.AADriskOne("bs", "call", NumericalParam(useSobol=True, numPath=n, precision="fp32"))
    assert out["bs_risks"] == list(b["risks"])
    # mcSimulAADMulti of a portfolio
    eng.putEuropeans([1.0, 1.0, 2.0], [90.0, 110.0, 100.0], "port")
    m = eng.AADriskMulti("d", "port", NumericalParam(useSobol=True, numPath=n))
    assert out["multi_shape"] == [201, 3]
    assert out["multi_risks"] == [m["risks"][0, 0], m["risks"][0, 2], m["risks"][1 + 4 * 10 + 2, 1]]
    assert out["multi_path0"] == list(eng.simulatePaths("d", "port", NumericalParam(useSobol=True, numPath=n))[0])
    # shapes: the UOC timeline (today + weekly dates), its defline, labels, simDim; RNG draws
    assert len(out["timeline"]) == 157 and out["timeline"][0] == 0.0 and out["timeline"][-1] == 3.0
    assert out["defline_n"] == 157 and out["defline_num_last"] == 1 and out["defline_num_first"] == 0
    assert out["label0"] == r["payoffIds"][0] and out["param5"] == r["paramIds"][5] and out["simdim"] == 156
    g = eng.gaussians(False, 12345, 1234, 156, 0, 2)
    assert out["g0"] == [g[0, 0], g[0, 1], g[0, 155]] and out["g1"] == [g[1, 0], g[1, 1], g[1, 155]]
    assert out["g1"][0] == -out["g0"][0]
    assert 0.0 < out["u0"][0] < 1.0 and out["incompatible"] == 1
    eng.close()
