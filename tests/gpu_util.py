"""Helpers shared by the GPU tests: engine fixture and golden-case loading."""
import numpy as np

import oracle as O
from compfinance_gb300 import Engine, NumericalParam


def rel_to_max(a, b):
    a = np.asarray(a, dtype=float).ravel()
    b = np.asarray(b, dtype=float).ravel()
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def put_model(eng, mid, spec):
    if spec["kind"] == "bs":
        eng.putBlackScholes(spec["spot"], spec["vol"], spec.get("qspot", 0), spec["rate"], spec["div"], mid)
    else:
        eng.putDupire(spec["spot"], spec["spots"], spec["times"], np.asarray(spec["vols"]), spec["maxdt"], mid)


def put_product(eng, pid, spec):
    if spec["kind"] == "european":
        eng.putEuropean(spec["strike"], spec["exercise"], spec["settlement"], pid)
    elif spec["kind"] == "contingent":
        eng.putContingent(spec["coupon"], spec["maturity"], spec["freq"], spec["smooth"], pid)
    elif spec["kind"] == "uoc":
        eng.putBarrier(spec["strike"], spec["barrier"], spec["maturity"], spec["freq"], spec["smooth"],
                       spec.get("callput", 0), pid)
    else:
        eng.putEuropeans(spec["mats"], spec["strikes"], pid)


def num(sobol, n, precision="fp64", seed1=12345, seed2=1234):
    return NumericalParam(parallel=True, useSobol=bool(sobol), numPath=int(n), seed1=seed1, seed2=seed2,
                          precision=precision)
