"""Shards of one run on one GPU (cf_enqueue_shard at different first paths, exact int64 sums of
the raw accumulators) give the results of one call over all the paths, bit for bit: the FP32
risk kernel and the FP64 kernel, mrg32k3a and Sobol, odd path counts."""
import numpy as np
import pytest

from compfinance_gb300 import Engine, NumericalParam
from compfinance_gb300 import workloads as W
from compfinance_gb300.api import results_from_raw
from compfinance_gb300.shard import shard_range

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
@pytest.mark.parametrize("sobol", [False, True])
def test_shards_sum_to_the_full_run(precision, sobol):
    eng = Engine(0)
    s, t, v = W.dupire_surface(60, 30)
    u = W.UOC_BARRIER
    eng.putDupire(W.DUPIRE_SPOT, s, t, v, W.DUPIRE_MAXDT, "shd")
    eng.putBarrier(u["strike"], u["barrier"], u["maturity"], u["monitor_freq"], u["smooth"], 0, "shu")
    npay, npar, _ = eng.shapes("shd", "shu")
    n = 50001
    num = NumericalParam(numPath=n, useSobol=sobol, precision=precision)
    for risk in (True, False):
        eng.enqueue("shd", "shu", num, risk=risk)
        full = eng.fetch(npay, npar if risk else 0)
        total = None
        for k in range(3):
            first, count = shard_range(n, k, 3)
            eng.enqueue_shard("shd", "shu", NumericalParam(numPath=count, useSobol=sobol, precision=precision), first,
                              risk=risk)
            acc = eng.fetch_raw()
            total = acc if total is None else total + acc
        got = results_from_raw(total, npar if risk else 0, npay, n)
        assert np.array_equal(got[0], full[0]) and np.array_equal(got[1], full[1])
        assert got[2] == full[2]
        if risk:
            assert np.array_equal(got[3], full[3])
    eng.close()
