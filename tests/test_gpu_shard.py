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


@pytest.mark.parametrize("prod", ["uoc", "european"])
@pytest.mark.parametrize("sobol", [False, True])
def test_multi_round_run_equals_single_round_shards(prod, sobol):
    """The FP32 risk kernel over 2^21 + 12345 paths runs several unit rounds per thread (7 with
    mrg32k3a, 14 with Sobol): live paths wait in the block's pending list and ring of round slots,
    and partial chunks are swept when a slot is about to be reused.  Sixteen shards of the same
    paths each run a single round.  Every contribution is rounded once, so the exact sums agree
    bit for bit: a path lost, swept twice or read from the wrong slot would show.  The 20x10 grid
    sends many contributions to the blocks' int64 slabs."""
    eng = Engine(0)
    s, t, v = W.dupire_surface(20, 10)
    u = W.UOC_BARRIER
    eng.putDupire(W.DUPIRE_SPOT, s, t, v, W.DUPIRE_MAXDT, "ring")
    if prod == "uoc":
        eng.putBarrier(u["strike"], u["barrier"], u["maturity"], u["monitor_freq"], u["smooth"], 0, "ringp")
    else:
        eng.putEuropean(110.0, 2.0, 2.0, "ringp")
    npay, npar, _ = eng.shapes("ring", "ringp")
    n = (1 << 21) + 12345
    eng.enqueue("ring", "ringp", NumericalParam(numPath=n, useSobol=sobol, precision="fp32"), risk=True)
    full = eng.fetch(npay, npar)
    total = None
    for k in range(16):
        first, count = shard_range(n, k, 16)
        eng.enqueue_shard("ring", "ringp", NumericalParam(numPath=count, useSobol=sobol, precision="fp32"), first,
                          risk=True)
        acc = eng.fetch_raw()
        total = acc if total is None else total + acc
    got = results_from_raw(total, npar, npay, n)
    assert np.array_equal(got[0], full[0]) and np.array_equal(got[3], full[3])
    assert np.abs(full[3]).max() > 0
    eng.close()
