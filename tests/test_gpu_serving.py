"""The serving loop on the GPU: each result is bit-identical alone and in the mix (exact
fixed-point sums, per-path random numbers), admission respects the device budget, and
host-injected failures, cancellations and time-outs leave the server running."""
import numpy as np
import pytest

from compfinance_gb300 import Engine, NumericalParam
from compfinance_gb300 import workloads as W
from compfinance_gb300.api import Server
from compfinance_gb300.serve_stream import load_store, num_of, run_stream

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng():
    e = Engine(0)
    models, products = W.serving_store()
    load_store(e, models, products)
    yield e
    e.close()


def _alone(eng, r):
    nm = num_of(r)
    if r["kind"] == "value":
        x = eng.value(r["model"], r["product"], nm)
        return x["values"], None
    if r["kind"] == "risk":
        x = eng.AADriskOne(r["model"], r["product"], nm)
        return x["payoffValues"], x["risks"]
    x = eng.AADriskMulti(r["model"], r["product"], nm)
    return x["values"], x["risks"]


def test_results_identical_alone_and_in_the_mix(eng):
    stream = W.serving_stream(n=120, rate=4000.0, seed=11)
    for r in stream:  # keep the test quick
        r["paths"] = min(r["paths"], 1 << 16)
    stats, makespan, status, res = run_stream(eng, stream, slots=6, keep_results=True)
    assert all(s == "done" for s in status.values()), status
    assert stats["maxInFlight"] > 1  # requests did overlap
    for i, r in enumerate(stream):
        v, k = _alone(eng, r)
        assert np.array_equal(res[i]["values"], v), i
        if k is not None:
            assert np.array_equal(res[i]["risks"], k), i
    assert stats["p99Ms"] >= stats["p50Ms"] > 0


def test_admission_budget_rejection_and_failures(eng):
    # A 60x30 barrier risk request at 2^16 FP32 paths runs one unit round and holds ~148 MB of
    # reverse-sweep scratch (7 fields x 157 dates x 2^15 threads x 4 B, plus the blocks' node
    # slabs); the same at 2^22 paths holds three round slots for the full resident grid
    # (~2 GB).  A 320 MB budget runs two small ones at a time and rejects the large one.
    srv = Server(eng, slots=4, hbm_budget=320 << 20)
    r = dict(kind="risk", model="dup100_60x30w", product="uoc100_1_1.4_156", paths=1 << 16, sobol=False)
    big = dict(r, paths=1 << 22)
    ids = [srv.submit("risk", r["model"], r["product"], num_of(r)) for _ in range(6)]
    rej = srv.submit("risk", big["model"], big["product"], num_of(big))
    assert srv.wait(rej) == "rejected" and "budget" in srv.error()
    assert all(srv.wait(i) == "done" for i in ids)
    st = srv.stats()
    assert st["maxInFlight"] <= 2 and st["peakFootprint"] <= 320 << 20
    # the next two starts fail (an allocation failure injected on the host)
    srv.inject_failures(2)
    bad = [srv.submit("value", "bs100", "eu100_1", num_of(dict(paths=1 << 14, sobol=True))) for _ in range(2)]
    assert all(srv.wait(i) == "failed" for i in bad) and "injected" in srv.error()
    st = srv.stats()
    assert st["failed"] == 2 and st["rejected"] == 1
    # the server still works after the failures
    ok = srv.submit("value", "bs100", "eu100_1", num_of(dict(paths=1 << 14, sobol=True)))
    assert srv.wait(ok) == "done"
    srv.close()


def test_cancel_and_queue_timeout(eng):
    srv = Server(eng, slots=1, hbm_budget=64 << 30)
    long_r = dict(kind="risk", model="dup100_120x60w", product="uoc100_1_1.4_520", paths=1 << 20, sobol=False)
    first = srv.submit("risk", long_r["model"], long_r["product"], num_of(long_r))
    q = srv.submit("risk", long_r["model"], long_r["product"], num_of(long_r))
    t = srv.submit("value", "bs100", "eu100_1", num_of(dict(paths=1 << 14, sobol=True)), queue_timeout_ms=0.001)
    srv.cancel(q)
    assert srv.wait(q) == "cancelled"
    assert srv.wait(first) == "done"
    assert srv.wait(t) in ("timeout", "done")
    srv.close()
