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


def test_lanes_and_chunked_long_requests_identical(eng):
    """The serving policy of cf_server_configure: short requests on high-priority slots, long risks
    on low-priority slots, launched as path-range chunks of bounded work.  Every result equals the
    synchronous call's bit for bit (exact sums over the chunks), in both lanes and both generators,
    with the long lane admitting its least work first; configuring after the first request is
    refused."""
    stream = W.serving_stream(n=80, rate=4000.0, seed=23)
    for r in stream:
        r["paths"] = min(r["paths"], 1 << 18)
    stream += [dict(t=0.0, kind="risk", model="dup100_60x30w", product="uoc100_1_1.4_520", paths=(1 << 18) + 4161,
                    sobol=sob) for sob in (False, True)]
    srv = Server(eng, slots=6, hbm_budget=64 << 30)
    srv.configure(short_slots=3, long_threshold=1e7, chunk_path_steps=5e6, long_blocks_per_sm=4)
    srv.order(1, 1, 50.0)  # long risks: least work first
    stats, _, status, res = run_stream(eng, stream, keep_results=True, server=srv)
    assert all(s == "done" for s in status.values()), status
    longs = 0
    for i, r in enumerate(stream):
        v, k = _alone(eng, r)
        assert np.array_equal(res[i]["values"], v), i
        if k is not None:
            assert np.array_equal(res[i]["risks"], k), i
        if r["kind"] == "risk" and r["paths"] * eng.shapes(r["model"], r["product"])[2] > 1e7:
            longs += 1
    assert longs >= 2  # chunked: 5e6 path-steps per launch
    with pytest.raises(Exception):
        srv.configure(short_slots=2, long_threshold=1e7)
    srv.close()


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


def test_model_replaced_while_requests_run(eng):
    """A model re-put while requests on it run: requests that started run on the model as it
    was when they started, requests that start later on the new one.  The replaced plan stays
    valid until its results have been fetched (the new plan takes over its device tables)."""
    import time
    s, t, v = W.dupire_surface(60, 30)
    u = W.UOC_BARRIER
    eng.putBarrier(u["strike"], u["barrier"], u["maturity"], u["monitor_freq"], u["smooth"], 0, "rp_uoc")
    num = NumericalParam(numPath=1 << 18, precision="fp32")
    eng.putDupire(W.DUPIRE_SPOT, s, t, v * 1.1, W.DUPIRE_MAXDT, "rp_dup")
    new = eng.AADriskOne("rp_dup", "rp_uoc", num)
    eng.putDupire(W.DUPIRE_SPOT, s, t, v, W.DUPIRE_MAXDT, "rp_dup")
    old = eng.AADriskOne("rp_dup", "rp_uoc", num)
    assert not np.array_equal(old["risks"], new["risks"])
    srv = Server(eng, slots=2, hbm_budget=64 << 30)
    ids = [srv.submit("risk", "rp_dup", "rp_uoc", num) for _ in range(2)]
    t0 = time.time()
    while any(srv.wait(i, timeout_ms=0) == "queued" for i in ids):
        assert time.time() - t0 < 30
        time.sleep(0.0005)
    eng.putDupire(W.DUPIRE_SPOT, s, t, v * 1.1, W.DUPIRE_MAXDT, "rp_dup")
    later = srv.submit("risk", "rp_dup", "rp_uoc", num)  # lowers the new plan when it starts
    assert srv.wait(later) == "done"
    for i in ids:
        assert srv.wait(i) == "done"
        got = srv.result(i)
        assert np.array_equal(got["risks"], old["risks"]) and np.array_equal(got["values"], old["payoffValues"])
    got = srv.result(later)
    assert np.array_equal(got["risks"], new["risks"]) and np.array_equal(got["values"], new["payoffValues"])
    srv.close()
