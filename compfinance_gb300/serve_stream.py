"""Drive the serving loop with a timed request stream (workloads.serving_stream) and, for
comparison, run the same requests one at a time through the synchronous entry points."""
import gc
import threading
import time

import numpy as np

from . import workloads as W
from .api import NumericalParam, Server


def load_store(eng, models, products):
    for mid, m in models.items():
        if m["kind"] == "bs":
            eng.putBlackScholes(m["spot"], m["vol"], m.get("qspot", 0), m["rate"], m["div"], mid)
        else:
            eng.putDupire(m["spot"], m["spots"], m["times"], m["vols"], m["maxdt"], mid)
    for pid, p in products.items():
        if p["kind"] == "european":
            eng.putEuropean(p["strike"], p["exercise"], p["settlement"], pid)
        elif p["kind"] == "uoc":
            eng.putBarrier(p["strike"], p["barrier"], p["maturity"], p["freq"], p["smooth"], p["callput"], pid)
        else:
            eng.putEuropeans(p["mats"], p["strikes"], pid)


def num_of(r, precision="fp32"):
    return NumericalParam(useSobol=r["sobol"], numPath=r["paths"], precision=precision)


def run_one_at_a_time(eng, stream, precision="fp32"):
    """Sequential execution of the stream's requests (no arrival gaps, no overlap)."""
    eng.synchronize()
    t0 = time.perf_counter()
    steps = 0
    for r in stream:
        nm = num_of(r, precision)
        if r["kind"] == "value":
            eng.value(r["model"], r["product"], nm)
        elif r["kind"] == "risk":
            eng.AADriskOne(r["model"], r["product"], nm)
        else:
            eng.AADriskMulti(r["model"], r["product"], nm)
        steps += r["paths"] * eng.shapes(r["model"], r["product"])[2]
    return time.perf_counter() - t0, steps


def run_stream(eng, stream, slots=8, budget=64 << 30, precision="fp32", keep_results=False, server=None):
    """Submit each request at its arrival time; returns stats, makespan and (optionally) results.
    With `server`, the stream runs on that server (its statistics reset first, its slots and
    their device buffers kept); otherwise on a new server of `slots` slots and `budget` bytes."""
    srv = server or Server(eng, slots=slots, hbm_budget=budget)
    if server is not None:
        srv.reset_stats()
    ids = [None] * len(stream)
    # a collection pause of this process would hold back submissions and release them as a
    # burst: the client, not the server, would shape the arrivals
    gc_was = gc.isenabled()
    gc.disable()
    try:
        t0 = time.perf_counter()

        lag = [0.0]

        def submitter():
            for i, r in enumerate(stream):
                dt = r["t"] - (time.perf_counter() - t0)
                if dt > 0:
                    time.sleep(dt)
                lag[0] = max(lag[0], time.perf_counter() - t0 - r["t"])
                ids[i] = srv.submit(r["kind"], r["model"], r["product"], num_of(r, precision))

        th = threading.Thread(target=submitter)
        th.start()
        th.join()
        results = {}
        status = {}
        for i, rid in enumerate(ids):
            st = srv.wait(rid)
            status[i] = st
            if keep_results and st == "done":
                results[i] = srv.result(rid)
            srv.release(rid)  # the server keeps a request's results until they are released
        makespan = time.perf_counter() - t0
    finally:
        if gc_was:
            gc.enable()
    stats = srv.stats()
    # how far the submitting thread fell behind the planned arrival times at worst: a late client
    # releases requests in bursts, which queue
    stats["submitLagMaxMs"] = 1000.0 * lag[0]
    if server is None:
        srv.close()
    return stats, makespan, status, results
