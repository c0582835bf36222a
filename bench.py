#!/usr/bin/env python3
"""Benchmark of the Dupire up-and-out AAD-risk workload on one GB300.

Workload (one "step"): AADriskOne of the smoothed up-and-out call (K=120, B=150, 1%
smoothing, T=3y, 156 weekly monitoring dates) on a Dupire local-vol surface of 60 spots x 30
times, mrg32k3a(12345, 1234), 2^22 paths, FP32 path arithmetic with exact fixed-point
accumulation: price plus the 1801 risks (spot + every local-vol node).  The same run in the
FP64 form is timed beside it (the FP32-vs-FP64 ratio and their difference in MC standard
errors are reported).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line.  `value` is device-timed throughput with the model resident in HBM;
`e2e` goes through the C ABI with host buffers each step (putDupire upload + risk + result
download).  `--impl reference` times the CPU restatement of the reference's algorithm
(oracle/, hand-written per-path adjoint, all host threads) on a bounded sample of the same
workload.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from compfinance_gb300 import workloads as W  # noqa: E402

METRIC = "AAD-risk paths/s (Dupire barrier), FP32 vs FP64 at equal error; serve p99 ms"
NPATH = 1 << 22
GRID = (60, 30)
FLOPS_PER_PATH_STEP = 53.0   # algorithmic FP work of value + adjoint per path-step (mrg32k3a)
TRAFFIC_BYTES_PER_PATH_STEP = 11.80  # measured DRAM traffic of the FP32 risk launch per path-step
INST_PER_PATH_STEP = 99.6  # measured thread instructions of the FP32 risk launch per path-step
# serving: slots of the short and long request classes, the path-steps above which a barrier risk
# is long, stream runs per offered load
SERVE_SHORT_SLOTS, SERVE_LONG_SLOTS, SERVE_LONG_THRESHOLD = 8, 3, 2e7
SERVE_LONG_BLOCKS_PER_SM = 4  # resident blocks per SM of a long request: room for short ones
# long risks are admitted least work first (a large one queued longer than this goes first)
SERVE_LONG_ORDER, SERVE_LONG_AGING_MS = 1, 50.0
SERVE_LOAD_RUNS = 5
# FP64 form (mc_kernel<double>): ncu of the same kernel at 2^18 paths measures its FP64 pipe 82.9%
# busy; GB300 executes 2 FP64 FMAs per SM per cycle (ncu's peak of the DFMA counter)
FP64_PIPE_BUSY_NCU = 0.829
DFMA_PER_SM_PER_CYCLE = 2
CONFIG = {
    "workload": "dupire_uoc_aad_risk_60x30_156steps_2^22paths_fp32path",
    "model": "Dupire local vol 60x30 (50-200 log-spaced x 0.1-3.0y), seeded synthetic surface",
    "product": "up-and-out call K=120 B=150 smooth 1% T=3y weekly (156 steps)",
    "rng": "mrg32k3a(12345,1234) antithetic",
    "paths": NPATH,
    "risks": 1801,
    "l2": "flushed between steps (256 MiB write outside the per-step events); the reverse-sweep scratch "
          "(three unit-round slots, ~2.3 GB) also exceeds L2",
}


def env_rank():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return json.load(fh)
    except OSError:
        return {}


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    def __init__(self, path):
        self.path = path
        self.proc = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-lms", "100"], stdout=self.fh, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            self.proc.wait()
            self.fh.close()

    def summary(self):
        try:
            rows = [r.split(", ") for r in open(self.path).read().strip().splitlines()]
        except OSError:
            return None
        rows = [r for r in rows if len(r) >= 9]
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = max(float(r[2]) for r in rows if r[2].replace(".", "").isdigit())
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].strip().lower() == "active"})
        loaded = [s for s in sm if s > 0.5 * mx] or sm
        return {"sm_mhz": statistics.median(loaded), "sm_max_mhz": mx, "reasons": reasons, "samples": len(rows)}


def _cpu_case():
    import oracle as O
    s, t, v = W.dupire_surface(*GRID)
    u = W.UOC_BARRIER
    m = O.Model(dict(kind="dupire", spot=W.DUPIRE_SPOT, spots=s, times=t, vols=v, maxdt=W.DUPIRE_MAXDT))
    p = O.Product(dict(kind="uoc", strike=u["strike"], barrier=u["barrier"], maturity=u["maturity"],
                       freq=u["monitor_freq"], smooth=u["smooth"], callput=0))
    return O, m, p, np.array([1.0, 0.0])


def _cpu_sample_size(O, m, p, w, threads, seconds):
    """Paths (even) that the threaded CPU adjoint runs in about `seconds`."""
    n = 1 << 12
    while True:  # a calibration run long enough that thread start-up does not dominate it
        t0 = time.perf_counter()
        O.risk(m, p, 0, n, w, fast=True, threads=threads)
        dt = time.perf_counter() - t0
        if dt >= 0.5 or n >= 1 << 22:
            break
        n *= 4
    n = int(min(1 << 25, max(n, n * seconds / max(dt, 1e-3))))
    return n - n % 2


def _host_desc():
    """The host the CPU legs ran on: architecture, the cores this process may use of those online."""
    import platform
    online = os.cpu_count() or 1
    usable = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else online
    return f"{platform.machine()}, {usable} usable of {online} online cores"


def cpu_baseline(seconds=18.0, threads=None):
    """The oracle's hand-written adjoint (multi-threaded) on a bounded sample of the workload."""
    O, m, p, w = _cpu_case()
    threads = threads or os.cpu_count() or 1
    n = _cpu_sample_size(O, m, p, w, threads, seconds)
    t0 = time.perf_counter()
    O.risk(m, p, 0, n, w, fast=True, threads=threads)
    dt = time.perf_counter() - t0
    return {"value": n / dt, "unit": "paths/s", "cores": threads, "kind": "port",
            "sample": f"{n} paths of the same workload (FP64, hand-written adjoint), {dt:.2f} s",
            "host": _host_desc()}


def multi_asset_leg(eng, npath=1 << 20):
    """The four-asset displaced model (one asset per dynamics, dividends, lambda-shifted
    correlation): AADriskOne of the 6-period autocall (1 payoff) and of the 5-strike basket (the
    first strike), 36 parameters, Sobol paths, FP32 and FP64 path arithmetic (wall clock,
    synchronous calls after a warm-up)."""
    from compfinance_gb300 import NumericalParam
    mid, ac, bk = W.put_md4(eng)
    out = {"paths": npath, "assets": len(W.MD4["assets"]), "params": eng.shapes(mid, ac)[1]}
    for name, pid in (("autocall", ac), ("basket", bk)):
        rec = {}
        for prec in ("fp32", "fp64"):
            num = NumericalParam(useSobol=True, numPath=npath, precision=prec)
            eng.AADriskOne(mid, pid, num)
            t0 = time.perf_counter()
            r = eng.AADriskOne(mid, pid, num)
            dt = time.perf_counter() - t0
            rec[prec] = {"risk_s": dt, "paths_per_s": npath / dt, "value": r["riskPayoffValue"]}
        out[name] = rec
    return out


def cpu_multi_asset(seconds=4.0):
    """The oracle's tape-based AADriskOne of the four-asset autocall, one thread, on a bounded
    sample (the reference's own procedure: a tape per path)."""
    import oracle as O
    m = O.MModel(dict(W.MD4, **{"lambda": W.MD4["lam"]}))
    p = O.MProduct(dict(kind="autocall", assets=W.MD4["assets"], **W.MD4_AUTOCALL))
    n = 1024
    while True:
        t0 = time.perf_counter()
        O.m_risk(m, p, 1, n, [1.0])
        dt = time.perf_counter() - t0
        if dt > seconds / 4 or n >= 1 << 20:
            break
        n *= 2
    return {"value": n / dt, "unit": "paths/s", "cores": 1, "kind": "port",
            "sample": f"{n} Sobol paths of the four-asset autocall AADriskOne (FP64 tape), {dt:.2f} s"}


def serving_leg(eng, n, seed):
    """Mixed request stream (seeded Poisson arrivals at 2,000 req/s; 40% BS values, 40% Dupire
    barrier risks of 2^16-2^20 paths on 20x10..120x60 grids with 12..520 steps, 20% European
    portfolio AADriskMulti), FP32 path form, 64 GB admission budget, 3 runs.  The server runs 8
    slots for short requests on high-priority streams (values, portfolio risks, barrier risks of
    at most 2e7 path-steps) and 3 for long risks at low priority with at most 4 resident blocks
    per SM, admitted least work first; then the same requests all submitted at once (the server's
    batch throughput), at arrival rates offering 80%, 85% and 90% of it (5 runs each), and one at a
    time through the synchronous entry points."""
    from compfinance_gb300.api import Server
    from compfinance_gb300.serve_stream import load_store, run_one_at_a_time, run_stream
    models, products = W.serving_store()
    load_store(eng, models, products)
    stream = W.serving_stream(n=n, rate=2000.0, seed=seed)
    for r in stream:  # lower every plan and warm each kernel variant before timing
        eng.shapes(r["model"], r["product"])
    # one server for every stream below: 8 slots, 64 GB admission budget.  The batch (the same
    # requests all submitted at once: the server's capacity) runs once untimed first, which
    # also grows every slot's device buffers to the stream's sizes, as a long-running server's are.
    srv = Server(eng, slots=SERVE_SHORT_SLOTS + SERVE_LONG_SLOTS, hbm_budget=64 << 30)
    srv.configure(SERVE_SHORT_SLOTS, SERVE_LONG_THRESHOLD, 0.0, SERVE_LONG_BLOCKS_PER_SM)
    srv.order(1, SERVE_LONG_ORDER, SERVE_LONG_AGING_MS)
    batch_reqs = [dict(r, t=0.0) for r in stream]
    run_stream(eng, batch_reqs, server=srv)
    stats, makespan, status, _ = run_stream(eng, stream, server=srv)
    p99_2000 = [stats["p99Ms"]] + [run_stream(eng, stream, server=srv)[0]["p99Ms"] for _ in range(2)]
    bstats, bmakespan, _, _ = run_stream(eng, batch_reqs, server=srv)
    t_seq, steps = run_one_at_a_time(eng, stream)
    served = stats["pathStepsDone"] / makespan
    batch_all = bstats["pathStepsDone"] / bmakespan
    batch = steps / t_seq
    # the same requests at arrival rates that offer 80%, 85% and 90% of the batch capacity
    # (arrival times scaled): p99 latency with the server under that load
    load = []
    for frac in (0.8, 0.85, 0.9):
        rate = frac * n / bmakespan
        scaled = [dict(r, t=r["t"] * 2000.0 / rate) for r in stream]
        runs = []
        for _ in range(SERVE_LOAD_RUNS):
            lstats, lmakespan, _, _ = run_stream(eng, scaled, server=srv)
            runs.append({"completed": lstats["completed"], "failed": lstats["failed"], "p50_ms": lstats["p50Ms"],
                         "p99_ms": lstats["p99Ms"], "makespan_s": lmakespan,
                         "served_over_batch": lstats["pathStepsDone"] / lmakespan / batch_all})
        p99s = [x["p99_ms"] for x in runs]
        load.append({"offered_over_batch": frac, "arrival_rate_req_s": rate, "runs": len(runs),
                     "p99_ms_median": statistics.median(p99s), "p99_ms_max": max(p99s),
                     "p50_ms_median": statistics.median(x["p50_ms"] for x in runs),
                     "served_over_batch_min": min(x["served_over_batch"] for x in runs),
                     "completed_min": min(x["completed"] for x in runs),
                     "failed_max": max(x["failed"] for x in runs), "p99_ms_runs": p99s})
    out = {"requests": n, "arrival_rate_req_s": 2000.0,
           "slots": {"short": SERVE_SHORT_SLOTS, "long": SERVE_LONG_SLOTS,
                     "long_threshold_path_steps": SERVE_LONG_THRESHOLD,
                     "long_blocks_per_sm": SERVE_LONG_BLOCKS_PER_SM,
                     "long_order": "least work first" if SERVE_LONG_ORDER else "arrival",
                     "long_aging_ms": SERVE_LONG_AGING_MS}, "hbm_budget_gb": 64,
           "p99_ms_runs_at_2000": p99_2000, "p99_ms_median_at_2000": statistics.median(p99_2000),
            "completed": stats["completed"], "failed": stats["failed"], "rejected": stats["rejected"],
            "p50_ms": stats["p50Ms"], "p99_ms": stats["p99Ms"], "mean_ms": stats["meanMs"],
            "makespan_s": makespan, "served_path_steps_per_s": served,
            "batch_makespan_s": bmakespan, "batch_path_steps_per_s": batch_all, "served_over_batch": served / batch_all,
            "one_at_a_time_s": t_seq, "one_at_a_time_path_steps_per_s": batch,
            "served_over_one_at_a_time": served / batch, "max_in_flight": stats["maxInFlight"],
            "peak_footprint_gb": stats["peakFootprint"] / 2**30, "load_sweep": load}
    srv.close()
    return out


def grid_sweep(eng, stream, flush, npath):
    """The precision workload's grid sweep: the same barrier risk on the 20x10, 60x30 and 120x60
    surfaces, FP32 path form and FP64 form (CUDA events on the engine's stream, L2 flushed
    between launches), and the FP32-FP64 difference of every risk in Monte Carlo standard
    errors (from 8 independent FP32 seed pairs at a quarter of the paths)."""
    import torch
    from compfinance_gb300 import NumericalParam
    u = W.UOC_BARRIER
    out = {}
    for g in ((20, 10), (60, 30), (120, 60)):
        s, t, v = W.dupire_surface(*g)
        mid = f"sweep{g[0]}x{g[1]}"
        eng.putDupire(W.DUPIRE_SPOT, s, t, v, W.DUPIRE_MAXDT, mid)
        npay, npar, dim = eng.shapes(mid, "uoc")
        res = {}
        risks = {}
        for prec, reps in (("fp32", 3), ("fp64", 2)):
            num = NumericalParam(numPath=npath, precision=prec)
            eng.enqueue(mid, "uoc", num, risk=True)
            torch.cuda.synchronize()
            ms = []
            for k in range(reps):
                flush.fill_(float(k))
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                eng.enqueue(mid, "uoc", num, risk=True)
                b.record(stream)
                torch.cuda.synchronize()
                ms.append(a.elapsed_time(b))
            risks[prec] = eng.fetch(npay, npar)
            best = min(ms)
            res[prec] = {"ms_per_step": best, "paths_per_s": npath / (best / 1e3),
                         "path_steps_per_s": npath * dim / (best / 1e3)}
        se = []
        for k in range(8):
            eng.enqueue(mid, "uoc", NumericalParam(numPath=npath // 4, precision="fp32", seed1=1000 + k,
                                                   seed2=77 + k), risk=True)
            se.append(eng.fetch(npay, npar)[3])
        se = np.std(np.array(se), axis=0, ddof=1) / 2.0
        r32, r64 = risks["fp32"][3], risks["fp64"][3]
        mask = se > 1e-3 * np.abs(r64).max()
        res["fp32_over_fp64"] = res["fp64"]["ms_per_step"] / res["fp32"]["ms_per_step"]
        res["max_risk_fp32_minus_fp64_in_stderr"] = float(np.max(np.abs(r32 - r64)[mask] / se[mask]))
        res["price_fp32_minus_fp64_in_stderr"] = float(abs(risks["fp32"][0][0] - risks["fp64"][0][0]) /
                                                       risks["fp64"][1][0])
        out[f"{g[0]}x{g[1]}"] = res
    return out


def superbucket_leg(eng, npath=1 << 20):
    """The superbucket workload: implied-vol surface (30 strikes x 12 maturities) calibrated to a
    60x30 local-vol grid in FP64; 200 Europeans (10 maturities x 20 strikes), 36 monthly steps,
    Sobol paths.  Times AADriskMulti (200 risk vectors of 1801 parameters) on the calibrated
    model and the whole dupireSuperbucket chain (calibration, MC adjoints, calibration adjoint
    to the 360 implied vols), in both precisions of the path arithmetic (wall clock, each call
    synchronous)."""
    from compfinance_gb300 import Engine, NumericalParam
    iv = Engine.ivs("param", 100.0, [W.SB_IVS["a"], W.SB_IVS["b"], W.SB_IVS["c"], W.SB_IVS["sref"]])
    isp, mds, itm, mdt = W.superbucket_grid(60, 30)
    rk, rm = W.superbucket_riskview(30, 12)
    mats, strikes = W.superbucket_portfolio(10, 20)
    eng.putEuropeans(mats, strikes, "c4port")
    cal = eng.dupireCalib(iv, isp, mds, itm, mdt)
    eng.putDupire(100.0, cal["spots"], cal["times"], cal["lVols"], 1.0 / 12.0, "c4dup")
    w = np.ones(len(mats))
    out = {"paths": npath, "payoffs": len(mats), "params": 1 + len(cal["spots"]) * len(cal["times"]),
           "implied_vols": len(rk) * len(rm)}
    for prec in ("fp32", "fp64"):
        num = NumericalParam(useSobol=True, numPath=npath, precision=prec)
        eng.AADriskMulti("c4dup", "c4port", num)  # warm-up (plan lowering, buffers)
        t0 = time.perf_counter()
        eng.AADriskMulti("c4dup", "c4port", num)
        t_multi = time.perf_counter() - t0
        eng.dupireSuperbucket(iv, 100.0, 1.0 / 12.0, "c4port", w, isp, mds, itm, mdt, rk, rm, num)
        t0 = time.perf_counter()
        sb = eng.dupireSuperbucket(iv, 100.0, 1.0 / 12.0, "c4port", w, isp, mds, itm, mdt, rk, rm, num)
        t_sb = time.perf_counter() - t0
        out[prec] = {"aad_risk_multi_s": t_multi, "aad_risk_multi_paths_per_s": npath / t_multi,
                     "superbucket_s": t_sb, "superbucket_value": sb["value"], "superbucket_delta": sb["delta"]}
    return out


def bump_leg(eng):
    """bumpRisk (finite differences, 1e-8 bumps of the 1801 parameters, FP64) of the C2 workload
    (60x30 barrier, 156 weekly steps, mrg32k3a): the pathwise procedure at 2^16 and 2^18 paths and
    full repricing at 2^16 (wall clock, synchronous calls), and their agreement."""
    from compfinance_gb300 import NumericalParam
    s, t, v = W.dupire_surface(60, 30)
    eng.putDupire(W.DUPIRE_SPOT, s, t, v, W.DUPIRE_MAXDT, "bumpdup")
    out = {"params": eng.shapes("bumpdup", "uoc")[1]}
    eng.bumpRisk("bumpdup", "uoc", NumericalParam(numPath=1 << 12), method="pathwise")  # warm-up
    res = {}
    for n, method in ((1 << 16, "pathwise"), (1 << 18, "pathwise"), (1 << 16, "reprice")):
        t0 = time.perf_counter()
        res[(n, method)] = eng.bumpRisk("bumpdup", "uoc", NumericalParam(numPath=n), method=method)["risks"]
        out[f"{method}_2^{n.bit_length() - 1}_s"] = time.perf_counter() - t0
    a, b = res[(1 << 16, "pathwise")], res[(1 << 16, "reprice")]
    out["pathwise_speedup_over_reprice_2^16"] = out["reprice_2^16_s"] / out["pathwise_2^16_s"]
    out["pathwise_minus_reprice_rel_to_max_2^16"] = float(np.abs(a - b).max() / np.abs(b).max())
    return out


def run_reference(args):
    """The reference arm: the CPU restatement of the reference's path (the reference's own
    sources are not on the GPU host) on all host threads, W untimed + K timed steps, each step
    a bounded sample of the workload (~4 s)."""
    rank, world, _ = env_rank()
    if rank != 0:
        return 0
    O, m, p, w = _cpu_case()
    threads = os.cpu_count() or 1
    n = _cpu_sample_size(O, m, p, w, threads, 4.0)
    for _ in range(args.warmup):
        O.risk(m, p, 0, min(n, 1 << 14), w, fast=True, threads=threads)
    ts = []
    for k in range(args.steps):
        t0 = time.perf_counter()
        O.risk(m, p, 0, n, w, fast=True, threads=threads, seed1=W.MRG_SEEDS[0] + k)
        ts.append(time.perf_counter() - t0)
    tot = sum(ts)
    value = n * args.steps / tot
    cb = {"value": value, "unit": "paths/s", "cores": threads, "kind": "port",
          "sample": f"{n} paths per step of the same workload (FP64, hand-written adjoint, {threads} threads)",
          "host": _host_desc()}
    out = {"impl": "reference", "metric": METRIC, "value": value, "unit": "paths/s", "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": tot / args.steps * 1e3,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic", "config": CONFIG, "cpu_baseline": cb,
           "e2e": {"value": value, "unit": "paths/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))
    return 0


def run_case(args):
    """One secondary workload alone, for profiler captures: `--case multi` is AADriskMulti of the
    superbucket portfolio (200 Europeans, 36 monthly steps, Sobol) on a synthetic Dupire grid;
    `--case autocall|basket` is AADriskOne of the four-asset autocall or basket (Sobol);
    `--case superbucket` the whole dupireSuperbucket chain of the portfolio (calibration of the
    parametric surface to 60x30 local vols, Monte Carlo adjoints, calibration adjoint to 30x12)."""
    paths = args.paths if args.paths != NPATH else 1 << 20
    if args.case == "superbucket":
        sec = W.run_superbucket(paths, args.reps, args.precision)
        print(f"dupireSuperbucket 30x12 -> 60x30, 200 Europeans, {args.precision} {paths} paths: "
              f"{1e3 * sec:.3f} ms per call")
        return 0
    if args.case == "multi":
        g = tuple(int(x) for x in args.grid.split("x"))
        sec = W.run_multi(g, paths, args.reps, args.precision)
        print(f"AADriskMulti {g[0]}x{g[1]} {args.precision} {paths} paths: {1e3 * sec:.3f} ms per call, "
              f"{paths / sec:.4g} paths/s")
    else:
        sec = W.run_md(args.case, paths, args.reps, args.precision)
        print(f"AADriskOne 4-asset {args.case} {args.precision} {paths} paths: {1e3 * sec:.3f} ms per call, "
              f"{paths / sec:.4g} paths/s")
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-serving", action="store_true", help="skip the serving-stream leg")
    ap.add_argument("--no-sweep", action="store_true", help="skip the grid sweep and superbucket legs")
    ap.add_argument("--serve-requests", type=int, default=10000)
    ap.add_argument("--paths", type=int, default=NPATH,
                    help="paths per step (default 2^22; smaller cases are for profiler captures only)")
    ap.add_argument("--case", choices=["multi", "autocall", "basket", "superbucket"],
                    help="time one secondary workload alone (for profiler captures) and exit: the superbucket "
                         "portfolio's AADriskMulti, AADriskOne of the four-asset autocall or basket, or the whole "
                         "dupireSuperbucket chain of that portfolio")
    ap.add_argument("--grid", default="60x30", help="--case multi: local-vol grid")
    ap.add_argument("--reps", type=int, default=1, help="--case: timed calls after one warm-up call")
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64"], help="--case: path precision")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        return run_reference(args)
    if args.case:
        return run_case(args)

    import torch
    from compfinance_gb300 import Engine, NumericalParam

    npath = args.paths
    config = dict(CONFIG, paths=npath)
    if npath != NPATH:
        config["workload"] = CONFIG["workload"].replace("2^22paths", f"{npath}paths")
    rank, world, local = env_rank()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    stream = torch.cuda.Stream()       # a real stream handle (the legacy default stream is 0)
    torch.cuda.set_stream(stream)
    eng = Engine(local)
    eng.set_stream(stream.cuda_stream)
    s, t, v = W.dupire_surface(*GRID)
    u = W.UOC_BARRIER
    eng.putDupire(W.DUPIRE_SPOT, s, t, v, W.DUPIRE_MAXDT, "dupire")
    eng.putBarrier(u["strike"], u["barrier"], u["maturity"], u["monitor_freq"], u["smooth"], 0, "uoc")
    npay, npar, dim = eng.shapes("dupire", "uoc")
    # With N ranks the step is one run of N x npath paths sharded by path range: rank r
    # simulates paths [r npath, (r + 1) npath) (weak scaling), and the exact int64 accumulators
    # are summed across ranks once, after the timed steps (compfinance_gb300/shard.py).
    num32 = NumericalParam(numPath=npath, precision="fp32")
    num64 = NumericalParam(numPath=npath, precision="fp64")
    first = rank * npath
    flush = torch.empty(64 << 20, dtype=torch.float32, device="cuda")

    def launch(num):
        if world > 1:
            return eng.enqueue_shard("dupire", "uoc", num, first, risk=True)
        return eng.enqueue("dupire", "uoc", num, risk=True)

    def timed(num, steps, warmup):
        for _ in range(warmup):
            launch(num)
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        launches = 0
        w0 = time.perf_counter()
        for k in range(steps):
            flush.fill_(float(k))
            evs[k][0].record(stream)
            launches += launch(num)
            evs[k][1].record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - w0
        ms = [a.elapsed_time(b) for a, b in evs]
        tot = sum(ms) / 1e3
        if world > 1:
            tt = torch.tensor([tot], device="cuda")
            torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
            tot = float(tt.item())
        return tot, ms, launches, wall

    with tempfile.TemporaryDirectory() as tmp:
        with Clocks(os.path.join(tmp, f"clocks_r{rank}.csv")) as ck:
            t32, ms32, launches, wall32 = timed(num32, args.steps, args.warmup)
        clocks = ck.summary()
    sharded = None
    if world > 1:
        from compfinance_gb300.shard import combine
        from compfinance_gb300.api import results_from_raw
        tot = combine(eng.fetch_raw())
        sv, se_, _, _ = results_from_raw(tot, npar, npay, world * npath)
        sharded = {"paths": world * npath, "ranks": world, "price": float(sv[0]), "price_stderr": float(se_[0])}
    v32, e32, agg32, r32 = eng.fetch(npay, npar)
    steps64 = max(2, min(args.steps, 4))
    t64, ms64, _, _ = timed(num64, steps64, 1)
    v64, e64, agg64, r64 = eng.fetch(npay, npar)

    # equal-error check: FP32 vs FP64 on the same paths, in Monte Carlo standard errors
    se = []
    for k in range(8):
        eng.enqueue("dupire", "uoc", NumericalParam(numPath=npath // 4, precision="fp32", seed1=1000 + k, seed2=77 + k),
                    risk=True)
        se.append(eng.fetch(npay, npar)[3])
    se = np.std(np.array(se), axis=0, ddof=1) / 2.0  # std at N/4 -> standard error at N
    mask = se > 1e-3 * np.abs(r64).max()
    risk_err_se = float(np.max(np.abs(r32 - r64)[mask] / se[mask]))
    price_err_se = float(abs(v32[0] - v64[0]) / e64[0])

    # end to end through the C ABI with host buffers
    h0, d0 = eng.transfer_stats()
    torch.cuda.synchronize()
    ke = max(2, min(args.steps, 5))
    w0 = time.perf_counter()
    for k in range(ke):
        eng.putDupire(W.DUPIRE_SPOT, s, t, v, W.DUPIRE_MAXDT, "dupire")
        eng.AADriskOne("dupire", "uoc", num32)
    e2e_t = (time.perf_counter() - w0) / ke
    h1, d1 = eng.transfer_stats()

    steps_tot = npath * dim
    per_step = t32 / args.steps
    value = world * npath / per_step
    pk = peaks()
    sm_max = float(pk.get("sm_max_mhz", 2070.0))
    peak_fp32 = 152 * 128 * 2 * sm_max * 1e6 / 1e12
    peak_fp64 = 152 * DFMA_PER_SM_PER_CYCLE * 2 * sm_max * 1e6 / 1e12
    achieved = FLOPS_PER_PATH_STEP * steps_tot / per_step / 1e12
    # DRAM bytes per launch: dram__bytes_read.sum + dram__bytes_write.sum of one ncu capture of
    # dupire_risk32 at 2^20 paths, per path-step, times the path-steps of this launch (same grid,
    # same scratch; the traffic grows with the path-steps)
    traffic = TRAFFIC_BYTES_PER_PATH_STEP * steps_tot if npath == NPATH else None
    out = {
        "metric": METRIC, "value": value, "unit": "paths/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": per_step * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": config,
        "path_steps_per_s": value * dim,
        "fp64": {"value": world * npath / (t64 / steps64), "unit": "paths/s", "ms_per_step": t64 / steps64 * 1e3,
                 "steps": steps64,
                 # the same 53 algorithmic flops per path-step against the FP64 FMA peak; the kernel's
                 # FP64 pipe itself is busier (comparisons, conversions, division/log/exp sequences)
                 "roofline": {"bound": "fp64_pipe",
                              "achieved": FLOPS_PER_PATH_STEP * steps_tot / (t64 / steps64) / 1e12,
                              "peak": peak_fp64, "unit": "TFLOP/s",
                              "frac": FLOPS_PER_PATH_STEP * steps_tot / (t64 / steps64) / 1e12 / peak_fp64,
                              "fp64_pipe_busy_ncu": FP64_PIPE_BUSY_NCU,
                              "peak_source": "152 SM x 2 DFMA x 2 x sm_max_mhz of MEASURED_PEAKS.json (the "
                                             "DFMA peak ncu reports; the file measures no FP64 peak)"}},
        "fp32_over_fp64": (t64 / steps64) / per_step,
        "equal_error": {"price_fp32_minus_fp64_in_stderr": price_err_se,
                        "max_risk_fp32_minus_fp64_in_stderr": risk_err_se,
                        "price": float(v64[0]), "price_stderr": float(e64[0])},
        "roofline": {"bound": "fp32_simt", "achieved": achieved, "peak": peak_fp32, "unit": "TFLOP/s",
                     "frac": achieved / peak_fp32, "traffic": traffic,
                     "peak_source": "152 SM x 128 FP32 lanes x 2 x sm_max_mhz of MEASURED_PEAKS.json "
                                    "(no tensor-core or HBM bound applies)",
                     "flops_per_path_step": FLOPS_PER_PATH_STEP,
                     # the same launch against the HBM roofline: its measured DRAM bytes (the
                     # reverse-sweep scratch) over the launch time, of the measured copy bandwidth
                     "hbm": ({"achieved_gbs": traffic / per_step / 1e9, "peak_gbs": pk.get("hbm_gbs"),
                              "frac": traffic / per_step / 1e9 / pk["hbm_gbs"]}
                             if traffic and pk.get("hbm_gbs") else None),
                     # and against instruction issue, its actual bound: thread instructions per
                     # path-step (smsp__inst_executed x active lanes, same ncu capture) over the
                     # launch time, of 152 SMs x 4 schedulers x 32 lanes x sm_max_mhz
                     "issue": {"achieved_tinst_per_s": INST_PER_PATH_STEP * steps_tot / per_step,
                               "peak_tinst_per_s": 152 * 4 * 32 * sm_max * 1e6,
                               "frac": INST_PER_PATH_STEP * steps_tot / per_step / (152 * 4 * 32 * sm_max * 1e6),
                               "inst_per_path_step": INST_PER_PATH_STEP}},
        "e2e": {"value": world * npath / e2e_t, "unit": "paths/s", "h2d_bytes_per_step": (h1 - h0) // ke,
                "d2h_bytes_per_step": (d1 - d0) // ke},
        "gpu_launches": launches,
        "sharded_run": sharded,
        "clocks": clocks,
        "step_ms": [round(x, 4) for x in ms32],
    }
    def leg(key, fn, *a, **k):
        """An auxiliary measurement: a failure is reported in the line, not fatal to it."""
        try:
            out[key] = fn(*a, **k)
        except Exception as e:  # noqa: BLE001
            out[key] = {"error": f"{type(e).__name__}: {e}"}

    if not args.no_sweep:
        leg("grid_sweep", grid_sweep, eng, stream, flush, npath)
        leg("superbucket", superbucket_leg, eng)
        leg("bump_risk", bump_leg, eng)
        leg("multi_asset", multi_asset_leg, eng)
    if not args.no_serving:
        leg("serving", serving_leg, eng, args.serve_requests, seed=2026 + rank)
    if rank == 0 and not args.no_cpu:
        leg("cpu_baseline", cpu_baseline)
        if "multi_asset" in out and "error" not in out["multi_asset"]:
            try:
                out["multi_asset"]["cpu_baseline"] = cpu_multi_asset()
            except Exception as e:  # noqa: BLE001
                out["multi_asset"]["cpu_baseline"] = {"error": f"{type(e).__name__}: {e}"}
    if rank == 0:
        print(json.dumps(out))
    eng.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
