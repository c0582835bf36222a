"""The bucket grid of the FP32 Dupire kernels (cf_bucket_grid, host code, no GPU).

dupire_risk32 finds a state's interval among the log-spot knots with one comparison: bucket
b = trunc(clamp((x - x0) * invW)) in FP32, then upper_bound(x) = first[b] + (knot first[b] <= x).
That is exact only because the host places the buckets so that no knot lies near an edge, where
the FP32 index can be one off.  These tests take the grid from the library and replay the
kernel's arithmetic in float32 on points spread over the grid and crowded around every edge and
knot, against the exact upper_bound."""
import ctypes

import numpy as np
import pytest

from compfinance_gb300 import workloads as W
from compfinance_gb300.api import lib

f32 = np.float32


def grid(knots):
    k = np.ascontiguousarray(knots, dtype=f32)
    x0, iw = ctypes.c_float(), ctypes.c_float()
    n, ok, one = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    fp = ctypes.POINTER(ctypes.c_float)
    assert lib().cf_bucket_grid(k.ctypes.data_as(fp), len(k), 0, ctypes.byref(x0), ctypes.byref(iw), ctypes.byref(n),
                                ctypes.byref(ok), ctypes.byref(one), None) == 0
    first = np.zeros(n.value, dtype=np.int32)
    assert lib().cf_bucket_grid(k.ctypes.data_as(fp), len(k), n.value, None, None, ctypes.byref(n), None, None,
                                first.ctypes.data_as(ctypes.POINTER(ctypes.c_int))) == 0
    return f32(x0.value), f32(iw.value), first, bool(ok.value), bool(one.value)


def kernel_search(x, knots, x0, iw, first):
    """The kernel's search, in float32: (x - x0) * invW, clamp, truncate, one comparison."""
    xs = np.concatenate([[-np.inf], knots, [np.inf]]).astype(f32)  # sentinel knot table
    fb = (x - x0).astype(f32) * iw
    fb = np.minimum(np.maximum(fb.astype(f32), f32(0)), f32(len(first) - 1))
    b = np.trunc(fb).astype(np.int64)
    l0 = first[b]
    return np.minimum(l0 + (xs[l0 + 1] <= x), len(knots))


def probe_points(knots, x0, iw, nb, rs):
    w = 1.0 / float(iw)
    pts = [rs.uniform(float(knots[0]) - 1.0, float(knots[-1]) + 1.0, 20000)]
    for e in float(x0) + np.arange(nb) * w:  # around every bucket edge
        pts.append(e + np.linspace(-3e-6, 3e-6, 13))
    for k in knots:  # around every knot, and its float neighbours
        pts.append(float(k) + np.linspace(-3e-6, 3e-6, 13))
    x = np.concatenate(pts).astype(f32)
    extra = [np.nextafter(knots, f32(np.inf)), np.nextafter(knots, f32(-np.inf)), knots,
             np.array([-np.inf, np.inf, -50.0, 50.0], dtype=f32)]
    return np.concatenate([x] + extra).astype(f32)


def knot_sets():
    rs = np.random.RandomState(5)
    sets = [W.dupire_surface(*g)[0] for g in ((20, 10), (60, 30), (120, 60))]
    sets += [np.array([100.0]), np.array([73.0])]  # one knot: local vol flat in spot
    sets += [50.0 * 4.0 ** (np.arange(n) / (n - 1)) for n in (2, 3, 7, 60, 121, 350, 510)]  # log-spaced
    sets += [np.linspace(50.0, 200.0, n) for n in (5, 60, 255, 500)]  # evenly spaced in spot
    sets += [np.sort(rs.uniform(40.0, 250.0, n)) for n in (5, 17, 60, 200) for _ in range(5)]
    return [np.unique(np.log(np.asarray(s, float) / 100.0).astype(f32)) for s in sets]


@pytest.mark.parametrize("i", range(len(knot_sets())))
def test_one_comparison_search_is_exact(i):
    knots = knot_sets()[i]
    x0, iw, first, ok, one = grid(knots)
    if not ok:
        pytest.skip("knots too close for the bucket table: the generic kernel runs")
    # at most one knot per bucket
    assert np.all(np.diff(first) <= 1)
    assert one, "no bucket grid keeps the knots away from the edges"
    x = probe_points(knots, x0, iw, len(first), np.random.RandomState(i))
    truth = np.searchsorted(knots, x, side="right")
    got = kernel_search(x, knots, x0, iw, first)
    assert np.array_equal(got, truth), np.nonzero(got != truth)[0][:5]


def test_benchmark_grids_run_the_fast_kernel():
    for g in ((20, 10), (60, 30), (120, 60)):
        knots = np.log(np.asarray(W.dupire_surface(*g)[0], float) / 100.0).astype(f32)
        _, _, first, ok, one = grid(knots)
        assert ok and one and len(first) <= 4098


def test_rejects_unsorted_knots():
    k = np.array([0.0, 0.5, 0.2], dtype=f32)
    n = ctypes.c_int()
    rc = lib().cf_bucket_grid(k.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), 3, 0, None, None, ctypes.byref(n),
                              None, None, None)
    assert rc != 0
