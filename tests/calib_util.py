"""Rounding scales of the Dupire calibration adjoint, shared by the CPU and GPU tests."""
import numpy as np


def support(spots, times, rk, rm, point_adj):
    """Per risk-view node, the sum of |adjoint| over the calibration points whose smoothstep
    interpolation cell (upper_bound in strike and maturity, flat outside) has the node as a
    corner, whatever the corner's weight: the scale on which rounding of the weights (~1e-16
    each) shows.  A point a last bit below a risk-view maturity gets weight 1 - s with s = 1 to
    rounding: exactly 0 as the GPU forms it, ~1e-16 through the reference's tape of
    z1 + (z2 - z1) s (interp.h:66-109), on point adjoints up to ~1e11."""
    import bisect
    out = np.zeros((len(rk), len(rm)))

    def cell(x, x0):
        k = bisect.bisect_right(x, x0)
        return (0, 0) if k == 0 else (len(x) - 1, len(x) - 1) if k == len(x) else (k - 1, k)
    for j, T in enumerate(times):
        for i, K in enumerate(spots):
            for pt, (Kp, Tp) in enumerate(((K, T), (K, T - 1.0e-04), (K, T + 1.0e-04), (K - 1.0e-04, T),
                                           (K + 1.0e-04, T))):
                a = abs(point_adj[j, i, pt])
                if a == 0.0:
                    continue
                rows, cols = set(cell(rk, Kp)), set(cell(rm, Tp))
                for r in rows:
                    for q in cols:
                        out[r, q] += a
    return out
