// Dupire calibration to an implied-vol surface and its adjoint, FP64 (mcMdlDupire.h:285-388,
// ivs.h:103-138, analytics.h:8-56).
//
// Local vol at (K, T) is Dupire's formula on finite differences of Black-Scholes calls priced
// off the implied surface plus the risk view's spreads: 5 calls per node, central difference
// in T and second difference in K with step 1e-4.  The adjoint maps local-vol adjoints (the
// Monte Carlo microbucket) back to the risk view's spread nodes.
#include <cuda_runtime.h>

#include "calib_params.h"
#include "cf_device.cuh"

namespace cf {



__device__ double dnormal_dens(double x) { return x < -10.0 || 10.0 < x ? 0.0 : exp(-0.5 * x * x) / 2.506628274631; }

__device__ double dnormal_cdf(double x)  // Zelen-Severo, gaussians.h:21-41
{
    if (x < -10.0) return 0.0;
    if (x > 10.0) return 1.0;
    const bool neg = x < 0.0;
    const double a = neg ? -x : x;
    const double t = 1.0 / (1.0 + 0.2316419 * a);
    const double pol =
        t * (0.319381530 + t * (-0.356563782 + t * (1.781477937 + t * (-1.821255978 + t * 1.330274429))));
    const double v = 1.0 - dnormal_dens(a) * pol;
    return neg ? 1.0 - v : v;
}

__device__ double dbs(double spot, double strike, double vol, double mat)
{
    const double sd = vol * sqrt(mat);
    if (sd <= 1.0e-08) return spot - strike > 0.0 ? spot - strike : 0.0;
    const double d2 = log(spot / strike) / sd - 0.5 * sd;
    const double d1 = d2 + sd;
    return spot * dnormal_cdf(d1) - strike * dnormal_cdf(d2);
}

// d call / d vol with the tape's rule for normalCdf (derivative = normalDens, AADExpr.h:434-447).
__device__ double dbs_vega(double spot, double strike, double vol, double mat)
{
    const double sq = sqrt(mat), sd = vol * sq;
    if (sd <= 1.0e-08) return 0.0;
    const double lg = log(spot / strike);
    const double d2 = lg / sd - 0.5 * sd;
    const double d1 = d2 + sd;
    const double dd2 = -lg / (sd * sd) - 0.5;
    return (spot * dnormal_dens(d1) * (dd2 + 1.0) - strike * dnormal_dens(d2) * dd2) * sq;
}

__device__ double dbs_ivol(double spot, double strike, double prem, double mat)  // analytics.h:23-56
{
    if (prem <= (spot - strike > 0.0 ? spot - strike : 0.0) + 1.0e-08) return 0.0;
    double u = 0.5;
    for (int it = 0; it < 64 && dbs(spot, strike, u, mat) < prem; ++it) u *= 2;
    double l = 0.05;
    for (int it = 0; it < 64 && dbs(spot, strike, l, mat) > prem; ++it) l /= 2;
    double pu = dbs(spot, strike, u, mat), pl = dbs(spot, strike, l, mat);
    for (int it = 0; it < 200 && u - l > 1.e-12; ++it)
    {
        const double m = 0.5 * (u + l), pm = dbs(spot, strike, m, mat);
        if (pm > prem) { u = m; pu = pm; }
        else { l = m; pl = pm; }
    }
    return l + (prem - pl) / (pu - pl) * (u - l);
}

__device__ double dmerton(double spot, double strike, double vol, double mat, double intens, double meanJmp,
                          double stdJmp)
{
    const double varJmp = stdJmp * stdJmp, mv2 = meanJmp + 0.5 * varJmp, comp = intens * (exp(mv2) - 1),
                 var = vol * vol, intensT = intens * mat;
    unsigned fact = 1;
    double iT = 1.0, res = 0.0;
    for (int n = 0; n < 10; ++n)
    {
        const double s = spot * exp(n * mv2 - comp * mat), v = sqrt(var + n * varJmp / mat);
        res += exp(-intensT) * iT / fact * dbs(s, strike, v, mat);
        fact *= unsigned(n + 1);
        iT *= intensT;
    }
    return res;
}

__device__ double dimplied(const CalibParams& p, double K, double T)
{
    if (p.ivsKind == 0)
    {
        const double l = log(K / p.ivp[3]);
        return p.ivp[0] + p.ivp[1] * l * l / sqrt(T) + p.ivp[2] * l;
    }
    return dbs_ivol(p.spot, K, dmerton(p.spot, K, p.ivp[0], T, p.ivp[1], p.ivp[2], p.ivp[3]), T);
}

// Finite-difference point p of node (K, T): 0 (K,T), 1 (K,T-h), 2 (K,T+h), 3 (K-h,T), 4 (K+h,T).
__device__ __forceinline__ void fd_point(int pt, double K, double T, double& Kp, double& Tp)
{
    Kp = K;
    Tp = T;
    if (pt == 1) Tp = T - 1.0e-04;
    if (pt == 2) Tp = T + 1.0e-04;
    if (pt == 3) Kp = K - 1.0e-04;
    if (pt == 4) Kp = K + 1.0e-04;
}

__device__ int rv_weights(const CalibParams& p, double K, double T, int* node, double* w);

__global__ void calib_points_kernel(CalibParams p)
{
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= p.nT * p.nS * 5) return;
    const int pt = idx % 5, i = (idx / 5) % p.nS, j = idx / (5 * p.nS);
    if (i < p.il[j] || i > p.ih[j]) return;
    double Kp, Tp;
    fd_point(pt, p.spots[i], p.times[j], Kp, Tp);
    double vol = dimplied(p, Kp, Tp);
    if (p.spreads)  // IVS::call adds the risk view's smoothstep-interpolated spread (ivs.h:103-116)
    {
        int node[4];
        double w[4];
        const int n = rv_weights(p, Kp, Tp, node, w);
        double sp = 0.0;
        for (int q = 0; q < n; ++q) sp += w[q] * p.spreads[node[q]];
        vol += sp;
    }
    p.c[idx] = dbs(p.spot, Kp, vol, Tp);
    p.vega[idx] = dbs_vega(p.spot, Kp, vol, Tp);
}

__global__ void calib_lvol_kernel(CalibParams p)
{
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= p.nT * p.nS) return;
    const int i = idx % p.nS, j = idx / p.nS;
    int src = i;
    if (i < p.il[j]) src = p.il[j];
    if (i > p.ih[j]) src = p.ih[j];
    const double* c = p.c + (size_t(j) * p.nS + src) * 5;
    const double ct = (c[2] - c[1]) * 0.5e04;
    const double ckk = (c[3] + c[4] - 2.0 * c[0]) * 1.0e08;
    p.lvT[idx] = sqrt(2.0 * ct / ckk) / p.spots[src];
}

// Smoothstep interpolation weights of the risk view at (K, T) (interp.h:66-109 with
// smoothStep = true): up to 4 (node, weight) pairs.
__device__ int rv_weights(const CalibParams& p, double K, double T, int* node, double* w)
{
    auto axis = [](const double* x, int n, double x0, int& a, int& b, double& wb) {
        int lo = 0, hi = n;
        while (lo < hi)
        {
            const int mid = (lo + hi) >> 1;
            if (x[mid] > x0) hi = mid;
            else lo = mid + 1;
        }
        if (lo == n || lo == 0)
        {
            a = b = lo == 0 ? 0 : n - 1;
            wb = 0.0;
            return;
        }
        a = lo - 1;
        b = lo;
        const double t = (x0 - x[a]) / (x[b] - x[a]);
        wb = t * t * (3.0 - 2 * t);
    };
    int ra, rb, ca, cb;
    double wr, wc;
    axis(p.rvK, p.nK, K, ra, rb, wr);
    axis(p.rvM, p.nM, T, ca, cb, wc);
    int n = 0;
    const int rr[2] = {ra, rb}, cc[2] = {ca, cb};
    const double wrr[2] = {1.0 - wr, wr}, wcc[2] = {1.0 - wc, wc};
    for (int x = 0; x < 2; ++x)
        for (int y = 0; y < 2; ++y)
        {
            const double ww = wrr[x] * wcc[y];
            if (ww == 0.0 || (x == 1 && rb == ra) || (y == 1 && cb == ca)) continue;
            node[n] = rr[x] * p.nM + cc[y];
            w[n++] = ww;
        }
    return n;
}

__global__ void calib_adjoint_kernel(CalibParams p)
{
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= p.nT * p.nS * 5) return;
    const int pt = idx % 5, i = (idx / 5) % p.nS, j = idx / (5 * p.nS);
    if (i < p.il[j] || i > p.ih[j]) return;
    const double a = p.seed[size_t(i) * p.nT + j];
    if (a == 0.0) return;
    const double K = p.spots[i];
    const double* c = p.c + (size_t(j) * p.nS + i) * 5;
    const double ct = (c[2] - c[1]) * 0.5e04;
    const double ckk = (c[3] + c[4] - 2.0 * c[0]) * 1.0e08;
    // sigma = sqrt(2 ct / ckk) / K
    const double u = 2.0 * ct / ckk;
    const double dsdu = 0.5 / sqrt(u) / K;
    const double dct = dsdu * 2.0 / ckk, dckk = -dsdu * 2.0 * ct / (ckk * ckk);
    const double dc = pt == 0 ? -2.0e08 * dckk : pt == 1 ? -0.5e04 * dct : pt == 2 ? 0.5e04 * dct : 1.0e08 * dckk;
    const double av = a * dc * p.vega[idx];
    if (p.pointAdj) p.pointAdj[idx] = av;
    double Kp, Tp;
    fd_point(pt, K, p.times[j], Kp, Tp);
    int node[4];
    double w[4];
    const int n = rv_weights(p, Kp, Tp, node, w);
    for (int q = 0; q < n; ++q) fix_add(&p.acc[2 * node[q]], av * w[q]);
}

int launch_calib(const CalibParams& p, int adjoint, void* stream)
{
    const int n5 = p.nT * p.nS * 5, n1 = p.nT * p.nS;
    if (adjoint)
    {
        calib_adjoint_kernel<<<(n5 + 127) / 128, 128, 0, (cudaStream_t)stream>>>(p);
        return (int)cudaGetLastError();
    }
    calib_points_kernel<<<(n5 + 127) / 128, 128, 0, (cudaStream_t)stream>>>(p);
    calib_lvol_kernel<<<(n1 + 127) / 128, 128, 0, (cudaStream_t)stream>>>(p);
    return (int)cudaGetLastError();
}

}  // namespace cf
