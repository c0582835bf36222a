// The Monte Carlo valuation / adjoint kernel.
//
// One thread owns a work unit: an antithetic pair of paths for mrg32k3a (both paths share
// one Gaussian vector, the second negated: mrg32k3a.h:150-184), or one path for Sobol
// (the 32 lanes of a warp take 32 consecutive Sobol indices).  Per unit the kernel runs
//   forward:  Gaussians -> model step (Dupire log-Euler with linear interpolation in log
//             spot, mcMdlDupire.h:238-280; or exact Black-Scholes steps, mcMdlBS.h:321-350)
//             -> product events (mcPrd.h payoffs), storing the per-step state it needs later;
//   reverse:  (risk launches) the hand-written adjoint of the same operations, step by step
//             from maturity back to today, replacing the reference's tape
//             (mcBase.h:427-532 records ~5 nodes per step and sweeps them back).
// Node adjoints of the local-vol grid, parameter adjoints and payoff sums are added to a
// block-private shared-memory slab in exact fixed point, flushed once per block.  In the
// FP32 form the local-vol adjoints first go through a per-warp row of the current step (see
// ROW_SHIFT in cf_params.h): two native 32-bit shared adds per path-step instead of four
// 64-bit ones, and one exact weighted add per touched grid spot per warp and step.
#pragma once
#include <type_traits>

#include "cf_device.cuh"

namespace cf {

constexpr int MC_BLOCK = 128;

template <class R>
__device__ __forceinline__ const R* pick(const double* d, const float* f);
template <>
__device__ __forceinline__ const double* pick<double>(const double* d, const float*) { return d; }
template <>
__device__ __forceinline__ const float* pick<float>(const double*, const float* f) { return f; }

__host__ __device__ inline size_t align16(size_t x) { return (x + 15) & ~size_t(15); }

// Shared-memory carve-up; identical on host (sizing) and device (pointers).
struct SmemLayout
{
    size_t slab, node, rows, mbar, claim, X, inv, bucket, Y, base, total;
};

__host__ __device__ inline SmemLayout mc_layout(int model, int rng, int fp32, int stageY, const McParams& p,
                                                int block)
{
    SmemLayout L;
    const size_t rs = fp32 ? 4 : 8;
    size_t off = 0;
    // slab: 4 scalar parameter adjoints + payoff / aggregate sums, two words each
    L.slab = off;
    off += align16(size_t(4 + 2 * p.nPay + 2) * 16);
    // local-vol node adjoints: one word each in the FP32 form, two in the FP64 form
    L.node = off;
    if (model == MODEL_DUPIRE && p.nRisk > 0) off += align16(size_t(p.nS) * p.nT * (fp32 ? 8 : 16));
    // FP32 form: one int32 row of the current step's vol adjoints per warp
    L.rows = off;
    if (model == MODEL_DUPIRE && p.nRisk > 0 && fp32) off += align16(size_t(block / 32) * p.nS * 4);
    L.mbar = off;
    off += 16;
    L.claim = off;  // the block's claimed chunk of unit rounds (first round, rounds)
    off += 16;
    L.X = L.inv = L.bucket = L.Y = L.base = off;
    if (model == MODEL_DUPIRE)
    {
        L.X = off;
        off += align16(size_t(p.nS) * rs);
        L.inv = off;
        off += align16(size_t(p.nS) * rs);
        L.bucket = off;
        off += align16(size_t(p.nBuckets) * 4);
        L.Y = off;
        if (stageY) off += align16(size_t(p.nSteps) * p.nS * rs);
    }
    L.base = off;
    if (rng == RNG_SOBOL) off += align16(size_t(block / 32) * (size_t(p.nSteps) | 1) * 4);
    L.total = off;
    return L;
}

template <int MODEL, int PROD, int RNGK, class Real, bool RISK>
__global__ void __launch_bounds__(MC_BLOCK) mc_kernel(const McParams p)
{
    constexpr int NP = RNGK == RNG_MRG ? 2 : 1;
    constexpr bool F32 = std::is_same<Real, float>::value;
    // FP32 local-vol adjoints gathered through per-warp step rows (the warp's step loops then
    // stay converged: lanes without a unit run them with no paths)
    constexpr bool ROWACC = F32 && MODEL == MODEL_DUPIRE && RISK;
    extern __shared__ __align__(128) unsigned char smem[];

    const SmemLayout L = mc_layout(MODEL, RNGK, F32, p.stageY, p, MC_BLOCK);
    long long* slab = reinterpret_cast<long long*>(smem + L.slab);  // scalar adjoints [0,4), payoffs from 8
    long long* paySlab = slab + 8;
    long long* node = reinterpret_cast<long long*>(smem + L.node);
    const int tid = threadIdx.x;
    const int lane = tid & 31;
    const int nNodes = (MODEL == MODEL_DUPIRE && RISK) ? p.nS * p.nT : 0;
    const int nodeWords = nNodes * (F32 ? 1 : 2);
    int* rows = reinterpret_cast<int*>(smem + L.rows) + (tid >> 5) * p.nS;  // this warp's row
    for (int i = tid; i < 2 * (4 + 2 * p.nPay + 2); i += MC_BLOCK) slab[i] = 0;
    for (int i = tid; i < nodeWords; i += MC_BLOCK) node[i] = 0;
    if (ROWACC)
        for (int i = tid; i < (MC_BLOCK / 32) * p.nS; i += MC_BLOCK) reinterpret_cast<int*>(smem + L.rows)[i] = 0;

    const int nSteps = p.nSteps;
    const int nS = p.nS, nT = p.nT;
    Real* sX = reinterpret_cast<Real*>(smem + L.X);
    Real* sInv = reinterpret_cast<Real*>(smem + L.inv);
    int* sBucket = reinterpret_cast<int*>(smem + L.bucket);
    const Real* Y = pick<Real>(p.Yd, p.Yf);
    if (MODEL == MODEL_DUPIRE)
    {
        const Real* gX = pick<Real>(p.Xd, p.Xf);
        const Real* gI = pick<Real>(p.invdXd, p.invdXf);
        for (int i = tid; i < nS; i += MC_BLOCK)
        {
            sX[i] = gX[i];
            sInv[i] = gI[i];
        }
        for (int i = tid; i < p.nBuckets; i += MC_BLOCK) sBucket[i] = p.bucket[i];
        if (p.stageY)
        {
            Real* sY = reinterpret_cast<Real*>(smem + L.Y);
            const unsigned bytes = (unsigned)align16(size_t(nSteps) * nS * sizeof(Real));
            // a copy that did not complete fails the launch (error flag): the block returns
            if (!bulk_copy_to_smem(sY, Y, bytes, reinterpret_cast<unsigned long long*>(smem + L.mbar), p.err))
                return;
            Y = sY;
        }
    }
    __syncthreads();

    const Real* bs = pick<Real>(p.bsD, p.bsF);
    const Real* ev = pick<Real>(p.evD, p.evF);
    const Real* kK = pick<Real>(p.kD, p.kF);
    const Real* cA = pick<Real>(p.cAd, p.cAf);
    const Real* cB = pick<Real>(p.cBd, p.cBf);
    const Real* wts = pick<Real>(p.w, p.wf);
    const int nEv = p.nEv;
    const int nPay = p.nPay;
    const int payBase = 0, sqBase = nPay, aggBase = 2 * nPay;  // in paySlab
    const Real strike = (Real)p.strike, barSmooth = (Real)p.barSmooth, minusSmooth = (Real)p.minusSmooth,
               twoSmooth = (Real)p.twoSmooth;
    const Real logBand = F32 ? (Real)p.logBandF : (Real)p.logBandD;
    // state variable: FP64 form x = log S; FP32 form y = log S - log spot, S = s0 * exp(y)
    const Real xStart = F32 ? Real(0) : (Real)p.x0d;
    const Real sScale = F32 ? (Real)p.s0f : Real(1);
    const Real spot = (Real)p.spot;
    const Real w0 = nPay > 0 ? wts[0] : Real(0), w1 = nPay > 1 ? wts[1] : Real(0);
    const Real cpn = (Real)p.coupon, cbSmooth = (Real)p.cbSmooth, cbTwo = Real(2) * (Real)p.cbSmooth;

    const long long T = (long long)gridDim.x * MC_BLOCK;
    const long long tg = (long long)blockIdx.x * MC_BLOCK + tid;
    // scratch element (field f, timeline point i) of this thread; the host keeps the whole
    // scratch below 2^31 elements so the offsets are 32-bit
    Real* scr = reinterpret_cast<Real*>(p.scratch) + tg;
    const int Ti = int(T);
    const int rowStride = (nSteps + 1) * Ti;
    auto SCR = [&](int f, int i) -> Real& { return scr[f * rowStride + i * Ti]; };
    constexpr int F_G = 0, F_X = 1, F_AL = 1 + NP;

    auto spotOf = [&](Real xs) -> Real {
        if (MODEL == MODEL_DUPIRE) return sScale * exp(xs);
        return xs;
    };

    // Interpolation of row s of Y at state xs: first knot above xs (upper_bound), linear
    // weight t, value v and slope dv/dx; flat extrapolation at both ends (interp.h:26-63).
    const Real bX0 = F32 ? (Real)p.bX0f : (Real)p.bX0d;
    const Real bInvW = F32 ? (Real)p.bInvWf : (Real)p.bInvWd;
    const int nB = p.nBuckets;
    auto interpRow = [&](int s, Real xs, int& k, Real& t, Real& v, Real& slope, bool& flat) {
        // upper_bound(X, xs): bucket guess, then exact adjustment in both directions
        const Real fb = (xs - bX0) * bInvW;
        int b = fb > Real(0) ? int(fb) : 0;
        b = b < nB - 1 ? b : nB - 1;
        int lo = sBucket[b];
        while (lo < nS && !(sX[lo] > xs)) ++lo;
        while (lo > 0 && sX[lo - 1] > xs) --lo;
        const Real* row = Y + size_t(s) * nS;
        if (lo == nS || lo == 0)
        {
            k = lo == 0 ? 0 : nS - 1;
            flat = true;
            t = Real(0);
            v = row[k];
            slope = Real(0);
        }
        else
        {
            k = lo - 1;
            flat = false;
            const Real y1 = row[k], y2 = row[k + 1];
            t = (xs - sX[k]) * sInv[k];
            v = y1 + (y2 - y1) * t;
            slope = (y2 - y1) * sInv[k];
        }
    };

    // FP32 local-vol adjoints.  rowAdd: contribution c to spot j of step s's vol row, into the
    // warp's row (or, when |c| >= ROW_MAX, exactly into the global accumulators of the two
    // nodes the row interpolates).  nodeAdd: an exact int64 product, in units of
    // 2^-NODE_SHIFT, into the block's node slab (or global when it could overflow the slab).
    // rowFlush: after step s, the warp moves its row into the nodes (time weights W of s).
    auto rowAdd = [&](int s, int j, float c) {
        if (c == 0.0f) return;
        if (fabsf(c) < ROW_MAX)
            atomicAdd(&rows[j], __float2int_rn(c * float(1 << ROW_SHIFT)));
        else
        {
            fix_add(&p.acc[2 * (1 + j * nT + p.colA[s])], c * p.cAf[s]);
            if (p.cBf[s] != 0.0f) fix_add(&p.acc[2 * (1 + j * nT + p.colB[s])], c * p.cBf[s]);
        }
    };
    auto nodeAdd = [&](int idx, long long v) {
        constexpr long long LIM = 1LL << 50;
        if (!p.nodeDirect && v < LIM && v > -LIM)
            atomicAdd(reinterpret_cast<unsigned long long*>(&node[idx]), (unsigned long long)v);
        else
            node_flush(&p.acc[2 * (1 + idx)], v);
    };
    auto rowFlush = [&](int s) {
        __syncwarp();
        const long long WA = p.wAi[s], WB = p.wBi[s];
        const int ca = p.colA[s], cb = p.colB[s];
        for (int j = lane; j < nS; j += 32)
        {
            const int r = rows[j];
            if (r != 0)
            {
                rows[j] = 0;
                nodeAdd(j * nT + ca, WA * r);
                if (WB != 0) nodeAdd(j * nT + cb, WB * r);
            }
        }
        __syncwarp();
    };

    // ---------------------------------------------------------------------------------
    // One work unit: nAct (0, 1 or 2) paths driven by the Gaussian generator gen(i); path0 is
    // the launch-local index of its first path (value launches with p.pathOut write every
    // path's payoffs there, [path][nPay]).
    // ---------------------------------------------------------------------------------
    auto runUnit = [&](int nAct, long long path0, auto&& gen) {
        double* const po = RISK ? nullptr : p.pathOut;
        Real x[NP], alive[NP], euro[NP], fE[NP], dE[NP], nE[NP], agg[NP];
        Real cPrev[NP], cPay[NP];  // contingent bond: spot at the previous date, payoff so far
        bool dead[NP];
#pragma unroll
        for (int a = 0; a < NP; ++a)
        {
            x[a] = MODEL == MODEL_DUPIRE ? xStart : spot;
            alive[a] = Real(1);
            euro[a] = fE[a] = dE[a] = Real(0);
            nE[a] = Real(1);
            agg[a] = Real(0);
            cPrev[a] = cPay[a] = Real(0);
            dead[a] = false;
        }

        // forward event handling at timeline point i for product date e
        auto eventFwd = [&](int e, int i, int a) {
            const bool last = e == nEv - 1;
            Real S;
            // Up-and-out on Dupire: below the smoothing band (tested in log space with a margin
            // that dominates exp/log rounding) a monitoring date changes nothing.
            if (PROD == PROD_UOC && MODEL == MODEL_DUPIRE && !last && (dead[a] || !(x[a] > logBand))) return;
            S = spotOf(x[a]);
            Real F = S, D = Real(1), N = Real(1);
            if (MODEL == MODEL_BS)
            {
                F = S * ev[e];
                D = ev[2 * nEv + e];
                if (ev[6 * nEv + e] != Real(0)) N = p.spotMeasure ? ev[4 * nEv + e] * S : ev[4 * nEv + e];
            }
            if (PROD == PROD_EUROPEAN)
            {
                fE[a] = F;
                dE[a] = D;
                nE[a] = N;
            }
            else if (PROD == PROD_UOC)
            {
                if (!dead[a])
                {
                    if (F > barSmooth) dead[a] = true;
                    else if (F > minusSmooth)
                    {
                        if (RISK) SCR(F_AL + a, i) = alive[a];
                        alive[a] *= (barSmooth - F) / twoSmooth;
                    }
                }
                if (last)
                {
                    fE[a] = F;
                    nE[a] = N;
                    const Real m = p.callPut ? (strike - F) : (F - strike);
                    euro[a] = (m > Real(0) ? m : Real(0)) / N;
                }
            }
            else if (PROD == PROD_CONTINGENT)
            {
                // mcPrd.h:522-573: at the end of each period, (libor + coupon) x coverage when the
                // spot rose (a digital smoothed over +-smooth), paid at the period's end; the
                // redemption at maturity
                if (e > 0)
                {
                    const Real dlt = F - cPrev[a];
                    const Real dig = dlt > cbSmooth ? Real(1) : dlt < -cbSmooth ? Real(0) : (dlt + cbSmooth) / cbTwo;
                    cPay[a] += dig * (ev[7 * nEv + e - 1] + cpn) * ev[9 * nEv + e - 1] / N;
                }
                cPrev[a] = F;
                if (last) cPay[a] += Real(1) / N;
            }
            else
            {
                const int k0 = p.evPayOff[e], k1 = p.evPayOff[e + 1];
                for (int k = k0; k < k1; ++k)
                {
                    const Real m = F - kK[k];
                    const Real pay = (m > Real(0) ? m : Real(0)) / N;
                    if (pay != Real(0))
                    {
                        fix_add(&paySlab[2 * (payBase + k)], pay);
                        fix_add(&paySlab[2 * (sqBase + k)], pay * pay);
                    }
                    if (po) po[(path0 + a) * nPay + k] = double(pay);
                    if (RISK) agg[a] += wts[k] * pay;
                }
            }
        };

        {
            const int e0 = p.evAtStep[0];
            if (e0 >= 0)
                #pragma unroll
                for (int a = 0; a < NP; ++a)
                    if (a < nAct) eventFwd(e0, 0, a);
        }
        for (int i = 0; i < nSteps; ++i)
        {
            const Real g = nAct ? gen(i) : Real(0);
            if (RISK) SCR(F_G, i) = g;
#pragma unroll
            for (int a = 0; a < NP; ++a)
            {
                if (a >= nAct) break;
                const Real ga = a ? -g : g;
                if (RISK) SCR(F_X + a, i) = x[a];
                if (MODEL == MODEL_DUPIRE)
                {
                    int k;
                    Real t, v, slope;
                    bool flat;
                    interpRow(i, x[a], k, t, v, slope, flat);
                    x[a] += v * (Real(-0.5) * v + ga);
                }
                else
                {
                    x[a] = x[a] * exp(bs[i] + bs[nSteps + i] * ga);
                }
            }
            const int e = p.evAtStep[i + 1];
            if (e >= 0)
                #pragma unroll
                for (int a = 0; a < NP; ++a)
                    if (a < nAct) eventFwd(e, i + 1, a);
        }

        // payoffs and value sums
#pragma unroll
        for (int a = 0; a < NP; ++a)
        {
            if (a >= nAct) break;
            if (PROD == PROD_EUROPEAN)
            {
                const Real m = fE[a] - strike;
                const Real pay = (m > Real(0) ? m : Real(0)) * dE[a] / nE[a];
                fix_add(&paySlab[2 * payBase], pay);
                fix_add(&paySlab[2 * sqBase], pay * pay);
                agg[a] = w0 * pay;
                if (po) po[(path0 + a) * nPay] = double(pay);
            }
            else if (PROD == PROD_UOC)
            {
                const Real p0 = dead[a] ? Real(0) : alive[a] * euro[a];
                fix_add(&paySlab[2 * payBase], p0);
                fix_add(&paySlab[2 * sqBase], p0 * p0);
                fix_add(&paySlab[2 * (payBase + 1)], euro[a]);
                fix_add(&paySlab[2 * (sqBase + 1)], euro[a] * euro[a]);
                agg[a] = w0 * p0 + w1 * euro[a];
                if (po)
                {
                    po[(path0 + a) * nPay] = double(p0);
                    po[(path0 + a) * nPay + 1] = double(euro[a]);
                }
            }
            else if (PROD == PROD_CONTINGENT)
            {
                fix_add(&paySlab[2 * payBase], cPay[a]);
                fix_add(&paySlab[2 * sqBase], cPay[a] * cPay[a]);
                agg[a] = w0 * cPay[a];
                if (po) po[(path0 + a) * nPay] = double(cPay[a]);
            }
            if (RISK)
            {
                fix_add(&paySlab[2 * aggBase], agg[a]);
                fix_add(&paySlab[2 * (aggBase + 1)], agg[a] * agg[a]);
            }
        }
        if (!RISK) return;

        // ---------------------------------------------------------------------------
        // Reverse sweep.
        // ---------------------------------------------------------------------------
        Real ax[NP], aAlive[NP], aEuro[NP], aVol[NP], aR[NP], aDv[NP], aSp[NP];
        Real cAprev[NP];  // contingent bond: adjoint of the previous date's spot
#pragma unroll
        for (int a = 0; a < NP; ++a)
        {
            ax[a] = aVol[a] = aR[a] = aDv[a] = aSp[a] = Real(0);
            cAprev[a] = Real(0);
            aEuro[a] = dead[a] ? w1 : w0 * alive[a] + w1;       // payoff0 = alive*euro, payoff1 = euro
            aAlive[a] = dead[a] ? Real(0) : w0 * euro[a];
        }
        for (int i = nSteps; i >= 0; --i)
        {
            const int e = p.evAtStep[i];
            if (e >= 0)
            {
#pragma unroll
                for (int a = 0; a < NP; ++a)
                {
                    if (a >= nAct) break;
                    const Real xi = i == nSteps ? x[a] : SCR(F_X + a, i);
                    const bool last = e == nEv - 1;
                    if (PROD == PROD_UOC && MODEL == MODEL_DUPIRE && !last && (dead[a] || !(xi > logBand)))
                        continue;
                    const Real S = spotOf(xi);
                    Real F = S, D = Real(1), N = Real(1), ff = Real(1), nf = Real(0);
                    const bool needN = MODEL == MODEL_BS ? ev[6 * nEv + e] != Real(0) : false;
                    if (MODEL == MODEL_BS)
                    {
                        ff = ev[e];
                        F = S * ff;
                        D = ev[2 * nEv + e];
                        nf = ev[4 * nEv + e];
                        if (needN) N = p.spotMeasure ? nf * S : nf;
                    }
                    Real aF = Real(0), aD = Real(0), aN = Real(0);
                    if (PROD == PROD_EUROPEAN)
                    {
                        const Real m = F - strike;
                        if (m > Real(0))
                        {
                            aF = w0 * D / N;
                            aD = w0 * m / N;
                            aN = -w0 * m * D / (N * N);
                        }
                    }
                    else if (PROD == PROD_UOC)
                    {
                        if (last)
                        {
                            const Real m = p.callPut ? (strike - F) : (F - strike);
                            if (m > Real(0))
                            {
                                aF = (p.callPut ? -aEuro[a] : aEuro[a]) / N;
                                aN = -aEuro[a] * m / (N * N);
                            }
                        }
                        if (!dead[a] && F > minusSmooth)
                        {
                            const Real before = SCR(F_AL + a, i);
                            aF += aAlive[a] * before * (Real(-1) / twoSmooth);
                            aAlive[a] *= (barSmooth - F) / twoSmooth;
                        }
                    }
                    else if (PROD == PROD_CONTINGENT)
                    {
                        aF = cAprev[a];  // from the period that starts here
                        cAprev[a] = Real(0);
                        if (last) aN = -w0 / (N * N);
                        if (e > 0)
                        {
                            // the period ending here: its start spot from the state at its date
                            const Real xp = SCR(F_X + a, p.evPoint[e - 1]);
                            const Real Fp = MODEL == MODEL_BS ? spotOf(xp) * ev[e - 1] : spotOf(xp);
                            const Real dlt = F - Fp;
                            const Real L = ev[7 * nEv + e - 1], cov = ev[9 * nEv + e - 1];
                            const Real dig = dlt > cbSmooth ? Real(1) : dlt < -cbSmooth ? Real(0) : (dlt + cbSmooth) / cbTwo;
                            if (!(dlt > cbSmooth) && !(dlt < -cbSmooth))
                            {
                                const Real aDl = w0 * (L + cpn) * cov / N / cbTwo;
                                aF += aDl;
                                cAprev[a] = -aDl;
                            }
                            aN -= w0 * dig * (L + cpn) * cov / (N * N);
                            if (MODEL == MODEL_BS) aR[a] += w0 * dig * cov / N * ev[8 * nEv + e - 1];  // d libor / d r
                        }
                    }
                    else
                    {
                        const int k0 = p.evPayOff[e], k1 = p.evPayOff[e + 1];
                        for (int k = k0; k < k1; ++k)
                        {
                            const Real m = F - kK[k];
                            if (m > Real(0))
                            {
                                aF += wts[k] / N;
                                aN -= wts[k] * m / (N * N);
                            }
                        }
                    }
                    if (MODEL == MODEL_DUPIRE)
                    {
                        ax[a] += aF * S;  // F = S = exp(x)
                    }
                    else
                    {
                        const Real tauF = ev[nEv + e], tauD = ev[3 * nEv + e], te = ev[5 * nEv + e];
                        ax[a] += aF * ff;
                        const Real aff = aF * S * ff;  // d ff / d mu = tauF * ff
                        aR[a] += aff * tauF;
                        aDv[a] -= aff * tauF;
                        aR[a] -= aD * D * tauD;       // D = exp(-r tauD)
                        if (needN)
                        {
                            if (p.spotMeasure)        // N = exp(d t) / spot * S
                            {
                                ax[a] += aN * nf;
                                aDv[a] += aN * N * te;
                                aSp[a] -= aN * N / spot;
                            }
                            else                      // N = exp(r t)
                                aR[a] += aN * N * te;
                        }
                    }
                }
            }
            if (i == 0) break;
            const int s = i - 1;
            const Real g = SCR(F_G, s);
#pragma unroll
            for (int a = 0; a < NP; ++a)
            {
                if (a >= nAct) break;
                const Real ga = a ? -g : g;
                const Real xs = SCR(F_X + a, s);
                if (MODEL == MODEL_DUPIRE)
                {
                    int k;
                    Real t, v, slope;
                    bool flat;
                    interpRow(s, xs, k, t, v, slope, flat);
                    const Real q = ga - v;             // d x_{s+1} / d v
                    const Real av = ax[a] * q;
                    ax[a] += av * slope;               // d x_{s+1} / d x_s = 1 + q dv/dx
                    if (ROWACC)
                    {
                        rowAdd(s, k, flat ? av : av * (Real(1) - t));
                        if (!flat) rowAdd(s, k + 1, av * t);
                    }
                    else
                    {
                        const int ca = p.colA[s], cb = p.colB[s];
                        const Real wa = cA[s], wb = cB[s];
                        auto put = [&](int j, Real aY) {
                            if (aY == Real(0)) return;
                            fix_add(&node[2 * (j * nT + ca)], aY * wa);
                            if (wb != Real(0)) fix_add(&node[2 * (j * nT + cb)], aY * wb);
                        };
                        if (flat) put(k, av);
                        else
                        {
                            put(k, av * (Real(1) - t));
                            put(k + 1, av * t);
                        }
                    }
                }
                else
                {
                    const Real E = exp(bs[s] + bs[nSteps + s] * ga);
                    const Real aArg = ax[a] * (xs * E);  // d S_{s+1} / d(drift + std g) = S_{s+1}
                    aVol[a] += aArg * bs[4 * nSteps + s] + aArg * ga * bs[3 * nSteps + s];
                    aR[a] += aArg * bs[2 * nSteps + s];
                    aDv[a] -= aArg * bs[2 * nSteps + s];
                    ax[a] *= E;
                }
            }
            if (ROWACC) rowFlush(s);
        }
        if (MODEL == MODEL_DUPIRE)
        {
            Real sp = Real(0);
#pragma unroll
            for (int a = 0; a < NP; ++a)
                if (a < nAct) sp += ax[a];
            fix_add(&slab[0], sp / spot);  // x_0 = log(spot)
        }
        else
        {
            Real s0 = 0, s1 = 0, s2 = 0, s3 = 0;
#pragma unroll
            for (int a = 0; a < NP; ++a)
            {
                if (a >= nAct) break;
                s0 += ax[a] + aSp[a];
                s1 += aVol[a];
                s2 += aR[a];
                s3 += aDv[a];
            }
            fix_add(&slab[0], s0);
            fix_add(&slab[2], s1);
            fix_add(&slab[4], s2);
            fix_add(&slab[6], s3);
        }
    };

    // FP32 node slab flushed to the global hi/lo accumulators (block-wide).
    auto flushNodes = [&]() {
        __syncthreads();
        for (int i = tid; i < nNodes; i += MC_BLOCK)
        {
            node_flush(&p.acc[2 * (1 + i)], node[i]);
            node[i] = 0;
        }
        __syncthreads();
    };

    // Unit rounds (MC_BLOCK units of the generator, or MC_BLOCK / 32 Sobol batches of 32 paths)
    // are claimed from the launch's counter in chunks of G consecutive rounds, G shrinking with
    // the rounds left (guided self-scheduling, as in dupire_risk32), so that the blocks of an SM
    // all run until the work is gone; a thread runs the G units of its chunk that follow each
    // other in its generator, with one skip-ahead.
    long long* sClaim = reinterpret_cast<long long*>(smem + L.claim);
    long long it = 0;  // rounds this block has run (the FP32 node slab is flushed by this count)
    auto claim = [&](long long nRounds) {  // chunk [sClaim[0], sClaim[0] + sClaim[1]) (uniform)
        __syncthreads();  // every thread has read the previous chunk
        if (tid == 0)
        {
            const long long seen = (long long)*reinterpret_cast<volatile unsigned long long*>(p.claim);
            const long long g = (nRounds - seen) / (2LL * gridDim.x);
            sClaim[1] = g > 1 ? g : 1;
            sClaim[0] = (long long)atomicAdd(p.claim, (unsigned long long)sClaim[1]);
        }
        __syncthreads();
    };
    if (RNGK == RNG_MRG)
    {
        const long long nUnits = (p.nPath + 1) / 2;
        const long long nRounds = (nUnits + MC_BLOCK - 1) / MC_BLOCK;
        for (;;)
        {
            claim(nRounds);
            const long long r0 = sClaim[0], G = sClaim[1];
            if (r0 >= nRounds) break;
            const long long u0 = r0 * MC_BLOCK + tid * G;  // this thread's units u0 .. u0 + G - 1
            MrgState st{};
            if (u0 < nUnits) st = mrg_jump(p.seed1, p.seed2, (unsigned long long)(p.firstPath / 2 + u0) * nSteps, p.mrgJumpA, p.mrgJumpB);
            for (long long j = 0; j < G; ++j, ++it)
            {
                const long long u = u0 + j;
                const int nAct = u < nUnits ? ((2 * u + 1 < p.nPath) ? 2 : 1) : 0;
                if (ROWACC || nAct) runUnit(nAct, 2 * u, [&](int) { return mrg_gauss<Real>(mrg_next(st)); });
                if (ROWACC && (it + 1) % p.nodeFlushUnits == 0) flushNodes();
            }
        }
    }
    else
    {
        // Sobol: in round r warp w takes batch b = r (MC_BLOCK / 32) + w; lane l runs index
        // n = 32b + l (path n-1).  state(n) = state(32b) ^ state(l) (gray code is linear over
        // the disjoint bit ranges of 32b and l).
        const int wib = tid >> 5;
        const int pitch = nSteps | 1;
        unsigned* base = reinterpret_cast<unsigned*>(smem + L.base) + wib * pitch;
        constexpr int WB = MC_BLOCK / 32;
        const long long nBatches = p.nPath / 32 + 1;
        const long long nRounds = (nBatches + WB - 1) / WB;
        for (;;)
        {
            claim(nRounds);
            const long long r0 = sClaim[0], G = sClaim[1];
            if (r0 >= nRounds) break;
            for (long long j = 0; j < G; ++j, ++it)
            {
                const long long b = (r0 + j) * WB + wib;
                if (ROWACC && it > 0 && it % p.nodeFlushUnits == 0) flushNodes();
                if (b >= nBatches) continue;
                __syncwarp();
                for (int d = lane; d < nSteps; d += 32)
                    base[d] = sobol_state(p.sobolDir, nSteps, d, (unsigned long long)(p.firstPath + b * 32));
                __syncwarp();
                const long long n = b * 32 + lane;
                const int nAct = (n >= 1 && n <= p.nPath) ? 1 : 0;
                if (ROWACC || nAct)
                    runUnit(nAct, n - 1, [&](int i) {
                        return sobol_gauss<Real>(base[i] ^ sobol_state(p.sobolDir, nSteps, i, (unsigned long long)lane));
                    });
            }
        }
    }

    __syncthreads();
    // flush: scalar parameter adjoints, node adjoints, payoff sums
    if (RISK)
    {
        const int nScal = MODEL == MODEL_BS ? 4 : 1;
        for (int i = tid; i < nScal; i += MC_BLOCK) fix_flush(&p.acc[2 * i], &slab[2 * i]);
        for (int i = tid; i < nNodes; i += MC_BLOCK)
        {
            if (F32) node_flush(&p.acc[2 * (1 + i)], node[i]);
            else fix_flush(&p.acc[2 * (1 + i)], &node[2 * i]);
        }
    }
    for (int i = tid; i < 2 * nPay + 2; i += MC_BLOCK) fix_flush(&p.acc[2 * (p.nRisk + i)], &paySlab[2 * i]);
}

}  // namespace cf
