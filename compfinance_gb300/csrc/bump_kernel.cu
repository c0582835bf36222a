// Pathwise bump-and-reprice of a Dupire model (bumpRisk, main.h:316-359, for local-vol and
// spot bumps), FP64, the arithmetic of the FP64 valuation kernel.
//
// bumpRisk revalues the product once per model parameter, each parameter bumped by 1e-8 on
// the same random numbers.  A bumped local-vol node (spot j, time c) enters a path only at
// steps whose time interpolation weighs column c and whose spot interpolation weighs spot j;
// before the first such step the bumped path is the base path, bit for bit, and a path that
// never touches the node keeps its payoffs exactly.  So each thread simulates its paths once,
// records per point the state, per step the spot interval, and then, walking the steps, re-
// simulates the path from the first step that touches each node, with that node bumped, and
// adds the payoff differences (exact fixed point) to the node's accumulators.  The spot bump
// moves every path (and the barrier's smoothing width, which the product takes from the
// first spot of the path) and re-simulates each path from today.  The work per path is the
// number of nodes it touches (about a hundred on a 60x30 grid over 156 steps) times a partial
// path, against one full path per parameter (1801) for repricing.
#include <cuda_runtime.h>

#include "bump_params.h"
#include "cf_device.cuh"

namespace cf {

namespace {

constexpr int BB = 128;  // threads per block

template <int PROD, int RNGK>
__global__ void __launch_bounds__(BB) dupire_bump64(const McParams p, const BumpArgs b)
{
    constexpr int NP = RNGK == RNG_MRG ? 2 : 1;
    constexpr bool UOC = PROD == PROD_UOC, EUR = PROD == PROD_EUROPEAN;
    const int nSteps = p.nSteps, nS = p.nS, nT = p.nT, nPay = p.nPay, nEv = p.nEv;
    const long long Ti = (long long)gridDim.x * BB;
    const long long tg = (long long)blockIdx.x * BB + threadIdx.x;

    // scratch rows [row][thread] (the layout of bump_scratch_rows)
    double* dRow = static_cast<double*>(b.scratch);
    const BumpRows R = bump_rows(nSteps, nPay, NP, b.maskWords);
    auto D = [&](int row) -> double& { return dRow[size_t(row) * Ti + tg]; };
    int* iRow = reinterpret_cast<int*>(dRow + size_t(R.nDouble) * Ti);
    auto I = [&](int row) -> int& { return iRow[size_t(row) * Ti + tg]; };
    unsigned* mRow = reinterpret_cast<unsigned*>(iRow + size_t(R.nInt) * Ti);
    auto M = [&](int w) -> unsigned& { return mRow[size_t(w) * Ti + tg]; };

    // interval of the state (upper_bound with the bucket hint, mc_kernel's interpRow)
    auto locate = [&](double xs) -> int {
        const double fb = (xs - p.bX0d) * p.bInvWd;
        int bk = fb > 0.0 ? int(fb) : 0;
        bk = bk < p.nBuckets - 1 ? bk : p.nBuckets - 1;
        int lo = __ldg(p.bucket + bk);
        while (lo < nS && !(__ldg(p.Xd + lo) > xs)) ++lo;
        while (lo > 0 && __ldg(p.Xd + lo - 1) > xs) --lo;
        return lo;
    };
    // sqrt(dt) sigma of spot j at step s with node (j, bc) bumped: the host's interp_lin in
    // time, rounded like the host (no contraction)
    auto yBumped = [&](int s, int j, int bc) -> double {
        const int ca = __ldg(p.colA + s), cb = __ldg(p.colB + s);
        double va = __ldg(p.volsD + size_t(j) * nT + ca), vb = __ldg(p.volsD + size_t(j) * nT + cb);
        if (ca == bc) va = __dadd_rn(va, BUMP_SIZE);
        if (cb == bc && cb != ca) vb = __dadd_rn(vb, BUMP_SIZE);
        const double sq = __ldg(p.stepSqD + s);
        if (ca == cb) return __dmul_rn(sq, va);
        return __dmul_rn(sq, __dadd_rn(va, __dmul_rn(__dsub_rn(vb, va), __ldg(p.stepTwD + s))));
    };
    // one step of the log-Euler scheme (mcMdlDupire.h:238-280) from state xs with Gaussian ga;
    // (bj, bc): the bumped node, or bj < 0
    auto step = [&](int s, double xs, double ga, int bj, int bc, int& lo) -> double {
        lo = locate(xs);
        const double* row = p.Yd + size_t(s) * nS;
        const bool hit = bj >= 0 && (__ldg(p.colA + s) == bc || (__ldg(p.cBd + s) != 0.0 && __ldg(p.colB + s) == bc));
        double v;
        if (lo == nS || lo == 0)
        {
            const int k = lo == 0 ? 0 : nS - 1;
            v = (hit && bj == k) ? yBumped(s, k, bc) : __ldg(row + k);
        }
        else
        {
            const int k = lo - 1;
            const double y1 = (hit && bj == k) ? yBumped(s, k, bc) : __ldg(row + k);
            const double y2 = (hit && bj == k + 1) ? yBumped(s, k + 1, bc) : __ldg(row + k + 1);
            const double t = (xs - __ldg(p.Xd + k)) * __ldg(p.invdXd + k);
            v = y1 + (y2 - y1) * t;
        }
        return xs + v * (-0.5 * v + ga);
    };

    // Path state: the log spot, the barrier's survival factor and knock-out, the spot at the
    // European's date (for the barrier: at maturity).
    struct St
    {
        double x, alive, fE;
        bool dead;
    };
    // product date at point i (mc_kernel's eventFwd for the Dupire model: F = S, D = N = 1);
    // European portfolio payoffs are written through pay(k, value)
    auto event = [&](int i, St& z, double barS, double minusS, double twoS, double logBand, auto&& pay) {
        const int e = __ldg(p.evAtStep + i);
        if (e < 0) return;
        const bool last = e == nEv - 1;
        if (UOC && !last && (z.dead || !(z.x > logBand))) return;
        const double F = exp(z.x);
        if (EUR) z.fE = F;
        else if (UOC)
        {
            if (!z.dead)
            {
                if (F > barS) z.dead = true;
                else if (F > minusS) z.alive *= (barS - F) / twoS;
            }
            if (last) z.fE = F;  // the European part: max(F - K, 0) at maturity
        }
        else
        {
            const int k0 = __ldg(p.evPayOff + e), k1 = __ldg(p.evPayOff + e + 1);
            for (int k = k0; k < k1; ++k)
            {
                const double m = F - __ldg(p.kD + k);
                pay(k, m > 0.0 ? m : 0.0);
            }
        }
    };
    // payoffs at the end of a path (mc_kernel's payoff code for the Dupire model)
    auto finals = [&](const St& z, double* out) {
        if (EUR)
        {
            const double m = z.fE - p.strike;
            out[0] = (m > 0.0 ? m : 0.0) * 1.0 / 1.0;
        }
        else if (UOC)
        {
            const double m = p.callPut ? (p.strike - z.fE) : (z.fE - p.strike);
            const double euro = (m > 0.0 ? m : 0.0) / 1.0;
            out[0] = z.dead ? 0.0 : z.alive * euro;
            out[1] = euro;
        }
    };
    auto addDiff = [&](int param, int k, double d) {
        if (d != 0.0) fix_add(&b.acc[2 * (size_t(param) * nPay + k)], d);
    };
    // one path a of the current unit, Gaussians in the scratch
    auto runPath = [&](int a) {
        const double sg = a ? -1.0 : 1.0;
        // base path: states per point, intervals per step, payoffs
        St z{p.x0d, 1.0, 0.0, false};
        auto basePay = [&](int k, double v) { D(R.dP0 + a * nPay + k) = v; };
        D(R.dX + a * (nSteps + 1)) = z.x;
        event(0, z, p.barSmooth, p.minusSmooth, p.twoSmooth, p.logBandD, basePay);
        D(R.dA + a * (nSteps + 1)) = z.dead ? -1.0 : z.alive;
        for (int s = 0; s < nSteps; ++s)
        {
            int lo;
            z.x = step(s, z.x, sg * D(R.dG + s), -1, 0, lo);
            I(R.iK + a * nSteps + s) = lo;
            event(s + 1, z, p.barSmooth, p.minusSmooth, p.twoSmooth, p.logBandD, basePay);
            D(R.dX + a * (nSteps + 1) + s + 1) = z.x;
            D(R.dA + a * (nSteps + 1) + s + 1) = z.dead ? -1.0 : z.alive;
        }
        if (EUR || UOC)
        {
            double fin[2] = {0.0, 0.0};
            finals(z, fin);
            for (int k = 0; k < nPay; ++k) D(R.dP0 + a * nPay + k) = fin[k];
        }
        for (int k = 0; k < nPay; ++k) fix_add(&b.acc[2 * (size_t(b.nParam) * nPay + k)], D(R.dP0 + a * nPay + k));

        // re-simulation from point s0 (state of the base path there) with a bump:
        // node (bj, bc), or the spot bump (bj < 0, s0 = 0, bumped start and smoothing)
        auto rerun = [&](int s0, int bj, int bc, int param) {
            const bool spotB = bj < 0;
            const double barS = spotB ? b.barSmoothB : p.barSmooth, minusS = spotB ? b.minusSmoothB : p.minusSmooth,
                         twoS = spotB ? b.twoSmoothB : p.twoSmooth, logBand = spotB ? b.logBandB : p.logBandD;
            St w;
            if (spotB)
            {
                w = St{b.x0Bumped, 1.0, 0.0, false};
                auto pay0 = [&](int k, double v) { addDiff(param, k, v - D(R.dP0 + a * nPay + k)); };
                event(0, w, barS, minusS, twoS, logBand, pay0);
            }
            else
            {
                // the base path's state at point s0 (its dates up to s0 do not change)
                const double al = D(R.dA + a * (nSteps + 1) + s0);
                w = St{D(R.dX + a * (nSteps + 1) + s0), al < 0.0 ? 0.0 : al, 0.0, al < 0.0};
            }
            auto payK = [&](int k, double v) { addDiff(param, k, v - D(R.dP0 + a * nPay + k)); };
            for (int s = s0; s < nSteps; ++s)
            {
                int lo;
                w.x = step(s, w.x, sg * D(R.dG + s), spotB ? -1 : bj, bc, lo);
                event(s + 1, w, barS, minusS, twoS, logBand, payK);
            }
            if (EUR || UOC)
            {
                double fin[2] = {0.0, 0.0};
                finals(w, fin);
                for (int k = 0; k < nPay; ++k) addDiff(param, k, fin[k] - D(R.dP0 + a * nPay + k));
            }
        };

        rerun(0, -1, 0, 0);  // spot
        for (int wd = 0; wd < b.maskWords; ++wd) M(wd) = 0u;
        for (int s = 0; s < nSteps; ++s)
        {
            const int lo = I(R.iK + a * nSteps + s);
            const int ca = __ldg(p.colA + s), cb = __ldg(p.colB + s);
            const bool twoCols = __ldg(p.cBd + s) != 0.0 && cb != ca;
            const bool flat = lo == 0 || lo == nS;
            const int j0 = flat ? (lo == 0 ? 0 : nS - 1) : lo - 1;
            for (int q = 0; q < (flat ? 1 : 2); ++q)
                for (int r = 0; r < (twoCols ? 2 : 1); ++r)
                {
                    const int j = j0 + q, c = r ? cb : ca;
                    const int bit = j * nT + c;
                    unsigned& mw = M(bit >> 5);
                    if (mw & (1u << (bit & 31))) continue;
                    mw |= 1u << (bit & 31);
                    rerun(s, j, c, 1 + bit);
                }
        }
    };

    if (RNGK == RNG_MRG)
    {
        const long long nUnits = (p.nPath + 1) / 2;
        const long long per = (nUnits + Ti - 1) / Ti;
        const long long u0 = tg * per;
        const long long u1 = u0 + per < nUnits ? u0 + per : nUnits;
        if (u0 >= u1) return;
        MrgState st = mrg_jump(p.seed1, p.seed2, (unsigned long long)u0 * nSteps, p.mrgJumpA, p.mrgJumpB);
        for (long long u = u0; u < u1; ++u)
        {
            for (int s = 0; s < nSteps; ++s) D(R.dG + s) = mrg_gauss<double>(mrg_next(st));
            runPath(0);
            if (2 * u + 1 < p.nPath) runPath(1);
        }
    }
    else
    {
        // Sobol: index n = 1 .. nPath (path n - 1), strided over the grid
        for (long long n = tg + 1; n <= p.nPath; n += Ti)
        {
            for (int s = 0; s < nSteps; ++s) D(R.dG + s) = sobol_gauss<double>(sobol_state(p.sobolDir, nSteps, s, n));
            runPath(0);
        }
    }
}

}  // namespace

const void* dupire_bump64_ptr(int prod, int rng)
{
#define CF_B(PR, RG) \
    if (prod == PR && rng == RG) return (const void*)&dupire_bump64<PR, RG>;
    CF_B(PROD_EUROPEAN, RNG_MRG)
    CF_B(PROD_EUROPEAN, RNG_SOBOL)
    CF_B(PROD_UOC, RNG_MRG)
    CF_B(PROD_UOC, RNG_SOBOL)
    CF_B(PROD_EUROPEANS, RNG_MRG)
    CF_B(PROD_EUROPEANS, RNG_SOBOL)
#undef CF_B
    return nullptr;
}

}  // namespace cf
