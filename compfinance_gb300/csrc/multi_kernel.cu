// AADriskMulti of a European portfolio (mcPrd.h:291-400; main.h:269-312, mcBase.h:775-989):
// the risk of every payoff to every model parameter in one pass over the paths.
//
// Payoff (e, j) = max(F_e - K_ej, 0) / N_e depends on the path only through maturity e, so a
// path needs one adjoint per maturity, not one per payoff (the reference carries an
// nPay-wide adjoint through every tape node).  With the strikes of a maturity sorted, the
// payoffs a path pays are the m_e strikes below F_e, and
//     d payoff_(e,j) / d theta = a_theta - K_j b_theta   for j < m_e, 0 otherwise,
// with a = dF/dtheta / N - F dN/dtheta / N^2 and b = -dN/dtheta / N^2 path quantities.  The
// kernel accumulates a and b into bucket (e, m_e); multi_finish turns buckets into per-strike
// risks by suffix sums over m.  Values and squares use the same buckets.
//
// Dupire: a = S_e dx_e/dtheta (N = 1), from a reverse sweep that carries one adjoint per
// maturity.  Black-Scholes: four parameters, forward tangents of log S.
#include <type_traits>

#include "cf_device.cuh"
#include "mc_kernel.cuh"

namespace cf {

constexpr int MULTI_MAXE = 16;  // maturities carried in registers by the fast kernel

struct MultiParams
{
    McParams p;          // model tables, RNG, sizes (nEv, nSteps, nS, nT, spot ...)
    int nParam;          // BS 4, Dupire 1 + nS*nT
    const int* evOff;    // [nEv+1] bucket offsets: bucket (e, m) = evOff[e] + m, m in [0, nK_e]
    const double* ksD;   // sorted strikes, flattened like evOff minus one per event: [evOff[e]-e + j]
    const float* ksF;
    long long* accRisk;  // [nBuckets][nParam][2] global fixed-point (bucket m=0 unused)
    long long* accVal;   // [nBuckets][5][2]: 1/N, F/N, 1/N^2, F/N^2, F^2/N^2
};

template <int MODEL, int RNGK, class Real>
__global__ void __launch_bounds__(MC_BLOCK) multi_kernel(const MultiParams mp)
{
    constexpr int NP = RNGK == RNG_MRG ? 2 : 1;
    constexpr bool F32 = std::is_same<Real, float>::value;
    const McParams& p = mp.p;
    extern __shared__ __align__(128) unsigned char smem[];
    const int tid = threadIdx.x;
    const int nEv = p.nEv, nSteps = p.nSteps, nS = p.nS, nT = p.nT;
    const int nBuckets = mp.evOff[nEv];
    // shared: value buckets [nBuckets][5] hi/lo, BS risk buckets [nBuckets][4][2] hi/lo,
    // Dupire grid (X, 1/dX, bucket index), Sobol base rows
    long long* sVal = reinterpret_cast<long long*>(smem);
    long long* sBs = sVal + 2 * 5 * nBuckets;
    const int nBsWords = MODEL == MODEL_BS ? 2 * 8 * nBuckets : 0;
    Real* sX = reinterpret_cast<Real*>(sBs + nBsWords);
    Real* sInv = sX + nS;
    int* sBk = reinterpret_cast<int*>(sInv + nS);
    unsigned* sBase = reinterpret_cast<unsigned*>(sBk + p.nBuckets);
    for (int i = tid; i < 10 * nBuckets + nBsWords; i += MC_BLOCK) sVal[i] = 0;
    if (MODEL == MODEL_DUPIRE)
    {
        const Real* gX = pick<Real>(p.Xd, p.Xf);
        const Real* gI = pick<Real>(p.invdXd, p.invdXf);
        for (int i = tid; i < nS; i += MC_BLOCK)
        {
            sX[i] = gX[i];
            sInv[i] = gI[i];
        }
        for (int i = tid; i < p.nBuckets; i += MC_BLOCK) sBk[i] = p.bucket[i];
    }
    __syncthreads();

    const Real* Y = pick<Real>(p.Yd, p.Yf);
    const Real* bs = pick<Real>(p.bsD, p.bsF);
    const Real* ev = pick<Real>(p.evD, p.evF);
    const Real* ks = pick<Real>(mp.ksD, mp.ksF);
    const Real* cA = pick<Real>(p.cAd, p.cAf);
    const Real* cB = pick<Real>(p.cBd, p.cBf);
    const Real xStart = F32 ? Real(0) : (Real)p.x0d;
    const Real sScale = F32 ? (Real)p.s0f : Real(1);
    const Real spot = (Real)p.spot;
    const Real bX0 = F32 ? (Real)p.bX0f : (Real)p.bX0d;
    const Real bInvW = F32 ? (Real)p.bInvWf : (Real)p.bInvWd;
    const long long T = (long long)gridDim.x * MC_BLOCK;
    const long long tg = (long long)blockIdx.x * MC_BLOCK + tid;
    Real* scr = reinterpret_cast<Real*>(p.scratch) + tg;
    const int Ti = int(T), rowStride = (nSteps + 1) * Ti;
    auto SCR = [&](int f, int i) -> Real& { return scr[f * rowStride + i * Ti]; };

    auto interpRow = [&](int s, Real xs, int& k, Real& t, Real& v, Real& slope, bool& flat) {
        const Real fb = (xs - bX0) * bInvW;
        int b = fb > Real(0) ? int(fb) : 0;
        b = b < p.nBuckets - 1 ? b : p.nBuckets - 1;
        int lo = sBk[b];
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
    // number of sorted strikes of maturity e strictly below F (the payoffs in the money)
    auto bucketOf = [&](int e, Real F) {
        const int o = mp.evOff[e] - e, n = mp.evOff[e + 1] - mp.evOff[e] - 1;
        int m = 0;
        while (m < n && ks[o + m] < F) ++m;
        return m;
    };

    auto runUnit = [&](int nAct, auto&& gen) {
        Real x[NP];
        // Black-Scholes forward tangents of log S: spot, vol, rate, div
        Real tv[NP], tr[NP];
#pragma unroll
        for (int a = 0; a < NP; ++a)
        {
            x[a] = MODEL == MODEL_DUPIRE ? xStart : spot;
            tv[a] = tr[a] = Real(0);
        }
        int eNext = 0;
        for (int i = 0; i <= nSteps; ++i)
        {
            if (i > 0)
            {
                const int s = i - 1;
                const Real g = gen(s);
                if (MODEL == MODEL_DUPIRE) SCR(0, s) = g;
#pragma unroll
                for (int a = 0; a < NP; ++a)
                {
                    if (a >= nAct) break;
                    const Real ga = a ? -g : g;
                    if (MODEL == MODEL_DUPIRE)
                    {
                        SCR(1 + a, s) = x[a];
                        int k;
                        Real t, v, slope;
                        bool flat;
                        interpRow(s, x[a], k, t, v, slope, flat);
                        x[a] += v * (Real(-0.5) * v + ga);
                    }
                    else
                    {
                        x[a] = x[a] * exp(bs[s] + bs[nSteps + s] * ga);
                        tv[a] += bs[4 * nSteps + s] + bs[3 * nSteps + s] * ga;
                        tr[a] += bs[2 * nSteps + s];
                    }
                }
            }
            const int e = p.evAtStep[i];
            if (e < 0) continue;
            eNext = e + 1;
#pragma unroll
            for (int a = 0; a < NP; ++a)
            {
                if (a >= nAct) break;
                const Real S = MODEL == MODEL_DUPIRE ? sScale * exp(x[a]) : x[a];
                Real F = S, N = Real(1);
                Real dlnN[4] = {0, 0, 0, 0}, dlnF[4] = {0, 0, 0, 0};
                if (MODEL == MODEL_BS)
                {
                    const Real ff = ev[e], tauF = ev[nEv + e], te = ev[5 * nEv + e], nf = ev[4 * nEv + e];
                    F = S * ff;
                    // d ln S / d theta
                    const Real dS[4] = {Real(1) / spot, tv[a], tr[a], -tr[a]};
                    for (int q = 0; q < 4; ++q) dlnF[q] = dS[q];
                    dlnF[2] += tauF;
                    dlnF[3] -= tauF;
                    if (p.spotMeasure)
                    {
                        N = nf * S;
                        for (int q = 0; q < 4; ++q) dlnN[q] = dS[q];
                        dlnN[0] -= Real(1) / spot;
                        dlnN[3] += te;
                    }
                    else
                    {
                        N = nf;
                        dlnN[2] = te;
                    }
                }
                const int m = bucketOf(e, F);
                const int bk = mp.evOff[e] + m;
                const Real iN = Real(1) / N;
                fix_add(&sVal[2 * (5 * bk + 0)], iN);
                fix_add(&sVal[2 * (5 * bk + 1)], F * iN);
                fix_add(&sVal[2 * (5 * bk + 2)], iN * iN);
                fix_add(&sVal[2 * (5 * bk + 3)], F * iN * iN);
                fix_add(&sVal[2 * (5 * bk + 4)], F * F * iN * iN);
                if (MODEL == MODEL_BS && m > 0)
                {
                    for (int q = 0; q < 4; ++q)
                    {
                        fix_add(&sBs[2 * (8 * bk + 2 * q)], F * iN * (dlnF[q] - dlnN[q]));  // a
                        fix_add(&sBs[2 * (8 * bk + 2 * q + 1)], -iN * dlnN[q]);              // b
                    }
                }
                if (MODEL == MODEL_DUPIRE)
                {
                    // event data kept for the reverse sweep: seed S_e (0 when out of the money)
                    SCR(1 + NP + a * 2, e) = m > 0 ? S : Real(0);
                    SCR(2 + NP + a * 2, e) = Real(m);
                }
            }
        }
        (void)eNext;
        if (MODEL != MODEL_DUPIRE) return;

        // Reverse sweep per path with one adjoint per maturity (MULTI_MAXE in registers).
        for (int a = 0; a < nAct; ++a)
        {
            Real ax[MULTI_MAXE];
            int bk[MULTI_MAXE];
#pragma unroll
            for (int e = 0; e < MULTI_MAXE; ++e)
            {
                ax[e] = Real(0);
                bk[e] = 0;
            }
            for (int i = nSteps; i >= 1; --i)
            {
                const int ei = p.evAtStep[i];
                if (ei >= 0)
                {
#pragma unroll
                    for (int e = 0; e < MULTI_MAXE; ++e)
                        if (e == ei)
                        {
                            ax[e] = SCR(1 + NP + a * 2, ei);
                            bk[e] = mp.evOff[ei] + int(SCR(2 + NP + a * 2, ei));
                        }
                }
                const int s = i - 1;
                const Real g = SCR(0, s);
                const Real ga = a ? -g : g;
                const Real xs = SCR(1 + a, s);
                int k;
                Real t, v, slope;
                bool flat;
                interpRow(s, xs, k, t, v, slope, flat);
                const Real q = ga - v;
                const int ca = p.colA[s], cb = p.colB[s];
                const Real wa = cA[s], wb = cB[s];
                const int n0 = 1 + k * nT, n1 = 1 + (k + 1) * nT;
#pragma unroll
                for (int e = 0; e < MULTI_MAXE; ++e)
                {
                    if (ax[e] == Real(0)) continue;
                    const Real av = ax[e] * q;
                    ax[e] += av * slope;
                    long long* base = mp.accRisk + 2 * (size_t)bk[e] * mp.nParam;
                    const Real a0 = flat ? av : av * (Real(1) - t);
                    fix_add(base + 2 * (n0 + ca), a0 * wa);
                    if (wb != Real(0)) fix_add(base + 2 * (n0 + cb), a0 * wb);
                    if (!flat)
                    {
                        const Real a1 = av * t;
                        fix_add(base + 2 * (n1 + ca), a1 * wa);
                        if (wb != Real(0)) fix_add(base + 2 * (n1 + cb), a1 * wb);
                    }
                }
            }
#pragma unroll
            for (int e = 0; e < MULTI_MAXE; ++e)
                if (ax[e] != Real(0)) fix_add(mp.accRisk + 2 * (size_t)bk[e] * mp.nParam, ax[e] / spot);
        }
    };

    if (RNGK == RNG_MRG)
    {
        const long long nUnits = (p.nPath + 1) / 2;
        const long long per = (nUnits + T - 1) / T;
        const long long u0 = tg * per;
        const long long u1 = u0 + per < nUnits ? u0 + per : nUnits;
        if (u0 < u1)
        {
            MrgState st = mrg_jump(p.seed1, p.seed2, (unsigned long long)(p.firstPath / 2 + u0) * nSteps, p.mrgJumpA, p.mrgJumpB);
            for (long long u = u0; u < u1; ++u)
                runUnit((2 * u + 1 < p.nPath) ? 2 : 1, [&](int) { return mrg_gauss<Real>(mrg_next(st)); });
        }
    }
    else
    {
        const int lane = tid & 31, wib = tid >> 5;
        const int pitch = nSteps | 1;
        unsigned* base = sBase + wib * pitch;
        const long long W = T / 32, gw = tg / 32;
        const long long nB = p.nPath / 32 + 1;
        for (long long b = gw; b < nB; b += W)
        {
            __syncwarp();
            for (int d = lane; d < nSteps; d += 32)
                base[d] = sobol_state(p.sobolDir, nSteps, d, (unsigned long long)(p.firstPath + b * 32));
            __syncwarp();
            const long long n = b * 32 + lane;
            if (n >= 1 && n <= p.nPath)
                runUnit(1, [&](int i) {
                    return sobol_gauss<Real>(base[i] ^ sobol_state(p.sobolDir, nSteps, i, (unsigned long long)lane));
                });
        }
    }
    __syncthreads();
    for (int i = tid; i < 5 * nBuckets; i += MC_BLOCK) fix_flush(&mp.accVal[2 * i], &sVal[2 * i]);
    if (MODEL == MODEL_BS)
        for (int i = tid; i < 8 * nBuckets; i += MC_BLOCK)
        {
            // BS buckets: accRisk[bucket][param] holds a, accVal... b goes to the second half
            const int bk = i / 8, q = (i % 8) / 2, ab = i % 2;
            fix_flush(&mp.accRisk[2 * ((size_t)bk * 8 + 2 * q + ab)], &sBs[2 * i]);
        }
}

size_t multi_smem_bytes(int model, int rng, int fp32, const McParams& p, int nBuckets)
{
    const size_t rs = fp32 ? 4 : 8;
    size_t b = size_t(nBuckets) * 5 * 16 + (model == MODEL_BS ? size_t(nBuckets) * 8 * 16 : 0);
    b += 2 * size_t(p.nS) * rs + size_t(p.nBuckets) * 4 + 16;
    if (rng == RNG_SOBOL) b += size_t(MC_BLOCK / 32) * (size_t(p.nSteps) | 1) * 4;
    return (b + 15) & ~size_t(15);
}

static const void* multi_ptr(int model, int rng, int fp32)
{
    if (model == MODEL_BS)
    {
        if (rng == RNG_MRG) return fp32 ? (const void*)&multi_kernel<MODEL_BS, RNG_MRG, float>
                                        : (const void*)&multi_kernel<MODEL_BS, RNG_MRG, double>;
        return fp32 ? (const void*)&multi_kernel<MODEL_BS, RNG_SOBOL, float>
                    : (const void*)&multi_kernel<MODEL_BS, RNG_SOBOL, double>;
    }
    if (rng == RNG_MRG) return fp32 ? (const void*)&multi_kernel<MODEL_DUPIRE, RNG_MRG, float>
                                    : (const void*)&multi_kernel<MODEL_DUPIRE, RNG_MRG, double>;
    return fp32 ? (const void*)&multi_kernel<MODEL_DUPIRE, RNG_SOBOL, float>
                : (const void*)&multi_kernel<MODEL_DUPIRE, RNG_SOBOL, double>;
}

int multi_occupancy(int model, int rng, int fp32, size_t smem, int* occ)
{
    const void* fn = multi_ptr(model, rng, fp32);
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return (int)e;
    return (int)cudaOccupancyMaxActiveBlocksPerMultiprocessor(occ, fn, MC_BLOCK, smem);
}

// Per-payoff risks from the bucket accumulators.  Bucket m of a maturity holds the adjoints of
// the paths whose spot lies between its (m-1)th and mth sorted strikes, so the payoff of the
// jth strike collects the buckets above j: thread (q, e) (one model parameter, one maturity)
// walks the maturity's buckets from the top, keeps exact integer suffix sums and writes
// risk[q][payoff] = sum / nPath.  Black-Scholes buckets hold a pair (a, b) per parameter and the
// strike's risk is (a - K b) / nPath.
__global__ void multi_finish(const long long* __restrict__ accR, int nAccParam, int nOut, const int* __restrict__ evOff,
                             const double* __restrict__ ks, const int* __restrict__ orig, int nPay, int bs, double n,
                             double* __restrict__ risks)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x, ev = blockIdx.y;
    if (q >= nOut) return;
    auto val = [](long long hi, long long lo) {
        return __dadd_rn(__dmul_rn((double)hi, 1.0 / 1048576.0), __dmul_rn((double)lo, 1.0 / 1152921504606846976.0));
    };
    const int b0 = evOff[ev], nK = evOff[ev + 1] - b0 - 1, sorted = b0 - ev;
    long long ha = 0, la = 0, hb = 0, lb = 0;
#pragma unroll 4
    for (int j = nK - 1; j >= 0; --j)
    {
        const size_t bk = size_t(b0 + j + 1);
        double r;
        if (bs)
        {
            const long long* a = accR + 2 * (bk * nAccParam + 2 * q);
            ha += a[0];
            la += a[1];
            hb += a[2];
            lb += a[3];
            r = __ddiv_rn(__dsub_rn(val(ha, la), __dmul_rn(ks[sorted + j], val(hb, lb))), n);
        }
        else
        {
            const long long* a = accR + 2 * (bk * nAccParam + q);
            ha += a[0];
            la += a[1];
            r = __ddiv_rn(val(ha, la), n);
        }
        risks[size_t(q) * nPay + orig[sorted + j]] = r;
    }
}

// Risks of a weighted sum of the payoffs: out[j] = sum_k w[k] risks[j][k] (the finished
// per-payoff risks, [nParam][nPay]); one thread per parameter, payoffs in order.
__global__ void multi_aggregate_kernel(const double* risks, int nParam, int nPay, const double* w, double* out)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nParam) return;
    const double* row = risks + size_t(j) * nPay;
    double a = 0.0;
    for (int k = 0; k < nPay; ++k) a += w[k] * row[k];
    out[j] = a;
}

int launch_multi_aggregate(const double* risks, int nParam, int nPay, const double* w, double* out, void* stream)
{
    multi_aggregate_kernel<<<(nParam + 127) / 128, 128, 0, (cudaStream_t)stream>>>(risks, nParam, nPay, w, out);
    return (int)cudaGetLastError();
}

int launch_multi_finish(const long long* accR, int nAccParam, int nOut, int nEv, const int* evOff, const double* ks,
                        const int* orig, int nPay, int bs, double n, double* risks, void* stream)
{
    multi_finish<<<dim3((nOut + 127) / 128, nEv), 128, 0, (cudaStream_t)stream>>>(accR, nAccParam, nOut, evOff, ks, orig,
                                                                                nPay, bs, n, risks);
    return (int)cudaGetLastError();
}

int launch_multi(int model, int rng, int fp32, int grid, size_t smem, const MultiParams& mp, void* stream)
{
    MultiParams q = mp;
    void* args[] = {&q};
    return (int)cudaLaunchKernel(multi_ptr(model, rng, fp32), dim3(grid), dim3(MC_BLOCK), args, smem,
                                 (cudaStream_t)stream);
}

}  // namespace cf
