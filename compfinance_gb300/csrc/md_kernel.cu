// Multiple correlated assets under displaced Black-Scholes dynamics with proportional
// dividends (mcMdlMultiDisplaced.h:28-717), with the products Baskets and Autocall
// (mcPrdMulti.h:181-439): values, and path-wise adjoints of one aggregate of the payoffs.
//
// The model's initialisation (displacements, lambda-shifted correlation and its Cholesky
// factor, per-step stds, drifts and dividend-adjusted forward factors, numeraires) runs once
// per plan on the host (multi_asset.cpp) and arrives here as the derived table of md_layout.
// A path step, per asset a with correlated Brownian cw = sum_{b<=a} L[a][b] w[b] and forward
// fwd = S ff[i][a]:
//   lognormal   S' = fwd exp(drift + std cw)
//   normal      S' = fwd + std cw
//   surnormal   S' = (fwd + alpha) exp(drift + std cw) - alpha
//   subnormal   S' = (fwd - alpha) exp(drift + std cw) + alpha
// In risk mode each path is swept back from its last product date, and the adjoints of the
// derived quantities (initial spots, Cholesky entries, stds, drifts, forward factors,
// displacements, numeraires) are summed in fixed point; the host maps them to the model
// parameters through the Jacobian of the initialisation, which is exactly the chain rule the
// reference's tape applies through init (mcBase.h:427-532).
//
// A thread runs an antithetic mrg32k3a pair (the second path with the negated Gaussian
// vector, mrg32k3a.h:150-184) or one Sobol path; the Gaussians of a path are drawn step-major,
// dimension i * nA + a for asset a at step i (mcMdlMultiDisplaced.h:638-639).
#include <type_traits>

#include "cf_device.cuh"

namespace cf {

namespace {

constexpr int MD_BLOCK = 128;

template <class R>
__device__ __forceinline__ const R* pickR(const double* d, const float* f);
template <>
__device__ __forceinline__ const double* pickR<double>(const double* d, const float*) { return d; }
template <>
__device__ __forceinline__ const float* pickR<float>(const double*, const float* f) { return f; }

struct MdSmem
{
    size_t acc, tab, asset, strike, weight, dyn, base, total;
};

// shared memory: accumulators, derived table, per-asset and per-payoff constants, Sobol bases
__host__ __device__ inline MdSmem md_smem(int rng, int fp32, const McParams& p)
{
    const size_t rs = fp32 ? 4 : 8;
    const MdLayout L = md_layout(p.nA, p.nSteps, p.nEv);
    MdSmem S;
    size_t off = 0;
    auto take = [&](size_t n) {
        const size_t o = off;
        off += (n + 15) & ~size_t(15);
        return o;
    };
    S.acc = take(size_t(p.nAcc) * 16);
    S.tab = take(size_t(L.total) * rs);
    S.asset = take(size_t(p.nA) * rs);
    S.strike = take(size_t(p.nPay) * rs);
    S.weight = take(size_t(p.nPay) * rs);
    S.dyn = take(size_t(p.nA) * 4);
    S.base = take(rng == RNG_SOBOL ? size_t(MD_BLOCK / 32) * (size_t(p.nSteps * p.nA) | 1) * 4 : 0);
    S.total = off;
    return S;
}

template <int RNGK, class Real, int NA>
__global__ void __launch_bounds__(MD_BLOCK) md_kernel(const McParams p)
{
    constexpr int NP = RNGK == RNG_MRG ? 2 : 1;
    constexpr bool F32 = std::is_same<Real, float>::value;
    extern __shared__ __align__(128) unsigned char smem[];
    const MdSmem S = md_smem(RNGK, F32, p);
    long long* sAcc = reinterpret_cast<long long*>(smem + S.acc);
    Real* tab = reinterpret_cast<Real*>(smem + S.tab);
    Real* sAsset = reinterpret_cast<Real*>(smem + S.asset);
    Real* sK = reinterpret_cast<Real*>(smem + S.strike);
    Real* sW = reinterpret_cast<Real*>(smem + S.weight);
    int* sDyn = reinterpret_cast<int*>(smem + S.dyn);
    const int tid = threadIdx.x, lane = tid & 31, wib = tid >> 5;
    const int nA = p.nA, nSteps = p.nSteps, nEv = p.nEv, nPay = p.nPay, nRisk = p.nRisk, dim = nSteps * nA;
    const MdLayout L = md_layout(nA, nSteps, nEv);
    const bool risk = nRisk > 0;
    const bool basket = p.prodKind == PROD_BASKETS;
    {
        const Real* gTab = pickR<Real>(p.mdD, p.mdF);
        const Real* gAsset = pickR<Real>(p.mdAssetD, p.mdAssetF);
        const Real* gK = pickR<Real>(p.kD, p.kF);
        const Real* gW = pickR<Real>(p.w, p.wf);
        for (int i = tid; i < 2 * p.nAcc; i += MD_BLOCK) sAcc[i] = 0;
        for (int i = tid; i < L.total; i += MD_BLOCK) tab[i] = gTab[i];
        for (int i = tid; i < nA; i += MD_BLOCK)
        {
            sAsset[i] = gAsset[i];
            sDyn[i] = p.mdDyn[i];
        }
        for (int i = tid; i < nPay; i += MD_BLOCK)
        {
            sK[i] = basket ? gK[i] : Real(0);
            sW[i] = gW[i];
        }
    }
    __syncthreads();
    long long* accPay = sAcc + 2 * nRisk;  // [nPay] sums, [nPay] squares, aggregate, its square
    const Real* chol = tab + L.chol;
    const Real ko = Real(p.acKo), kput = Real(p.acStrike), cpn = Real(p.acCpn), dtc = Real(p.acDt),
               sm = Real(p.acSmooth);

    // reverse-sweep scratch [field][thread]: Gaussians [dim], spots after each step [NP][dim],
    // autocall notional alive before each date [NP][nEv]
    const long long T = (long long)gridDim.x * MD_BLOCK;
    const long long tg = (long long)blockIdx.x * MD_BLOCK + tid;
    Real* scr = reinterpret_cast<Real*>(p.scratch) + tg;
    auto SW = [&](int d) -> Real& { return scr[size_t(d) * T]; };
    auto SS = [&](int a, int d) -> Real& { return scr[size_t(dim + a * dim + d) * T]; };
    auto SA = [&](int a, int e) -> Real& { return scr[size_t(dim + NP * dim + a * nEv + e) * T]; };

    // worst performance at date e (the first minimum, as min_element), its asset
    auto worstOf = [&](const Real* s, int& wi) {
        Real w = s[0] / sAsset[0];
        wi = 0;
#pragma unroll
        for (int a = 1; a < NA; ++a)
            if (a < nA)
            {
                const Real q = s[a] / sAsset[a];
                if (q < w)
                {
                    w = q;
                    wi = a;
                }
            }
        return w;
    };

    auto runUnit = [&](int nAct, auto&& gen) {
        Real s[NP][NA], alive[NP], pay[NP];
#pragma unroll
        for (int ap = 0; ap < NP; ++ap)
        {
#pragma unroll
            for (int a = 0; a < NA; ++a) s[ap][a] = a < nA ? tab[L.s0 + a] : Real(0);
            alive[ap] = Real(1);
            pay[ap] = Real(0);
        }
        for (int i = 0; i < nSteps; ++i)
        {
            Real w[NA];
#pragma unroll
            for (int a = 0; a < NA; ++a)
                if (a < nA)
                {
                    w[a] = gen(i * nA + a);
                    if (risk) SW(i * nA + a) = w[a];
                }
#pragma unroll
            for (int a = 0; a < NA; ++a)
            {
                if (a >= nA) break;
                Real cw = Real(0);
#pragma unroll
                for (int b = 0; b <= a; ++b) cw += chol[a * nA + b] * w[b];
                const Real sd = tab[L.std_ + i * nA + a], dr = tab[L.drift + i * nA + a],
                           ff = tab[L.ff + i * nA + a], al = tab[L.alpha + a];
                const int dy = sDyn[a];
#pragma unroll
                for (int ap = 0; ap < NP; ++ap)
                {
                    if (ap >= nAct) break;
                    const Real c = ap ? -cw : cw;
                    const Real fwd = s[ap][a] * ff;
                    Real nx;
                    if (dy == MD_LOGNORMAL) nx = fwd * exp(dr + sd * c);
                    else if (dy == MD_NORMAL) nx = fwd + sd * c;
                    else if (dy == MD_SURNORMAL) nx = (fwd + al) * exp(dr + sd * c) - al;
                    else nx = (fwd - al) * exp(dr + sd * c) + al;
                    s[ap][a] = nx;
                    if (risk) SS(ap, i * nA + a) = nx;
                }
            }
            const int e = p.evAtStep[i + 1];
            if (e < 0) continue;
            const Real num = tab[L.num + e];
#pragma unroll
            for (int ap = 0; ap < NP; ++ap)
            {
                if (ap >= nAct) break;
                if (basket)
                {
                    Real b = Real(0);
#pragma unroll
                    for (int a = 0; a < NA; ++a)
                        if (a < nA) b = b + sAsset[a] * s[ap][a];
                    Real agg = Real(0);
                    for (int k = 0; k < nPay; ++k)
                    {
                        const Real m = b - sK[k];
                        const Real v = (m > Real(0) ? m : Real(0)) / num;
                        fix_add(&accPay[2 * k], v);
                        fix_add(&accPay[2 * (nPay + k)], v * v);
                        agg += sW[k] * v;
                    }
                    fix_add(&accPay[2 * (2 * nPay)], agg);
                    fix_add(&accPay[2 * (2 * nPay + 1)], agg * agg);
                    continue;
                }
                // autocall (mcPrdMulti.h:368-416)
                if (risk) SA(ap, e) = alive[ap];
                int wi;
                const Real worst = worstOf(s[ap], wi);
                pay[ap] += alive[ap] * cpn * dtc / num;
                if (e < nEv - 1)
                {
                    const Real x = (ko + sm - worst) / Real(2) / sm;
                    const Real f = x > Real(1) ? Real(1) : x > Real(0) ? x : Real(0);
                    const Real surv = alive[ap] * f;
                    pay[ap] += (alive[ap] - surv) / num;
                    alive[ap] = surv;
                }
                else
                {
                    pay[ap] += alive[ap] / num;
                    const Real m = kput - worst;
                    pay[ap] -= alive[ap] * (m > Real(0) ? m : Real(0)) / kput / num;
                    fix_add(&accPay[0], pay[ap]);
                    fix_add(&accPay[2 * nPay], pay[ap] * pay[ap]);
                    const Real agg = sW[0] * pay[ap];
                    fix_add(&accPay[2 * (2 * nPay)], agg);
                    fix_add(&accPay[2 * (2 * nPay + 1)], agg * agg);
                }
            }
        }
        if (!risk) return;

        // reverse sweep of each path: adjoint of the aggregate sum_k w_k payoff_k
#pragma unroll
        for (int ap = 0; ap < NP; ++ap)
        {
            if (ap >= nAct) break;
            const Real sgn = ap ? Real(-1) : Real(1);
            Real sb[NA], ab[NA], lb[NA * (NA + 1) / 2];
#pragma unroll
            for (int a = 0; a < NA; ++a) sb[a] = ab[a] = Real(0);
#pragma unroll
            for (int q = 0; q < NA * (NA + 1) / 2; ++q) lb[q] = Real(0);
            Real aliveBar = Real(0);  // adjoint of the notional alive after the date being undone
            for (int i = nSteps - 1; i >= 0; --i)
            {
                const int e = p.evAtStep[i + 1];
                if (e >= 0)
                {
                    const Real num = tab[L.num + e];
                    Real sp[NA];
#pragma unroll
                    for (int a = 0; a < NA; ++a) sp[a] = a < nA ? SS(ap, i * nA + a) : Real(0);
                    if (basket)
                    {
                        Real b = Real(0);
#pragma unroll
                        for (int a = 0; a < NA; ++a)
                            if (a < nA) b = b + sAsset[a] * sp[a];
                        Real bb = Real(0), nb = Real(0);
                        for (int k = 0; k < nPay; ++k)
                        {
                            const Real m = b - sK[k];
                            if (m > Real(0))
                            {
                                bb += sW[k] / num;
                                nb -= sW[k] * (m / num) / num;
                            }
                        }
#pragma unroll
                        for (int a = 0; a < NA; ++a)
                            if (a < nA) sb[a] += bb * sAsset[a];
                        fix_add(&sAcc[2 * (L.num + e)], nb);
                    }
                    else
                    {
                        const Real A = SA(ap, e), w0 = sW[0];
                        int wi;
                        const Real worst = worstOf(sp, wi);
                        Real worstBar, payE;
                        if (e == nEv - 1)
                        {
                            const Real m = kput - worst;
                            const Real put = m > Real(0) ? m : Real(0);
                            payE = A * cpn * dtc / num + A / num - A * put / kput / num;
                            aliveBar = w0 * (cpn * dtc + Real(1) - put / kput) / num;
                            worstBar = m > Real(0) ? w0 * A / kput / num : Real(0);
                        }
                        else
                        {
                            const Real x = (ko + sm - worst) / Real(2) / sm;
                            const bool inside = x > Real(0) && x < Real(1);
                            const Real f = x > Real(1) ? Real(1) : x > Real(0) ? x : Real(0);
                            payE = A * cpn * dtc / num + (A - A * f) / num;
                            const Real fBar = -w0 * A / num + aliveBar * A;
                            aliveBar = w0 * (cpn * dtc + Real(1) - f) / num + aliveBar * f;
                            worstBar = inside ? -fBar / Real(2) / sm : Real(0);
                        }
                        fix_add(&sAcc[2 * (L.num + e)], -w0 * payE / num);
#pragma unroll
                        for (int a = 0; a < NA; ++a)
                            if (a == wi) sb[a] += worstBar / sAsset[a];
                    }
                }
                // undo step i, asset by asset (assets are coupled only through the Gaussians)
#pragma unroll
                for (int a = 0; a < NA; ++a)
                {
                    if (a >= nA) break;
                    Real cw = Real(0);
                    Real wv[NA];
#pragma unroll
                    for (int b = 0; b <= a; ++b)
                    {
                        wv[b] = sgn * SW(i * nA + b);
                        cw += chol[a * nA + b] * wv[b];
                    }
                    const Real sd = tab[L.std_ + i * nA + a], dr = tab[L.drift + i * nA + a],
                               ff = tab[L.ff + i * nA + a], al = tab[L.alpha + a];
                    const Real sPrev = i > 0 ? SS(ap, (i - 1) * nA + a) : tab[L.s0 + a];
                    const Real fwd = sPrev * ff, abar = sb[a];
                    const int dy = sDyn[a];
                    Real fwdBar, cwBar;
                    if (dy == MD_NORMAL)
                    {
                        fwdBar = abar;
                        fix_add(&sAcc[2 * (L.std_ + i * nA + a)], abar * cw);
                        cwBar = abar * sd;
                    }
                    else
                    {
                        const Real E = exp(dr + sd * cw);
                        const Real base = dy == MD_LOGNORMAL ? fwd : dy == MD_SURNORMAL ? fwd + al : fwd - al;
                        const Real ub = abar * base * E;
                        fwdBar = abar * E;
                        if (dy == MD_SURNORMAL) ab[a] += abar * (E - Real(1));
                        if (dy == MD_SUBNORMAL) ab[a] += abar * (Real(1) - E);
                        fix_add(&sAcc[2 * (L.drift + i * nA + a)], ub);
                        fix_add(&sAcc[2 * (L.std_ + i * nA + a)], ub * cw);
                        cwBar = ub * sd;
                    }
                    fix_add(&sAcc[2 * (L.ff + i * nA + a)], fwdBar * sPrev);
                    sb[a] = fwdBar * ff;
#pragma unroll
                    for (int b = 0; b <= a; ++b) lb[a * (a + 1) / 2 + b] += cwBar * wv[b];
                }
            }
#pragma unroll
            for (int a = 0; a < NA; ++a)
                if (a < nA)
                {
                    fix_add(&sAcc[2 * (L.s0 + a)], sb[a]);
                    if (ab[a] != Real(0)) fix_add(&sAcc[2 * (L.alpha + a)], ab[a]);
#pragma unroll
                    for (int b = 0; b <= a; ++b)
                        if (lb[a * (a + 1) / 2 + b] != Real(0))
                            fix_add(&sAcc[2 * (L.chol + a * nA + b)], lb[a * (a + 1) / 2 + b]);
                }
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
            MrgState st = mrg_jump(p.seed1, p.seed2, (unsigned long long)(p.firstPath / 2 + u0) * dim, p.mrgJumpA,
                                   p.mrgJumpB);
            for (long long u = u0; u < u1; ++u)
                runUnit((2 * u + 1 < p.nPath) ? 2 : 1, [&](int) { return mrg_gauss<Real>(mrg_next(st)); });
        }
    }
    else
    {
        const int pitch = dim | 1;
        unsigned* base = reinterpret_cast<unsigned*>(smem + S.base) + wib * pitch;
        const long long nB = p.nPath / 32 + 1;
        for (;;)
        {
            // warps take batches from the launch counter one at a time: the warps of an SM
            // progress at different speeds, and a fixed share each would leave the last ones alone
            unsigned long long bc = 0;
            if (lane == 0) bc = atomicAdd(p.claim, 1ull);
            const long long b = (long long)__shfl_sync(0xffffffffu, bc, 0);
            if (b >= nB) break;
            __syncwarp();
            for (int d = lane; d < dim; d += 32)
                base[d] = sobol_state(p.sobolDir, dim, d, (unsigned long long)(p.firstPath + b * 32));
            __syncwarp();
            const long long n = b * 32 + lane;
            if (n >= 1 && n <= p.nPath)
                runUnit(1, [&](int d) {
                    return sobol_gauss<Real>(base[d] ^ sobol_state(p.sobolDir, dim, d, (unsigned long long)lane));
                });
        }
    }
    __syncthreads();
    for (int i = tid; i < p.nAcc; i += MD_BLOCK) fix_flush(&p.acc[2 * i], &sAcc[2 * i]);
}

template <int RNGK, class Real>
const void* md_ptr_na(int nA)
{
    if (nA <= 4) return (const void*)&md_kernel<RNGK, Real, 4>;
    if (nA <= 8) return (const void*)&md_kernel<RNGK, Real, 8>;
    return (const void*)&md_kernel<RNGK, Real, 16>;
}

const void* md_ptr(int rng, int fp32, int nA)
{
    if (rng == RNG_MRG) return fp32 ? md_ptr_na<RNG_MRG, float>(nA) : md_ptr_na<RNG_MRG, double>(nA);
    return fp32 ? md_ptr_na<RNG_SOBOL, float>(nA) : md_ptr_na<RNG_SOBOL, double>(nA);
}

}  // namespace

size_t md_smem_bytes(int rng, int fp32, const McParams& p) { return md_smem(rng, fp32, p).total; }

// reverse-sweep scratch fields per thread (each a Real per thread of the grid)
int md_scratch_fields(int rng, const McParams& p)
{
    const int NP = rng == RNG_MRG ? 2 : 1, dim = p.nSteps * p.nA;
    return dim + NP * dim + NP * p.nEv;
}

int md_occupancy(int rng, int fp32, int nA, size_t smem, int* occ)
{
    const void* fn = md_ptr(rng, fp32, nA);
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(occ, fn, MD_BLOCK, smem);
    return (int)e;
}

int launch_md(int rng, int fp32, int grid, size_t smem, const McParams& p, void* stream)
{
    McParams q = p;
    void* args[] = {&q};
    return (int)cudaLaunchKernel(md_ptr(rng, fp32, p.nA), dim3(grid), dim3(MD_BLOCK), args, smem, (cudaStream_t)stream);
}

}  // namespace cf
