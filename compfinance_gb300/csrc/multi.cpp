// AADriskMulti (main.h:269-312, mcBase.h:775-989): the risk of every payoff to every model
// parameter.
//
// European portfolios (up to 16 maturities) run the dedicated multi kernel (multi_kernel.cu):
// one adjoint per maturity and strike buckets, turned into per-payoff risks here by suffix
// sums.  Other products (one or two payoffs) run one adjoint sweep per payoff over the same
// random numbers; both give the exact per-payoff path averages.
#include <algorithm>
#include <cstring>
#include <numeric>
#include <vector>

#include "engine.h"

namespace cf {

struct MultiParams
{
    McParams p;
    int nParam;
    const int* evOff;
    const double* ksD;
    const float* ksF;
    long long* accRisk;
    long long* accVal;
};
size_t multi_smem_bytes(int model, int rng, int fp32, const McParams& p, int nBuckets);
int multi_occupancy(int model, int rng, int fp32, size_t smem, int* occ);
int launch_multi(int model, int rng, int fp32, int grid, size_t smem, const MultiParams& mp, void* stream);

constexpr int kMultiMaxE = 16;

int Context::riskMulti(Plan& plan, const cf_num_param& num, double* values, double* risks)
{
    const ProductDesc* pd = nullptr;
    for (auto& kv : products)
        if (kv.second.version == plan.pver) pd = &kv.second;
    if (plan.prod != PROD_EUROPEANS || plan.nEv > kMultiMaxE || !pd)
    {
        std::vector<double> w(plan.nPay, 0.0), r(plan.nParam);
        for (int k = 0; k < plan.nPay; ++k)
        {
            std::fill(w.begin(), w.end(), 0.0);
            w[k] = 1.0;
            int rc = enqueue(plan, num, true, w.data());
            if (rc) return rc;
            rc = fetch(k == 0 ? values : nullptr, nullptr, nullptr, r.data());
            if (rc) return rc;
            for (int j = 0; j < plan.nParam; ++j) risks[size_t(j) * plan.nPay + k] = r[j];
        }
        launches = plan.nPay;
        return CF_OK;
    }
    if (num.numPath <= 0) return fail(CF_E_ARG, "numPath must be positive");
    const bool sobol = num.useSobol != 0, fp32 = num.precision == CF_FP32;
    if (sobol && !plan.sobolOk) return fail(CF_E_SHAPE, "Sobol dimension exceeds the direction numbers");
    // strikes of each maturity sorted; payoff index of each sorted position
    const int nEv = plan.nEv;
    std::vector<int> evOff(nEv + 1, 0), orig;
    std::vector<double> ks;
    for (int e = 0; e < nEv; ++e)
    {
        const int k0 = pd->payOff[e], k1 = pd->payOff[e + 1];
        std::vector<int> idx(k1 - k0);
        std::iota(idx.begin(), idx.end(), k0);
        std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return pd->kflat[a] < pd->kflat[b]; });
        for (int k : idx)
        {
            orig.push_back(k);
            ks.push_back(pd->kflat[k]);
        }
        evOff[e + 1] = evOff[e] + (k1 - k0) + 1;
    }
    const int nBuckets = evOff[nEv];
    const int nParam = plan.model == MODEL_BS ? 8 : plan.nParam;  // BS: (a, b) per parameter
    std::vector<float> ksf(ks.begin(), ks.end());
    const size_t offKs = 256 * ((evOff.size() * 4 + 255) / 256);
    const size_t offKsf = offKs + 256 * ((ks.size() * 8 + 255) / 256);
    const size_t offAccR = offKsf + 256 * ((ksf.size() * 4 + 255) / 256);
    const size_t accRBytes = size_t(nBuckets) * nParam * 16, accVBytes = size_t(nBuckets) * 5 * 16;
    const size_t offAccV = offAccR + 256 * ((accRBytes + 255) / 256);
    int rc = multiBuf.ensure(offAccV + accVBytes);
    if (rc) return rc;
    char* d = static_cast<char*>(multiBuf.ptr);
    cudaError_t e = cudaMemcpyAsync(d, evOff.data(), evOff.size() * 4, cudaMemcpyHostToDevice, stream);
    if (!e) e = cudaMemcpyAsync(d + offKs, ks.data(), ks.size() * 8, cudaMemcpyHostToDevice, stream);
    if (!e) e = cudaMemcpyAsync(d + offKsf, ksf.data(), ksf.size() * 4, cudaMemcpyHostToDevice, stream);
    if (!e) e = cudaMemsetAsync(d + offAccR, 0, offAccV + accVBytes - offAccR, stream);
    if (!e) e = cudaMemsetAsync(err.ptr, 0, 4, stream);
    if (e) return cuda_fail(e, "multi upload");
    h2d += evOff.size() * 4 + ks.size() * 12;

    MultiParams mp;
    mp.p = plan.base;
    McParams& p = mp.p;
    p.nPath = num.numPath;
    p.seed1 = unsigned(num.seed1);
    p.seed2 = unsigned(num.seed2);
    p.mrgJumpA = jumpA;
    p.mrgJumpB = jumpB;
    p.err = static_cast<int*>(err.ptr);
    mp.nParam = nParam;
    mp.evOff = reinterpret_cast<const int*>(d);
    mp.ksD = reinterpret_cast<const double*>(d + offKs);
    mp.ksF = reinterpret_cast<const float*>(d + offKsf);
    mp.accRisk = reinterpret_cast<long long*>(d + offAccR);
    mp.accVal = reinterpret_cast<long long*>(d + offAccV);

    const size_t smem = multi_smem_bytes(plan.model, sobol, fp32, p, nBuckets);
    int occ = 0;
    rc = multi_occupancy(plan.model, sobol, fp32, smem, &occ);
    if (rc) return cuda_fail(cudaError_t(rc), "multi occupancy");
    if (occ < 1) return fail(CF_E_SHAPE, "multi kernel does not fit on an SM");
    const long long threadsNeeded = sobol ? (p.nPath / 32 + 1) * 32 : (p.nPath + 1) / 2;
    long long grid = std::min<long long>((threadsNeeded + 127) / 128, (long long)numSMs * occ);
    const int NP = sobol ? 1 : 2;
    const long long perThread = (long long)(1 + 3 * NP) * (plan.nSteps + 1);
    grid = std::max(1LL, std::min(grid, ((1LL << 31) - 1) / perThread / 128));
    if (plan.model == MODEL_DUPIRE)
    {
        p.scratchThreads = grid * 128;
        p.scratchFields = 1 + 3 * NP;
        if ((rc = scratch.ensure(size_t(perThread) * p.scratchThreads * (fp32 ? 4 : 8)))) return rc;
        p.scratch = scratch.ptr;
    }
    rc = launch_multi(plan.model, sobol, fp32, int(grid), smem, mp, stream);
    if (rc) return cuda_fail(cudaError_t(rc), "multi kernel launch");
    launches = 1;

    std::vector<long long> accR(accRBytes / 8), accV(accVBytes / 8);
    int flag = 0;
    e = cudaMemcpyAsync(accR.data(), mp.accRisk, accRBytes, cudaMemcpyDeviceToHost, stream);
    if (!e) e = cudaMemcpyAsync(accV.data(), mp.accVal, accVBytes, cudaMemcpyDeviceToHost, stream);
    if (!e) e = cudaMemcpyAsync(&flag, err.ptr, 4, cudaMemcpyDeviceToHost, stream);
    if (!e) e = cudaStreamSynchronize(stream);
    if (e) return cuda_fail(e, "multi fetch");
    d2h += accRBytes + accVBytes + 4;
    if (flag) return fail(CF_E_DEVICE, "kernel error flag " + std::to_string(flag));

    // suffix sums over buckets m > j for each sorted strike j
    const double n = double(num.numPath);
    auto V = [&](const std::vector<long long>& a, size_t i) { return fix_value_host(a[2 * i], a[2 * i + 1]); };
    const int nP = plan.nParam;
    std::vector<double> sumR(nParam), sumV(5);
    int sorted = 0;
    for (int ev = 0; ev < nEv; ++ev)
    {
        const int nK = evOff[ev + 1] - evOff[ev] - 1;
        std::fill(sumR.begin(), sumR.end(), 0.0);
        std::fill(sumV.begin(), sumV.end(), 0.0);
        for (int j = nK - 1; j >= 0; --j)
        {
            const int bk = evOff[ev] + j + 1;  // bucket m = j + 1 pays strikes 0..j
            for (int q = 0; q < 5; ++q) sumV[q] += V(accV, size_t(bk) * 5 + q);
            for (int q = 0; q < nParam; ++q) sumR[q] += V(accR, size_t(bk) * nParam + q);
            const double K = ks[sorted + j];
            const int k = orig[sorted + j];
            if (values) values[k] = (sumV[1] - K * sumV[0]) / n;
            if (plan.model == MODEL_BS)
                for (int q = 0; q < 4; ++q) risks[size_t(q) * plan.nPay + k] = (sumR[2 * q] - K * sumR[2 * q + 1]) / n;
            else
                for (int q = 0; q < nP; ++q) risks[size_t(q) * plan.nPay + k] = sumR[q] / n;
        }
        sorted += nK;
    }
    return CF_OK;
}

}  // namespace cf
