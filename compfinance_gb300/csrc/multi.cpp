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

const ProductDesc* Context::productOf(const Plan& plan) const
{
    for (auto& kv : products)
        if (kv.second.version == plan.pver) return &kv.second;
    return nullptr;
}

bool Context::multiFast(const Plan& plan) const
{
    return plan.prod == PROD_EUROPEANS && plan.nEv <= kMultiMaxE && productOf(plan) != nullptr;
}

int Context::enqueueMulti(Slot& slot, Plan& plan, const cf_num_param& num)
{
    const ProductDesc* pd = productOf(plan);
    if (!multiFast(plan)) return fail(CF_E_UNSUPPORTED, "multi kernel: European portfolios of <= 16 maturities");
    if (num.numPath <= 0) return fail(CF_E_ARG, "numPath must be positive");
    const bool sobol = num.useSobol != 0, fp32 = num.precision == CF_FP32;
    if (sobol && !plan.sobolOk) return fail(CF_E_SHAPE, "Sobol dimension exceeds the direction numbers");
    cudaStream_t st = slot.stream;
    // strikes of each maturity sorted; payoff index of each sorted position
    const int nEv = plan.nEv;
    slot.evOff.assign(nEv + 1, 0);
    slot.orig.clear();
    slot.ks.clear();
    for (int e = 0; e < nEv; ++e)
    {
        const int k0 = pd->payOff[e], k1 = pd->payOff[e + 1];
        std::vector<int> idx(k1 - k0);
        std::iota(idx.begin(), idx.end(), k0);
        std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return pd->kflat[a] < pd->kflat[b]; });
        for (int k : idx)
        {
            slot.orig.push_back(k);
            slot.ks.push_back(pd->kflat[k]);
        }
        slot.evOff[e + 1] = slot.evOff[e] + (k1 - k0) + 1;
    }
    const int nBuckets = slot.evOff[nEv];
    const int nParam = plan.model == MODEL_BS ? 8 : plan.nParam;  // BS: (a, b) per parameter
    std::vector<float> ksf(slot.ks.begin(), slot.ks.end());
    auto up = [](size_t n) { return 256 * ((n + 255) / 256); };
    const size_t offKs = up(slot.evOff.size() * 4);
    const size_t offKsf = offKs + up(slot.ks.size() * 8);
    const size_t offAccR = offKsf + up(ksf.size() * 4);
    slot.accRBytes = size_t(nBuckets) * nParam * 16;
    slot.accVBytes = size_t(nBuckets) * 5 * 16;
    const size_t offAccV = offAccR + up(slot.accRBytes);
    const size_t offErr = offAccV + up(slot.accVBytes);
    int rc = slot.multiBuf.ensure(offErr + 256);
    if (rc) return rc;
    if ((rc = slot.hostAcc.ensure(slot.accRBytes + slot.accVBytes + 16))) return rc;
    if ((rc = slot.hostW.ensure(slot.evOff.size() * 4 + slot.ks.size() * 12 + 64))) return rc;
    char* hw = static_cast<char*>(slot.hostW.ptr);
    std::memcpy(hw, slot.evOff.data(), slot.evOff.size() * 4);
    std::memcpy(hw + slot.evOff.size() * 4, slot.ks.data(), slot.ks.size() * 8);
    std::memcpy(hw + slot.evOff.size() * 4 + slot.ks.size() * 8, ksf.data(), ksf.size() * 4);
    char* d = static_cast<char*>(slot.multiBuf.ptr);
    cudaError_t e = cudaMemcpyAsync(d, hw, slot.evOff.size() * 4, cudaMemcpyHostToDevice, st);
    if (!e) e = cudaMemcpyAsync(d + offKs, hw + slot.evOff.size() * 4, slot.ks.size() * 8, cudaMemcpyHostToDevice, st);
    if (!e)
        e = cudaMemcpyAsync(d + offKsf, hw + slot.evOff.size() * 4 + slot.ks.size() * 8, ksf.size() * 4,
                            cudaMemcpyHostToDevice, st);
    if (!e) e = cudaMemsetAsync(d + offAccR, 0, offErr + 16 - offAccR, st);
    if (e) return cuda_fail(e, "multi upload");
    h2d += slot.evOff.size() * 4 + slot.ks.size() * 12;

    MultiParams mp;
    mp.p = plan.base;
    McParams& p = mp.p;
    p.nPath = num.numPath;
    p.seed1 = unsigned(num.seed1);
    p.seed2 = unsigned(num.seed2);
    p.mrgJumpA = jumpA;
    p.mrgJumpB = jumpB;
    p.err = reinterpret_cast<int*>(d + offErr);
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
        if ((rc = slot.scratch.ensure(size_t(perThread) * p.scratchThreads * (fp32 ? 4 : 8)))) return rc;
        p.scratch = slot.scratch.ptr;
    }
    rc = launch_multi(plan.model, sobol, fp32, int(grid), smem, mp, st);
    if (rc) return cuda_fail(cudaError_t(rc), "multi kernel launch");
    char* ha = static_cast<char*>(slot.hostAcc.ptr);
    e = cudaMemcpyAsync(ha, mp.accRisk, slot.accRBytes, cudaMemcpyDeviceToHost, st);
    if (!e) e = cudaMemcpyAsync(ha + slot.accRBytes, mp.accVal, slot.accVBytes, cudaMemcpyDeviceToHost, st);
    if (!e) e = cudaMemcpyAsync(ha + slot.accRBytes + slot.accVBytes, p.err, 4, cudaMemcpyDeviceToHost, st);
    if (!e && !slot.done) e = cudaEventCreateWithFlags(&slot.done, cudaEventDisableTiming);
    if (!e) e = cudaEventRecord(slot.done, st);
    if (e) return cuda_fail(e, "multi download");
    d2h += slot.accRBytes + slot.accVBytes + 4;
    slot.plan = &plan;
    slot.multi = true;
    slot.risk = true;
    slot.multiParams = nParam;
    slot.multiPaths = num.numPath;
    slot.launches = 1;
    return CF_OK;
}

int Context::finishMulti(Slot& slot, double* values, double* risks)
{
    const Plan& plan = *slot.plan;
    const char* ha = static_cast<const char*>(slot.hostAcc.ptr);
    const long long* accR = reinterpret_cast<const long long*>(ha);
    const long long* accV = reinterpret_cast<const long long*>(ha + slot.accRBytes);
    const int flag = *reinterpret_cast<const int*>(ha + slot.accRBytes + slot.accVBytes);
    if (flag) return fail(CF_E_DEVICE, "kernel error flag " + std::to_string(flag));
    // suffix sums over buckets m > j for each sorted strike j
    const double n = double(slot.multiPaths);
    auto V = [](const long long* a, size_t i) { return fix_value_host(a[2 * i], a[2 * i + 1]); };
    const int nParam = slot.multiParams, nP = plan.nParam, nEv = plan.nEv;
    std::vector<double> sumR(nParam), sumV(5);
    int sorted = 0;
    for (int ev = 0; ev < nEv; ++ev)
    {
        const int nK = slot.evOff[ev + 1] - slot.evOff[ev] - 1;
        std::fill(sumR.begin(), sumR.end(), 0.0);
        std::fill(sumV.begin(), sumV.end(), 0.0);
        for (int j = nK - 1; j >= 0; --j)
        {
            const int bk = slot.evOff[ev] + j + 1;  // bucket m = j + 1 pays strikes 0..j
            for (int q = 0; q < 5; ++q) sumV[q] += V(accV, size_t(bk) * 5 + q);
            for (int q = 0; q < nParam; ++q) sumR[q] += V(accR, size_t(bk) * nParam + q);
            const double K = slot.ks[sorted + j];
            const int k = slot.orig[sorted + j];
            if (values) values[k] = (sumV[1] - K * sumV[0]) / n;
            if (!risks) continue;
            if (plan.model == MODEL_BS)
                for (int q = 0; q < 4; ++q) risks[size_t(q) * plan.nPay + k] = (sumR[2 * q] - K * sumR[2 * q + 1]) / n;
            else
                for (int q = 0; q < nP; ++q) risks[size_t(q) * plan.nPay + k] = sumR[q] / n;
        }
        sorted += nK;
    }
    return CF_OK;
}

int Context::riskMulti(Plan& plan, const cf_num_param& num, double* values, double* risks)
{
    main.stream = stream;
    if (multiFast(plan))
    {
        int rc = enqueueMulti(main, plan, num);
        if (rc) return rc;
        return fetch(main, values, nullptr, nullptr, risks);
    }
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
    main.launches = plan.nPay;
    return CF_OK;
}

}  // namespace cf
