// AADriskMulti (main.h:269-312, mcBase.h:775-989): the risk of every payoff to every model
// parameter.
//
// European portfolios (up to 16 maturities) run the dedicated multi kernels: one adjoint per
// maturity and strike buckets (multi_kernel.cu; FP32 on Dupire: paths grouped by bucket and
// summed in shared memory, multi_risk32.cu), turned into per-payoff risks on the device by
// suffix sums (multi_finish).  Other products (one or two payoffs) run one adjoint sweep per
// payoff over the same random numbers; both give the exact per-payoff path averages.
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <vector>

#include "engine.h"
#include "multi32.h"

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
int launch_multi_aggregate(const double* risks, int nParam, int nPay, const double* w, double* out, void* stream);
int launch_multi_finish(const long long* accR, int nAccParam, int nOut, int nEv, const int* evOff, const double* ks,
                        const int* orig, int nPay, int bs, double n, double* risks, void* stream);

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

int Context::enqueueMulti(Slot& slot, Plan& plan, const cf_num_param& num, double* directRisks,
                          const double* aggWeights)
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
    const bool fast = multi32Use(plan, num);
    std::vector<float> ksf(slot.ks.begin(), slot.ks.end());
    // device buffer: inputs (bucket offsets, strikes, payoff index per sorted strike), the
    // zeroed accumulators and counters, the bucket segments of the FP32 kernels, the risks
    auto up = [](size_t n) { return 256 * ((n + 255) / 256); };
    const size_t offKs = up(slot.evOff.size() * 4);
    const size_t offKsf = offKs + up(slot.ks.size() * 8);
    const size_t offOrig = offKsf + up(ksf.size() * 4);
    const size_t offAccR = offOrig + up(slot.orig.size() * 4);
    const size_t accRBytes = size_t(nBuckets) * nParam * 16;
    slot.accVBytes = size_t(nBuckets) * 5 * 16;
    const size_t offAccV = offAccR + up(accRBytes);
    const size_t offErr = offAccV + up(slot.accVBytes);  // error flag, reverse chunk counter, batch counter
    const size_t offCnt = offErr + 256;
    const size_t offCur = offCnt + up(size_t(nBuckets) * 4);
    const size_t zeroEnd = offCur + up(size_t(nBuckets) * 4);
    const size_t offStart = zeroEnd;
    const size_t offChunk = offStart + up(size_t(nBuckets + 1) * 4);
    const size_t offRisk = offChunk + up(size_t(nBuckets + 1) * 4);
    const size_t riskBytes = size_t(plan.nParam) * plan.nPay * 8;
    const size_t offW = offRisk + up(riskBytes);  // aggregation weights, then the aggregate's risks
    const size_t offAgg = offW + up(size_t(plan.nPay) * 8);
    int rc = slot.multiBuf.ensure(offAgg + up(size_t(plan.nParam) * 8), st);
    if (rc) return rc;
    // the finished risks come back through the pinned buffer (all of them, or those of the
    // weighted aggregate), or straight into the caller's array (synchronous calls: a pageable
    // copy, which returns once the data is there)
    slot.aggW.assign(aggWeights ? aggWeights : nullptr, aggWeights ? aggWeights + plan.nPay : nullptr);
    slot.accRBytes = aggWeights ? size_t(plan.nParam) * 8 : directRisks ? 0 : riskBytes;
    if ((rc = slot.hostAcc.ensure(slot.accRBytes + slot.accVBytes + 16))) return rc;
    const size_t wBytes = slot.evOff.size() * 4 + slot.ks.size() * 12 + slot.orig.size() * 4;
    if ((rc = slot.hostW.ensure(wBytes + size_t(plan.nPay) * 8 + 64))) return rc;
    char* hw = static_cast<char*>(slot.hostW.ptr);
    char* hKs = hw + slot.evOff.size() * 4;
    char* hKsf = hKs + slot.ks.size() * 8;
    char* hOrig = hKsf + ksf.size() * 4;
    std::memcpy(hw, slot.evOff.data(), slot.evOff.size() * 4);
    std::memcpy(hKs, slot.ks.data(), slot.ks.size() * 8);
    std::memcpy(hKsf, ksf.data(), ksf.size() * 4);
    std::memcpy(hOrig, slot.orig.data(), slot.orig.size() * 4);
    char* d = static_cast<char*>(slot.multiBuf.ptr);
    cudaError_t e = cudaMemcpyAsync(d, hw, slot.evOff.size() * 4, cudaMemcpyHostToDevice, st);
    if (!e) e = cudaMemcpyAsync(d + offKs, hKs, slot.ks.size() * 8, cudaMemcpyHostToDevice, st);
    if (!e) e = cudaMemcpyAsync(d + offKsf, hKsf, ksf.size() * 4, cudaMemcpyHostToDevice, st);
    if (!e) e = cudaMemcpyAsync(d + offOrig, hOrig, slot.orig.size() * 4, cudaMemcpyHostToDevice, st);
    if (!e) e = cudaMemsetAsync(d + offAccR, 0, zeroEnd - offAccR, st);
    if (!e && aggWeights)
    {
        std::memcpy(hw + wBytes, aggWeights, size_t(plan.nPay) * 8);  // hostW holds wBytes + nPay doubles
        e = cudaMemcpyAsync(d + offW, hw + wBytes, size_t(plan.nPay) * 8, cudaMemcpyHostToDevice, st);
        h2d += size_t(plan.nPay) * 8;
    }
    if (e) return cuda_fail(e, "multi upload");
    h2d += wBytes;

    McParams p = plan.base;
    p.nPath = num.numPath;
    p.seed1 = unsigned(num.seed1);
    p.seed2 = unsigned(num.seed2);
    p.mrgJumpA = jumpA;
    p.mrgJumpB = jumpB;
    p.err = reinterpret_cast<int*>(d + offErr);
    p.claim = reinterpret_cast<unsigned long long*>(d + offErr + 64);  // multi32_forward's Sobol batch counter
    const int* dEvOff = reinterpret_cast<const int*>(d);
    long long* dAccR = reinterpret_cast<long long*>(d + offAccR);
    long long* dAccV = reinterpret_cast<long long*>(d + offAccV);
    if (fast)
    {
        // FP32 Dupire: forward, bucket segments, chunked reverse sweeps (multi_risk32.cu)
        Multi32Args A;
        A.p = p;
        A.p.invnF = sobol ? invnSobol : invnMrg;
        A.nParam = nParam;
        A.nBuckets = nBuckets;
        A.nKs = int(ksf.size());
        A.pitch = (plan.nSteps + 1) & ~1;
        A.evOff = dEvOff;
        A.ksF = reinterpret_cast<const float*>(d + offKsf);
        A.accRisk = dAccR;
        A.accVal = dAccV;
        A.cnt = reinterpret_cast<int*>(d + offCnt);
        A.cursor = reinterpret_cast<int*>(d + offCur);
        A.start = reinterpret_cast<int*>(d + offStart);
        A.chunkStart = reinterpret_cast<int*>(d + offChunk);
        A.work = reinterpret_cast<int*>(d + offErr + 16);
        const size_t nP = size_t(num.numPath), nE = size_t(nEv);
        const size_t recBytes = up(nP * A.pitch * 8), evBBytes = up(nE * nP * 2), evSBytes = up(nE * nP * 4);
        if ((rc = slot.scratch.ensure(recBytes + evBBytes + evSBytes + nE * nP * 8, st))) return rc;
        char* sc = static_cast<char*>(slot.scratch.ptr);
        A.rec = reinterpret_cast<unsigned*>(sc);
        A.evB = reinterpret_cast<unsigned short*>(sc + recBytes);
        A.evS = reinterpret_cast<float*>(sc + recBytes + evBBytes);
        A.list = reinterpret_cast<int*>(sc + recBytes + evBBytes + evSBytes);
        const size_t smemF = m32_forward_smem(sobol, A), smemR = m32_reverse_smem(A);
        int occF = 0, occR = 0;
        rc = m32_occupancy(sobol, smemF, smemR, &occF, &occR);
        if (rc) return cuda_fail(cudaError_t(rc), "multi occupancy");
        if (occF < 1 || occR < 1) return fail(CF_E_SHAPE, "multi kernel does not fit on an SM");
        const long long threadsNeeded = sobol ? (p.nPath / 32 + 1) * 32 : (p.nPath + 1) / 2;
        const long long gridF = std::max(1LL, std::min<long long>((threadsNeeded + 127) / 128, (long long)numSMs * occF));
        rc = launch_multi32(sobol, int(gridF), smemF, numSMs * occR, smemR, A, st);
        if (rc) return cuda_fail(cudaError_t(rc), "multi kernel launch");
        slot.launches = 5;
    }
    else
    {
        MultiParams mp;
        mp.p = p;
        mp.nParam = nParam;
        mp.evOff = dEvOff;
        mp.ksD = reinterpret_cast<const double*>(d + offKs);
        mp.ksF = reinterpret_cast<const float*>(d + offKsf);
        mp.accRisk = dAccR;
        mp.accVal = dAccV;
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
            mp.p.scratchThreads = grid * 128;
            mp.p.scratchFields = 1 + 3 * NP;
            if ((rc = slot.scratch.ensure(size_t(perThread) * mp.p.scratchThreads * (fp32 ? 4 : 8), st))) return rc;
            mp.p.scratch = slot.scratch.ptr;
        }
        rc = launch_multi(plan.model, sobol, fp32, int(grid), smem, mp, st);
        if (rc) return cuda_fail(cudaError_t(rc), "multi kernel launch");
        slot.launches = 2;
    }
    double* dRisk = reinterpret_cast<double*>(d + offRisk);
    rc = launch_multi_finish(dAccR, nParam, plan.model == MODEL_BS ? 4 : plan.nParam, nEv, dEvOff,
                             reinterpret_cast<const double*>(d + offKs), reinterpret_cast<const int*>(d + offOrig),
                             plan.nPay, plan.model == MODEL_BS ? 1 : 0, double(num.numPath), dRisk, st);
    if (rc) return cuda_fail(cudaError_t(rc), "multi finish launch");
    double* dAgg = reinterpret_cast<double*>(d + offAgg);
    if (aggWeights)
    {
        rc = launch_multi_aggregate(dRisk, plan.nParam, plan.nPay, reinterpret_cast<const double*>(d + offW), dAgg, st);
        if (rc) return cuda_fail(cudaError_t(rc), "multi aggregate launch");
    }
    char* ha = static_cast<char*>(slot.hostAcc.ptr);
    e = cudaSuccess;
    if (slot.accRBytes) e = cudaMemcpyAsync(ha, aggWeights ? dAgg : dRisk, slot.accRBytes, cudaMemcpyDeviceToHost, st);
    if (!e) e = cudaMemcpyAsync(ha + slot.accRBytes, dAccV, slot.accVBytes, cudaMemcpyDeviceToHost, st);
    if (!e) e = cudaMemcpyAsync(ha + slot.accRBytes + slot.accVBytes, p.err, 4, cudaMemcpyDeviceToHost, st);
    if (!e && directRisks && !aggWeights) e = cudaMemcpyAsync(directRisks, dRisk, riskBytes, cudaMemcpyDeviceToHost, st);
    if (!e && !slot.done) e = cudaEventCreateWithFlags(&slot.done, cudaEventDisableTiming);
    if (!e) e = cudaEventRecord(slot.done, st);
    if (e) return cuda_fail(e, "multi download");
    d2h += (aggWeights ? slot.accRBytes : riskBytes) + slot.accVBytes + 4;
    slot.plan = &plan;
    slot.planRef = plan.weak_from_this().lock();
    slot.multi = true;
    slot.risk = true;
    slot.multiParams = nParam;
    slot.multiPaths = num.numPath;
    return CF_OK;
}

bool Context::multi32Use(const Plan& plan, const cf_num_param& num) const
{
    if (!plan.multi32 || num.precision != CF_FP32 || plan.model != MODEL_DUPIRE) return false;
    // list positions are int32
    if ((long long)plan.nEv * num.numPath >= (1LL << 30)) return false;
    const char* env = std::getenv("CF_FAST32");
    return !(env && env[0] == '0');
}

int Context::finishMulti(Slot& slot, double* values, double* risks, double* aggregate)
{
    const Plan& plan = *slot.plan;
    const char* ha = static_cast<const char*>(slot.hostAcc.ptr);
    const long long* accV = reinterpret_cast<const long long*>(ha + slot.accRBytes);
    const int flag = *reinterpret_cast<const int*>(ha + slot.accRBytes + slot.accVBytes);
    if (flag) return fail(CF_E_DEVICE, "kernel error flag " + std::to_string(flag));
    // risks: finished on the device (multi_finish); values: suffix sums over buckets m > j for
    // each sorted strike j
    if (risks && slot.accRBytes) std::memcpy(risks, ha, slot.accRBytes);
    const bool agg = aggregate && !slot.aggW.empty();
    std::vector<double> own;
    if (!values && agg)
    {
        own.resize(plan.nPay);
        values = own.data();
    }
    if (!values) return CF_OK;
    const double n = double(slot.multiPaths);
    auto V = [](const long long* a, size_t i) { return fix_value_host(a[2 * i], a[2 * i + 1]); };
    const int nEv = plan.nEv;
    std::vector<double> sumV(5);
    int sorted = 0;
    for (int ev = 0; ev < nEv; ++ev)
    {
        const int nK = slot.evOff[ev + 1] - slot.evOff[ev] - 1;
        std::fill(sumV.begin(), sumV.end(), 0.0);
        for (int j = nK - 1; j >= 0; --j)
        {
            const int bk = slot.evOff[ev] + j + 1;  // bucket m = j + 1 pays strikes 0..j
            for (int q = 0; q < 5; ++q) sumV[q] += V(accV, size_t(bk) * 5 + q);
            const double K = slot.ks[sorted + j];
            values[slot.orig[sorted + j]] = (sumV[1] - K * sumV[0]) / n;
        }
        sorted += nK;
    }
    if (agg)
    {
        double a = 0.0;
        for (int k = 0; k < plan.nPay; ++k) a += slot.aggW[k] * values[k];
        *aggregate = a;
    }
    return CF_OK;
}

int Context::aggregateRisk(Plan& plan, const cf_num_param& num, const double* weights, double* values,
                           double* aggregate, double* risks)
{
    main.stream = stream;
    // FP32 European portfolios on Dupire: the portfolio kernels (every payoff's risks, then their
    // weighted sum on the device) take the work in a fraction of the time of one aggregated
    // adjoint through the generic kernel; the risks are the same linear functional of the paths
    if (multiFast(plan) && multi32Use(plan, num))
    {
        int rc = enqueueMulti(main, plan, num, nullptr, weights);
        if (rc) return rc;
        return fetch(main, values, nullptr, aggregate, risks);
    }
    int rc = enqueue(main, plan, num, true, weights);
    if (rc) return rc;
    return fetch(main, values, nullptr, aggregate, risks);
}

int Context::riskMulti(Plan& plan, const cf_num_param& num, double* values, double* risks)
{
    main.stream = stream;
    if (multiFast(plan))
    {
        int rc = enqueueMulti(main, plan, num, risks);
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
