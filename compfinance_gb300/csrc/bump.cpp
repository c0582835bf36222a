// bumpRisk (main.h:316-359): risks by one-sided finite differences.  Every model parameter is
// bumped by 1e-8 in turn and the product repriced on the same random numbers (common random
// numbers: the same seeds or Sobol points), risk[i][k] = 1e8 (value_k(bumped) - value_k(base)).
// The valuation is FP64 whatever the requested precision: a 1e-8 bump is below FP32 resolution.
//
// Two procedures give the same numbers:
//  * reprice: the reference's own procedure, one full valuation of a freshly lowered bumped
//    model per parameter (any model and product);
//  * pathwise (Dupire local-vol bumps): a bumped local-vol node changes only the paths whose
//    interpolation touches it, and an untouched path is bit-identical to its base path, so the
//    kernel re-simulates only the touched paths of each node and sums the exact payoff
//    differences (bump_kernel.cu).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "bump_params.h"
#include "engine.h"

namespace cf {

const void* dupire_bump64_ptr(int prod, int rng);

namespace {

constexpr double kBump = 1.0e-08;  // main.h:346


}  // namespace

int bump_risk_reprice(Context& c, const std::string& mid, const std::string& pid, const cf_num_param& num,
                      double* values, double* risks)
{
    Plan* base = nullptr;
    int rc = c.getPlan(mid, pid, base);
    if (rc) return rc;
    cf_num_param n64 = num;
    n64.precision = CF_FP64;
    const int nPay = base->nPay, nParam = base->nParam;
    std::vector<double> v0(nPay), vb(nPay);
    if ((rc = c.enqueue(*base, n64, false, nullptr)) || (rc = c.fetch(v0.data(), nullptr, nullptr, nullptr))) return rc;
    if (values) std::memcpy(values, v0.data(), size_t(nPay) * 8);
    const ModelDesc& m0 = c.models.at(mid);
    const ProductDesc& pd = c.products.at(pid);
    ModelDesc mb = m0;
    for (int i = 0; i < nParam; ++i)
    {
        double& x = mb.param(i);
        const double keep = x;
        x += kBump;
        Plan bp;
        if ((rc = c.buildPlan(mb, pd, bp))) return rc;
        if ((rc = c.enqueue(bp, n64, false, nullptr)) || (rc = c.fetch(vb.data(), nullptr, nullptr, nullptr)))
            return rc;
        x = keep;
        for (int k = 0; k < nPay; ++k) risks[size_t(i) * nPay + k] = 1.0e+08 * (vb[k] - v0[k]);
    }
    return CF_OK;
}

bool bump_pathwise_ok(const Plan& plan)
{
    return plan.model == MODEL_DUPIRE &&
           (plan.prod == PROD_UOC || plan.prod == PROD_EUROPEAN || plan.prod == PROD_EUROPEANS);
}

int bump_risk_pathwise(Context& c, Plan& plan, const ModelDesc& m, const ProductDesc& pd, const cf_num_param& num,
                       double* values, double* risks)
{
    const bool sobol = num.useSobol != 0;
    if (sobol && !plan.sobolOk) return fail(CF_E_SHAPE, "bumpRisk() : Sobol dimension exceeds the direction numbers");
    const int nPay = plan.nPay, nParam = plan.nParam, NP = sobol ? 1 : 2;
    McParams p = plan.base;
    p.nPath = num.numPath;
    p.seed1 = unsigned(num.seed1);
    p.seed2 = unsigned(num.seed2);
    p.mrgJumpA = c.jumpA;
    p.mrgJumpB = c.jumpB;
    BumpArgs b{};
    b.nParam = nParam;
    b.maskWords = (p.nS * p.nT + 31) / 32;
    // the spot bump (plan lowering's constants from the bumped spot)
    b.x0Bumped = std::log(m.spot + BUMP_SIZE);
    const double smooth = std::exp(b.x0Bumped) * pd.smooth;
    b.barSmoothB = pd.barrier + smooth;
    b.minusSmoothB = pd.barrier - smooth;
    b.twoSmoothB = 2 * smooth;
    b.logBandB = (b.minusSmoothB > 0 ? std::log(b.minusSmoothB) : -INFINITY) - 1e-9;
    // grid: units (antithetic pairs or Sobol paths) over at most 4 blocks per SM
    const long long units = sobol ? num.numPath : (num.numPath + 1) / 2;
    const long long grid = std::max(1LL, std::min<long long>((units + 127) / 128, 4LL * c.numSMs));
    const BumpRows R = bump_rows(p.nSteps, nPay, NP, b.maskWords);
    const size_t threads = size_t(grid) * 128;
    const size_t scrBytes = threads * (size_t(R.nDouble) * 8 + size_t(R.nInt) * 4 + size_t(R.nMask) * 4);
    const size_t nAcc = size_t(nParam + 1) * nPay;
    Slot& sl = c.main;
    sl.stream = c.stream;
    int rc;
    if ((rc = sl.scratch.ensure(scrBytes)) || (rc = sl.multiBuf.ensure(nAcc * 16))) return rc;
    b.scratch = sl.scratch.ptr;
    b.acc = static_cast<long long*>(sl.multiBuf.ptr);
    cudaError_t e = cudaMemsetAsync(b.acc, 0, nAcc * 16, sl.stream);
    if (e != cudaSuccess) return cuda_fail(e, "bumpRisk() : accumulator reset");
    const void* fn = dupire_bump64_ptr(plan.prod, sobol ? RNG_SOBOL : RNG_MRG);
    void* args[] = {&p, &b};
    if ((e = cudaLaunchKernel(fn, dim3(unsigned(grid)), dim3(128), args, 0, sl.stream)) != cudaSuccess)
        return cuda_fail(e, "bumpRisk() : kernel launch");
    std::vector<long long> acc(nAcc * 2);
    if ((e = cudaMemcpyAsync(acc.data(), b.acc, nAcc * 16, cudaMemcpyDeviceToHost, sl.stream)) != cudaSuccess ||
        (e = cudaStreamSynchronize(sl.stream)) != cudaSuccess)
        return cuda_fail(e, "bumpRisk() : result download");
    c.d2h += nAcc * 16;
    const double n = double(num.numPath);
    for (int i = 0; i < nParam; ++i)
        for (int k = 0; k < nPay; ++k)
        {
            const size_t q = size_t(i) * nPay + k;
            risks[q] = 1.0e+08 * (fix_value_host(acc[2 * q], acc[2 * q + 1]) / n);
        }
    if (values)
        for (int k = 0; k < nPay; ++k)
        {
            const size_t q = size_t(nParam) * nPay + k;
            values[k] = fix_value_host(acc[2 * q], acc[2 * q + 1]) / n;
        }
    return CF_OK;
}

}  // namespace cf

using namespace cf;

extern "C" int cf_bump_risk(cf_context* ctx, const char* modelId, const char* productId, const cf_num_param* num,
                            int method, double* values, double* risks)
{
    if (!ctx) return fail(CF_E_ARG, "null context");
    if (!num || !risks) return fail(CF_E_ARG, "null argument");
    std::lock_guard<std::mutex> lock(ctx->mu);
    Context& c = ctx->c;
    cudaSetDevice(c.device);
    const std::string mid = modelId ? modelId : "", pid = productId ? productId : "";
    if (!c.models.count(mid) || !c.products.count(pid))
        return fail(CF_E_NOTFOUND, "bumpRisk() : Could not retrieve model and product");
    if (method != CF_BUMP_AUTO && method != CF_BUMP_REPRICE && method != CF_BUMP_PATHWISE)
        return fail(CF_E_ARG, "bumpRisk() : unknown method");
    Plan* plan = nullptr;
    int rc = c.getPlan(mid, pid, plan);
    if (rc) return rc;
    const bool pathwise = bump_pathwise_ok(*plan);
    if (method == CF_BUMP_PATHWISE && !pathwise)
        return fail(CF_E_ARG, "bumpRisk() : pathwise bumps need a Dupire model and a European, barrier or "
                              "European portfolio product");
    if (method == CF_BUMP_REPRICE || !pathwise) return bump_risk_reprice(c, mid, pid, *num, values, risks);
    return bump_risk_pathwise(c, *plan, c.models.at(mid), c.products.at(pid), *num, values, risks);
}
