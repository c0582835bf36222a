// Multi-asset displaced model (mcMdlMultiDisplaced.h:28-717) with Baskets and Autocall
// (mcPrdMulti.h:181-439): plan lowering and launch.
//
// The model's initialisation (init, mcMdlMultiDisplaced.h:407-566) is small and runs on the
// host in FP64, recorded on a reverse-mode tape whose leaves are the model parameters in the
// order of the parameter labels.  Its outputs, the derived quantities of md_layout, become the
// device tables, and one reverse sweep of the tape per derived quantity gives the Jacobian
// d derived / d parameter.  The kernel (md_kernel.cu) sums the path adjoints of the derived
// quantities; the parameter risks are their Jacobian-weighted sums, the chain rule the
// reference's tape applies through init.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <stdexcept>
#include <vector>

#include "engine.h"
#include "host_math.h"

namespace cf {

size_t md_smem_bytes(int rng, int fp32, const McParams& p);
int md_scratch_fields(int rng, const McParams& p);
int md_occupancy(int rng, int fp32, int nA, size_t smem, int* occ);
int launch_md(int rng, int fp32, int grid, size_t smem, const McParams& p, void* stream);

namespace {

// ---------------------------------------------------------------------------------------
// Host tape: node k has up to two parents with their partial derivatives.
// ---------------------------------------------------------------------------------------
struct HostTape
{
    std::vector<int> pa, pb;
    std::vector<double> da, db;
    int push(int a, double dA, int b, double dB)
    {
        pa.push_back(a);
        da.push_back(dA);
        pb.push_back(b);
        db.push_back(dB);
        return int(pa.size()) - 1;
    }
    // adjoints of every node below `from` for a unit seed on node `from`
    void sweep(int from, std::vector<double>& adj) const
    {
        std::fill(adj.begin(), adj.begin() + from + 1, 0.0);
        adj[from] = 1.0;
        for (int k = from; k >= 0; --k)
        {
            const double a = adj[k];
            if (a == 0.0) continue;
            if (pa[k] >= 0) adj[pa[k]] += da[k] * a;
            if (pb[k] >= 0) adj[pb[k]] += db[k] * a;
        }
    }
};

HostTape* gTape = nullptr;  // the tape being recorded (plans are built under the context lock)

// A recorded value: node index, or -1 for a constant.
struct HV
{
    double v;
    int i;
    HV(double x = 0.0) : v(x), i(-1) {}
    HV(double x, int k) : v(x), i(k) {}
};
HV leafHV(double x) { return HV(x, gTape->push(-1, 0.0, -1, 0.0)); }
HV un(double v, const HV& a, double d) { return a.i < 0 ? HV(v) : HV(v, gTape->push(a.i, d, -1, 0.0)); }
HV bin(double v, const HV& a, double dA, const HV& b, double dB)
{
    if (a.i < 0 && b.i < 0) return HV(v);
    return HV(v, gTape->push(a.i, dA, b.i, dB));
}
HV operator+(const HV& a, const HV& b) { return bin(a.v + b.v, a, 1.0, b, 1.0); }
HV operator-(const HV& a, const HV& b) { return bin(a.v - b.v, a, 1.0, b, -1.0); }
HV operator*(const HV& a, const HV& b) { return bin(a.v * b.v, a, b.v, b, a.v); }
HV operator/(const HV& a, const HV& b) { return bin(a.v / b.v, a, 1.0 / b.v, b, -a.v / (b.v * b.v)); }
HV operator*(double c, const HV& a) { return un(c * a.v, a, c); }
HV operator-(double c, const HV& a) { return un(c - a.v, a, -1.0); }
HV operator-(const HV& a) { return un(-a.v, a, -1.0); }
HV hexp(const HV& a)
{
    const double e = std::exp(a.v);
    return un(e, a, e);
}
HV hsqrt(const HV& a)
{
    const double r = std::sqrt(a.v);
    return un(r, a, 0.5 / r);
}

}  // namespace

// ---------------------------------------------------------------------------------------
// Plan: simulation timeline = today + the product dates; tables of the derived quantities.
// ---------------------------------------------------------------------------------------
int Context::buildPlanMd(const ModelDesc& m, const ProductDesc& pd, Plan& plan)
{
    if (pd.kind != PROD_BASKETS && pd.kind != PROD_AUTOCALL)
        return fail(CF_E_UNSUPPORTED, "the multi-asset model prices Baskets and Autocall products");
    const int nA = int(m.assets.size()), nD = int(m.divDates.size());
    if (nA < 1 || nA > 16) return fail(CF_E_SHAPE, "the multi-asset kernel takes 1 to 16 assets");
    if (pd.timeline.empty() || pd.timeline.front() <= 0.0)
        return fail(CF_E_ARG, "multi-asset product dates must lie after today");
    plan.model = MODEL_MULTI;
    plan.prod = pd.kind;
    plan.nPay = int(pd.labels.size());
    plan.nParam = m.numParams();
    plan.nEv = int(pd.timeline.size());
    plan.nSteps = plan.nEv;  // every product date is a simulation step (mcMdlMultiDisplaced.h:378-384)
    plan.timeline = {0.0};
    plan.timeline.insert(plan.timeline.end(), pd.timeline.begin(), pd.timeline.end());
    const int nS = plan.nSteps, nEv = plan.nEv;
    McParams& P = plan.base;
    std::memset(&P, 0, sizeof(P));
    P.nEv = nEv;
    P.nPay = plan.nPay;
    P.nSteps = nS;
    P.nA = nA;
    P.prodKind = pd.kind;

    // --- init on the host tape (mcMdlMultiDisplaced.h:407-566, choldc.h:8-49) ---
    HostTape tape;
    gTape = &tape;
    std::vector<HV> par;
    auto mk = [&](double x) {
        par.push_back(leafHV(x));
        return par.back();
    };
    const HV disc = mk(m.disc);
    std::vector<HV> spot(nA), spread(nA), divs(size_t(nA) * nD), atm(nA), skew(nA), correl(size_t(nA) * nA);
    for (int a = 0; a < nA; ++a) spot[a] = mk(m.aSpots[a]);
    for (int a = 0; a < nA; ++a) spread[a] = mk(m.spreads[a]);
    for (int d = 0; d < nD; ++d)
        for (int a = 0; a < nA; ++a) divs[size_t(d) * nA + a] = mk(m.divs[size_t(d) * nA + a]);
    for (int a = 0; a < nA; ++a) atm[a] = mk(m.atms[a]);
    for (int a = 0; a < nA; ++a) skew[a] = mk(m.skews[a]);
    for (int i = 1; i < nA; ++i)
        for (int j = 0; j < i; ++j) correl[size_t(i) * nA + j] = mk(m.correl[size_t(i) * nA + j]);
    const HV lambda = mk(m.lambda);

    const MdLayout L = md_layout(nA, nS, nEv);
    std::vector<HV> der(L.total);
    std::vector<int> dyn(nA);
    std::vector<HV> repo(nA), beta(nA), alpha(nA);
    for (int a = 0; a < nA; ++a) repo[a] = disc - spread[a];
    for (int a = 0; a < nA; ++a)
    {
        // displacement from ATM and skew (mcMdlMultiDisplaced.h:418-444)
        beta[a] = atm[a] + 2.0 * skew[a];
        if (std::fabs(skew[a].v) < 1.0e-05)
        {
            dyn[a] = MD_LOGNORMAL;
            alpha[a] = HV(0.0);
        }
        else if (std::fabs(beta[a].v) < 1.0e-05)
        {
            dyn[a] = MD_NORMAL;
            alpha[a] = -2.0 * spot[a] * skew[a];
            beta[a] = HV(0.0);
        }
        else if (beta[a].v > 0)
        {
            dyn[a] = MD_SURNORMAL;
            alpha[a] = (-2.0 * spot[a]) / beta[a] * skew[a];
        }
        else
        {
            dyn[a] = MD_SUBNORMAL;
            beta[a] = -1.0 * beta[a];
            alpha[a] = (-2.0 * spot[a]) / beta[a] * skew[a];
        }
    }
    // unit-diagonal symmetric correl from its lower triangle, lambda shift, Cholesky factor
    std::vector<HV> used(size_t(nA) * nA), chol(size_t(nA) * nA, HV(0.0));
    for (int i = 0; i < nA; ++i)
        for (int j = 0; j < nA; ++j)
        {
            const HV raw = i == j ? HV(1.0) : i > j ? correl[size_t(i) * nA + j] : correl[size_t(j) * nA + i];
            used[size_t(i) * nA + j] = lambda * (1.0 - raw) + raw;
        }
    for (int i = 0; i < nA; ++i)
        for (int j = 0; j <= i; ++j)
        {
            HV sum = used[size_t(i) * nA + j];
            for (int k = 0; k < j; ++k) sum = sum - chol[size_t(i) * nA + k] * chol[size_t(j) * nA + k];
            if (i == j)
            {
                if (sum.v < -1.0e-15)
                {
                    gTape = nullptr;
                    return fail(CF_E_ARG, "choldc : matrix not positive definite");
                }
                if (sum.v < 1.0e-15) sum = HV(0.0);
                chol[size_t(i) * nA + i] = hsqrt(sum);
            }
            else
                chol[size_t(i) * nA + j] =
                    std::fabs(chol[size_t(j) * nA + j].v) < 1.0e-15 ? HV(0.0) : sum / chol[size_t(j) * nA + j];
        }
    for (int a = 0; a < nA; ++a) der[L.s0 + a] = spot[a];
    for (int k = 0; k < nA * nA; ++k) der[L.chol + k] = chol[k];
    // per step: dividend-adjusted forward factors (mcMdlMultiDisplaced.h:343-364), stds and drifts
    for (int i = 0; i < nS; ++i)
    {
        const double t1 = plan.timeline[i], t2 = plan.timeline[i + 1], dt = t2 - t1;
        for (int a = 0; a < nA; ++a)
        {
            HV divProd(1.0);
            int d = int(std::lower_bound(m.divDates.begin(), m.divDates.end(), t1) - m.divDates.begin());
            while (d < nD && m.divDates[d] < t2)
            {
                divProd = divProd * (1.0 - divs[size_t(d) * nA + a]);
                ++d;
            }
            der[L.ff + i * nA + a] = divProd * hexp(repo[a] * HV(dt));
            HV sd, dr;
            switch (dyn[a])
            {
            case MD_LOGNORMAL: sd = beta[a] * HV(std::sqrt(dt)); dr = -0.5 * sd * sd; break;
            case MD_NORMAL: sd = alpha[a] * HV(std::sqrt(dt)); dr = HV(0.0); break;
            case MD_SURNORMAL: sd = beta[a] * HV(std::sqrt(dt)); dr = -0.5 * beta[a] * beta[a] * HV(dt); break;
            default: sd = -beta[a] * HV(std::sqrt(dt)); dr = -0.5 * beta[a] * beta[a] * HV(dt); break;
            }
            der[L.std_ + i * nA + a] = sd;
            der[L.drift + i * nA + a] = dr;
        }
    }
    for (int a = 0; a < nA; ++a) der[L.alpha + a] = alpha[a];
    // numeraires exp(r t) of the product dates; the samples' forward factors exp(repo * 0) = 1
    for (int e = 0; e < nEv; ++e) der[L.num + e] = hexp(disc * HV(pd.timeline[e]));
    gTape = nullptr;

    // Jacobian [derived][parameter]: one reverse sweep per recorded derived quantity
    plan.mdTotal = L.total;
    plan.mdDerived.resize(L.total);
    plan.mdJac.assign(size_t(L.total) * plan.nParam, 0.0);
    std::vector<double> adj(tape.pa.size());
    for (int d = 0; d < L.total; ++d)
    {
        plan.mdDerived[d] = der[d].v;
        if (der[d].i < 0) continue;
        tape.sweep(der[d].i, adj);
        for (int j = 0; j < plan.nParam; ++j)
            if (par[j].i <= der[d].i) plan.mdJac[size_t(d) * plan.nParam + j] = adj[par[j].i];
    }

    // --- device tables ---
    std::vector<unsigned char> buf;
    auto put = [&](const void* src, size_t n) {
        const size_t off = (buf.size() + 255) & ~size_t(255);
        buf.resize(off + ((n + 15) & ~size_t(15)), 0);
        if (n) std::memcpy(buf.data() + off, src, n);
        return off;
    };
    std::vector<float> derF(plan.mdDerived.begin(), plan.mdDerived.end());
    const std::vector<double>& asset = pd.kind == PROD_BASKETS ? pd.weights : pd.refs;
    std::vector<float> assetF(asset.begin(), asset.end());
    std::vector<double> ks = pd.kind == PROD_BASKETS ? pd.strikes : std::vector<double>{0.0};
    std::vector<float> ksF(ks.begin(), ks.end());
    std::vector<int> evAtStep(nS + 1, -1);
    for (int i = 1; i <= nS; ++i) evAtStep[i] = i - 1;
    const size_t oD = put(plan.mdDerived.data(), plan.mdDerived.size() * 8), oF = put(derF.data(), derF.size() * 4);
    const size_t oAs = put(asset.data(), asset.size() * 8), oAsF = put(assetF.data(), assetF.size() * 4);
    const size_t oK = put(ks.data(), ks.size() * 8), oKF = put(ksF.data(), ksF.size() * 4);
    const size_t oDyn = put(dyn.data(), dyn.size() * 4), oEv = put(evAtStep.data(), evAtStep.size() * 4);
    const int dim = nS * nA;
    plan.sobolOk = dim <= sobol_max_dim();
    size_t oDir = 0;
    if (plan.sobolOk)
    {
        const std::vector<unsigned> dirs = sobol_dirs(dim);
        oDir = put(dirs.data(), dirs.size() * 4);
    }
    int rc = plan.tables.ensure(buf.size());
    if (rc) return rc;
    CF_CUDA(cudaMemcpyAsync(plan.tables.ptr, buf.data(), buf.size(), cudaMemcpyHostToDevice, stream));
    // the pageable source must outlive the copy
    CF_CUDA(cudaStreamSynchronize(stream));
    h2d += buf.size();
    const unsigned char* dv = static_cast<const unsigned char*>(plan.tables.ptr);
    P.mdD = reinterpret_cast<const double*>(dv + oD);
    P.mdF = reinterpret_cast<const float*>(dv + oF);
    P.mdAssetD = reinterpret_cast<const double*>(dv + oAs);
    P.mdAssetF = reinterpret_cast<const float*>(dv + oAsF);
    P.kD = reinterpret_cast<const double*>(dv + oK);
    P.kF = reinterpret_cast<const float*>(dv + oKF);
    P.mdDyn = reinterpret_cast<const int*>(dv + oDyn);
    P.evAtStep = reinterpret_cast<const int*>(dv + oEv);
    P.sobolDir = plan.sobolOk ? reinterpret_cast<const unsigned*>(dv + oDir) : nullptr;
    P.acKo = pd.ko;
    P.acStrike = pd.strike;
    P.acCpn = pd.cpn;
    P.acDt = pd.kind == PROD_AUTOCALL ? pd.maturity / pd.periods : 0.0;
    P.acSmooth = std::max(pd.smooth, 1.0e-08);  // mcPrdMulti.h:297 (EPS, utility.h:9)
    plan.evAtStep = evAtStep;
    return CF_OK;
}

// ---------------------------------------------------------------------------------------
// Launch: value (risk = false) or the adjoint of sum_k weights[k] payoff_k.
// ---------------------------------------------------------------------------------------
int Context::enqueueMd(Slot& slot, Plan& plan, const cf_num_param& num, bool risk, const double* weights,
                       long long firstPath)
{
    const bool sobol = num.useSobol != 0, fp32 = num.precision == CF_FP32;
    const int rng = sobol ? RNG_SOBOL : RNG_MRG;
    McParams p = plan.base;
    if (sobol && !plan.sobolOk)
        return fail(CF_E_SHAPE, "Sobol dimension " + std::to_string(p.nSteps * p.nA) + " exceeds the " +
                                    std::to_string(sobol_max_dim()) + " dimensions of the direction numbers");
    cudaStream_t st = slot.stream;
    p.nPath = num.numPath;
    p.firstPath = firstPath;
    p.seed1 = unsigned(num.seed1);
    p.seed2 = unsigned(num.seed2);
    p.mrgJumpA = jumpA;
    p.mrgJumpB = jumpB;
    p.nRisk = risk ? plan.mdTotal : 0;
    p.nAcc = p.nRisk + 2 * plan.nPay + 2;
    const size_t wBytes = ((size_t(plan.nPay) * 12 + 255) & ~size_t(255));
    const size_t accBytes = size_t(p.nAcc) * 16;
    int rc = slot.work.ensure(wBytes + accBytes + 256, st);
    if (rc) return rc;
    if ((rc = slot.hostAcc.ensure(accBytes + 16))) return rc;
    if ((rc = slot.hostW.ensure(size_t(plan.nPay) * 12 + 16))) return rc;
    double* wd = static_cast<double*>(slot.hostW.ptr);
    float* wf = reinterpret_cast<float*>(wd + plan.nPay);
    for (int k = 0; k < plan.nPay; ++k)
    {
        wd[k] = weights ? weights[k] : 0.0;
        wf[k] = float(wd[k]);
    }
    char* wbase = static_cast<char*>(slot.work.ptr);
    CF_CUDA(cudaMemcpyAsync(wbase, wd, size_t(plan.nPay) * 12, cudaMemcpyHostToDevice, st));
    h2d += size_t(plan.nPay) * 12;
    p.w = reinterpret_cast<const double*>(wbase);
    p.wf = reinterpret_cast<const float*>(wbase + size_t(plan.nPay) * 8);
    p.acc = reinterpret_cast<long long*>(wbase + wBytes);
    p.err = reinterpret_cast<int*>(wbase + wBytes + accBytes);
    p.claim = reinterpret_cast<unsigned long long*>(wbase + wBytes + accBytes + 8);  // zeroed with the flag
    CF_CUDA(cudaMemsetAsync(p.acc, 0, accBytes + 16, st));

    const size_t smem = md_smem_bytes(rng, fp32, p);
    int occ = 0;
    rc = md_occupancy(rng, fp32, p.nA, smem, &occ);
    if (rc) return cuda_fail(cudaError_t(rc), "multi-asset kernel occupancy");
    if (occ < 1) return fail(CF_E_SHAPE, "multi-asset kernel does not fit on an SM");
    const long long threadsNeeded = sobol ? (p.nPath / 32 + 1) * 32 : (p.nPath + 1) / 2;
    long long grid = std::max(1LL, std::min<long long>((threadsNeeded + 127) / 128, (long long)numSMs * occ));
    if (risk)
    {
        const size_t fields = size_t(md_scratch_fields(rng, p));
        if ((rc = slot.scratch.ensure(fields * size_t(grid) * 128 * (fp32 ? 4 : 8), st))) return rc;
        p.scratch = slot.scratch.ptr;
    }
    rc = launch_md(rng, fp32, int(grid), smem, p, st);
    if (rc) return cuda_fail(cudaError_t(rc), "multi-asset kernel launch");
    CF_CUDA(cudaMemcpyAsync(slot.hostAcc.ptr, p.acc, accBytes + 16, cudaMemcpyDeviceToHost, st));
    d2h += accBytes + 16;
    if (!slot.done) CF_CUDA(cudaEventCreateWithFlags(&slot.done, cudaEventDisableTiming));
    CF_CUDA(cudaEventRecord(slot.done, st));
    slot.last = p;
    slot.plan = &plan;
    slot.planRef = plan.weak_from_this().lock();
    slot.risk = risk;
    slot.multi = false;
    slot.launches = 1;
    return CF_OK;
}

}  // namespace cf
