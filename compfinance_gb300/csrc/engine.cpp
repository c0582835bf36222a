// Host engine behind the C ABI (include/cfgpu.h): the model / product store, the lowering
// of a (model, product) pair into flat device tables, and the launch of the Monte Carlo
// kernels.  Reference interfaces mirrored: store.h (registry), mcBase.h Model/Product
// (allocate/init/timeline/defline/payoffLabels/parameterLabels), main.h entry points.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/cfgpu.h"
#include "cf_params.h"
#include "engine.h"
#include "host_math.h"

namespace cf {

int launch_sobol_points(const unsigned* dir, int dim, long long first, int n, unsigned* out, void* stream);
int launch_mrg_state(const unsigned* A, const unsigned* B, unsigned s1, unsigned s2,
                     unsigned long long skip, unsigned* out, void* stream);
int launch_gauss(int sobol, int uniform, const unsigned* dir, const unsigned* A, const unsigned* B,
                 unsigned s1, unsigned s2, int dim, long long first, int n, double* out, void* stream);

thread_local std::string g_lastError;

int fail(int code, const std::string& msg)
{
    g_lastError = msg;
    return code;
}

int cuda_fail(cudaError_t e, const char* what)
{
    return fail(e == cudaErrorMemoryAllocation ? CF_E_NOMEM : CF_E_CUDA,
                std::string(what) + ": " + cudaGetErrorString(e));
}


// ------------------------------------------------------------------------------------
// Device buffers
// ------------------------------------------------------------------------------------
std::atomic<unsigned long long> DevBuf::growths{0};

int DevBuf::ensure(size_t n, cudaStream_t stream)
{
    if (n <= bytes) return CF_OK;
    ++growths;
    const size_t want = n + n / 4;
    cudaError_t e;
    if (stream)
    {
        // the old buffer is freed after the stream's earlier work, the new one is ready for its later work
        if (ptr) cudaFreeAsync(ptr, stream);
        ptr = nullptr;
        bytes = 0;
        e = cudaMallocAsync(&ptr, want, stream);
    }
    else
    {
        release();
        e = cudaMalloc(&ptr, want);
    }
    if (e != cudaSuccess)
    {
        ptr = nullptr;
        bytes = 0;
        return cuda_fail(e, "cudaMalloc");
    }
    bytes = want;
    return CF_OK;
}

void DevBuf::release()
{
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
}

int PinnedBuf::ensure(size_t n)
{
    if (n <= bytes) return CF_OK;
    release();
    // at least 16 MB (the finished risks of a 200-payoff portfolio on a 120x60 grid are 11.5 MB):
    // freeing pinned memory waits for the device, so a serving slot should not regrow it
    const size_t want = std::max(n + n / 4, size_t(16) << 20);
    cudaError_t e = cudaMallocHost(&ptr, want);
    if (e != cudaSuccess)
    {
        ptr = nullptr;
        bytes = 0;
        return cuda_fail(e, "cudaMallocHost");
    }
    bytes = want;
    return CF_OK;
}

void PinnedBuf::release()
{
    if (ptr) cudaFreeHost(ptr);
    ptr = nullptr;
    bytes = 0;
}

Slot::~Slot()
{
    if (done) cudaEventDestroy(done);
    if (ownsStream && stream) cudaStreamDestroy(stream);
}

// ------------------------------------------------------------------------------------
// Products: timelines, deflines and labels (mcPrd.h:43-80, 149-211, 305-340).
// ------------------------------------------------------------------------------------
void ProductDesc::build()
{
    timeline.clear();
    fwdMat.clear();
    discMat.clear();
    needNum.clear();
    labels.clear();
    kflat.clear();
    payOff.clear();
    libEnd.clear();
    if (kind == PROD_CONTINGENT)
    {
        // mcPrd.h:426-480: today, every payFreq while more than a day remains, maturity
        constexpr double kOneDay = 0.003773585;  // mcPrd.h:27
        timeline.push_back(0.0);
        double t = freq;
        while (maturity - t > kOneDay)
        {
            timeline.push_back(t);
            t += freq;
        }
        timeline.push_back(maturity);
        const size_t n = timeline.size();
        for (size_t i = 0; i < n; ++i)
        {
            fwdMat.push_back(timeline[i]);
            discMat.push_back(NAN);
            needNum.push_back(i > 0 ? 1 : 0);
            libEnd.push_back(i + 1 < n ? timeline[i + 1] : NAN);
        }
        labels = {"contingent bond " + fmt2(maturity) + " " + fmt2(coupon)};
    }
    else if (kind == PROD_EUROPEAN)
    {
        timeline = {exercise};
        fwdMat = {settlement};
        discMat = {settlement};
        needNum = {1};
        labels = {settlement == exercise ? "call " + fmt2(strike) + " " + fmt2(exercise)
                                         : "call " + fmt2(strike) + " " + fmt2(exercise) + " " + fmt2(settlement)};
    }
    else if (kind == PROD_UOC)
    {
        timeline.push_back(0.0);
        double t = freq;
        while (maturity - t > kOneHour)
        {
            timeline.push_back(t);
            t += freq;
        }
        timeline.push_back(maturity);
        for (double x : timeline)
        {
            fwdMat.push_back(x);
            discMat.push_back(NAN);
            needNum.push_back(0);
        }
        needNum.back() = 1;
        const std::string l1 = std::string(callPut ? "put " : "call ") + fmt2(maturity) + " " + fmt2(strike);
        labels = {l1 + " up and out " + fmt2(barrier) + " monitoring freq " + fmt2(freq) + " smooth " + fmt2(smooth),
                  l1};
    }
    else if (kind == PROD_BASKETS)
    {
        // mcPrdMulti.h:201-221: the maturity, numeraire and spot(T) of every asset
        timeline = {maturity};
        fwdMat = {maturity};
        discMat = {NAN};
        needNum = {1};
        for (double k : strikes) labels.push_back("basket strike " + fmt2(k));
        kflat = strikes;
    }
    else if (kind == PROD_AUTOCALL)
    {
        // mcPrdMulti.h:297-324: periods equally spaced dates (accumulated as the reference does)
        double t = 0.0;
        const double dt = maturity / periods;
        for (int k = 0; k < periods; ++k)
        {
            t += dt;
            timeline.push_back(t);
            fwdMat.push_back(t);
            discMat.push_back(NAN);
            needNum.push_back(1);
        }
        constexpr double kEps = 1.0e-08;  // utility.h:9
        labels = {"autocall strike " + std::to_string(int(100 * strike + kEps)) + " KO " +
                  std::to_string(int(100 * ko + kEps)) + " CPN " + std::to_string(int(100 * cpn + kEps)) + " " +
                  std::to_string(periods) + " periods of " + std::to_string(int(12 * maturity / periods + kEps)) +
                  "m"};
    }
    else
    {
        std::map<double, std::vector<double>> opts;
        for (size_t i = 0; i < mats.size(); ++i) opts[mats[i]].push_back(strikes[i]);
        for (auto& kv : opts)
        {
            timeline.push_back(kv.first);
            fwdMat.push_back(kv.first);
            discMat.push_back(NAN);
            needNum.push_back(1);
            payOff.push_back(int(kflat.size()));
            for (double k : kv.second)
            {
                kflat.push_back(k);
                labels.push_back("call " + fmt2(kv.first) + " " + fmt2(k));
            }
        }
        payOff.push_back(int(kflat.size()));
    }
}

void ModelDesc::build()
{
    labels_.clear();
    labelsReady_ = false;
}

const std::vector<std::string>& ModelDesc::labels() const
{
    if (labelsReady_) return labels_;
    labelsReady_ = true;
    std::vector<std::string>& labels = labels_;
    labels.clear();
    if (kind == MODEL_MULTI)
    {
        // mcMdlMultiDisplaced.h:146-209
        const size_t n = assets.size();
        labels.push_back("disc rate");
        for (size_t a = 0; a < n; ++a) labels.push_back("spot " + assets[a]);
        for (size_t a = 0; a < n; ++a) labels.push_back("repo spread " + assets[a]);
        for (double d : divDates)
            for (size_t a = 0; a < n; ++a) labels.push_back("div " + assets[a] + " " + fmt2(d));
        for (size_t a = 0; a < n; ++a) labels.push_back("ATM " + assets[a]);
        for (size_t a = 0; a < n; ++a) labels.push_back("skew " + assets[a]);
        for (size_t i = 1; i < n; ++i)
            for (size_t j = 0; j < i; ++j) labels.push_back("correl " + assets[i] + " " + assets[j]);
        labels.push_back("lambda");
        return labels_;
    }
    labels.push_back("spot");
    if (kind == MODEL_BS)
    {
        labels.push_back("vol");
        labels.push_back("rate");
        labels.push_back("div");
    }
    else
    {
        std::vector<std::string> ft(times.size());
        for (size_t j = 0; j < times.size(); ++j) ft[j] = " " + fmt2(times[j]);
        labels.reserve(1 + spots.size() * times.size());
        for (size_t i = 0; i < spots.size(); ++i)
        {
            const std::string fs = "lvol " + fmt2(spots[i]);
            for (size_t j = 0; j < times.size(); ++j) labels.push_back(fs + ft[j]);
        }
    }
    return labels_;
}

int ModelDesc::numParams() const
{
    if (kind == MODEL_MULTI)
    {
        const int n = int(assets.size());
        return 1 + 2 * n + n * int(divDates.size()) + 2 * n + n * (n - 1) / 2 + 1;
    }
    return kind == MODEL_BS ? 4 : 1 + int(spots.size() * times.size());
}

double& ModelDesc::param(int i)
{
    if (kind != MODEL_MULTI)
    {
        if (i == 0) return spot;
        if (kind == MODEL_BS) return i == 1 ? vol : i == 2 ? rate : div;
        return vols[size_t(i - 1)];  // spot-major, the order of the parameter labels
    }
    const int n = int(assets.size()), nD = int(divDates.size());
    if (i == 0) return disc;
    --i;
    if (i < n) return aSpots[i];
    i -= n;
    if (i < n) return spreads[i];
    i -= n;
    if (i < n * nD) return divs[size_t(i)];
    i -= n * nD;
    if (i < n) return atms[i];
    i -= n;
    if (i < n) return skews[i];
    i -= n;
    for (int r = 1; r < n; ++r)
        for (int c = 0; c < r; ++c)
            if (i-- == 0) return correl[size_t(r) * n + c];
    return lambda;
}

namespace {
const std::vector<std::string> kDefaultAsset = {"spot"};  // mcBase.h:125, 160
}

const std::vector<std::string>& ModelDesc::assetNames() const
{
    return kind == MODEL_MULTI ? assets : kDefaultAsset;
}

const std::vector<std::string>& ProductDesc::assetNames() const
{
    return kind == PROD_BASKETS || kind == PROD_AUTOCALL ? assets : kDefaultAsset;
}

// ------------------------------------------------------------------------------------
// Plan: the flat device tables of one (model, product) pair.
// ------------------------------------------------------------------------------------
namespace {

struct Packer
{
    std::vector<unsigned char> buf;
    size_t put(const void* p, size_t n)
    {
        const size_t off = (buf.size() + 255) & ~size_t(255);
        buf.resize(off + ((n + 15) & ~size_t(15)), 0);
        if (n) std::memcpy(buf.data() + off, p, n);
        return off;
    }
    template <class T>
    size_t vec(const std::vector<T>& v) { return put(v.data(), v.size() * sizeof(T)); }
};

template <class T>
std::vector<float> to_f(const std::vector<T>& v)
{
    return std::vector<float>(v.begin(), v.end());
}

}  // namespace

int Context::buildPlan(const ModelDesc& m, const ProductDesc& pd, Plan& plan)
{
    // plan arrives freshly constructed (getPlan makes a new one per build)
    if (m.assetNames() != pd.assetNames()) return fail(CF_E_ARG, "Model and product are not compatible");  // mcBase.h:253-259
    if (m.kind == MODEL_MULTI) return buildPlanMd(m, pd, plan);
    if (pd.kind == PROD_BASKETS || pd.kind == PROD_AUTOCALL)
        return fail(CF_E_UNSUPPORTED, "Baskets and Autocall products run on the multi-asset model");
    plan.model = m.kind;
    plan.prod = pd.kind;
    plan.nPay = int(pd.labels.size());
    plan.nParam = m.numParams();
    plan.nEv = int(pd.timeline.size());
    McParams& P = plan.base;
    std::memset(&P, 0, sizeof(P));
    P.nEv = plan.nEv;
    P.nPay = plan.nPay;
    P.spot = m.spot;
    P.vol = m.vol;
    P.spotMeasure = m.qSpot ? 1 : 0;
    P.callPut = pd.callPut;
    P.strike = pd.strike;

    Packer pk;
    std::vector<double> tl;
    std::vector<int> evAtStep;
    std::vector<double> ev(10 * size_t(plan.nEv), 0.0);
    double frontSpot = m.spot;
    size_t oBs = 0, oX = 0, oInv = 0, oY = 0, oXf = 0, oInvf = 0, oYf = 0, oCA = 0, oCB = 0, oCAf = 0, oCBf = 0,
           oColA = 0, oColB = 0, oBsF = 0, oBucket = 0, oWA = 0, oWB = 0, oXs = 0, oIr = 0, oTd = 0, oBf = 0, oVols = 0, oSq = 0, oTw = 0, oSc = 0;

    if (m.kind == MODEL_BS)
    {
        // mcMdlBS.h:149-277: timeline = today + product dates after today.
        tl.push_back(0.0);
        for (double t : pd.timeline)
            if (t > 0.0) tl.push_back(t);
        const bool todayOn = pd.timeline[0] == 0.0;
        const int n = int(tl.size()) - 1;
        evAtStep.assign(n + 1, -1);
        if (todayOn) evAtStep[0] = 0;
        for (int i = 1; i <= n; ++i) evAtStep[i] = todayOn ? i : i - 1;
        const double mu = m.rate - m.div;
        std::vector<double> bsd(5 * size_t(n));
        for (int i = 0; i < n; ++i)
        {
            const double dt = tl[i + 1] - tl[i];
            bsd[i] = m.qSpot ? (mu + 0.5 * m.vol * m.vol) * dt : (mu - 0.5 * m.vol * m.vol) * dt;
            bsd[n + i] = m.vol * std::sqrt(dt);
            bsd[2 * n + i] = dt;
            bsd[3 * n + i] = std::sqrt(dt);
            bsd[4 * n + i] = (m.qSpot ? m.vol : -m.vol) * dt;
        }
        for (int e = 0; e < plan.nEv; ++e)
        {
            const double t = pd.timeline[e];
            ev[e] = std::exp(mu * (pd.fwdMat[e] - t));
            ev[plan.nEv + e] = pd.fwdMat[e] - t;
            const bool hasD = !std::isnan(pd.discMat[e]);
            ev[2 * plan.nEv + e] = hasD ? std::exp(-m.rate * (pd.discMat[e] - t)) : 1.0;
            ev[3 * plan.nEv + e] = hasD ? pd.discMat[e] - t : 0.0;
            ev[4 * plan.nEv + e] = m.qSpot ? std::exp(m.div * t) / m.spot : std::exp(m.rate * t);
            ev[5 * plan.nEv + e] = t;
            ev[6 * plan.nEv + e] = pd.needNum[e] ? 1.0 : 0.0;
            if (!pd.libEnd.empty() && !std::isnan(pd.libEnd[e]))  // mcMdlBS.h:266-272
            {
                const double dt = pd.libEnd[e] - t;
                ev[7 * plan.nEv + e] = (std::exp(m.rate * dt) - 1.0) / dt;
                ev[8 * plan.nEv + e] = std::exp(m.rate * dt);
            }
        }
        frontSpot = m.spot * ev[0];  // path.front() forward of the first product date
        oBs = pk.vec(bsd);
        oBsF = pk.vec(to_f(bsd));
        plan.nSteps = n;
    }
    else
    {
        // mcMdlDupire.h:165-217: refined timeline, event flags, vols pre-interpolated in time.
        tl = fill_data(pd.timeline, m.maxDt, kHalfDay, {0.0});
        const int n = int(tl.size()) - 1;
        if (n < 1) return fail(CF_E_SHAPE, "Dupire: empty simulation timeline");
        evAtStep.assign(n + 1, -1);
        int e = 0;
        for (int i = 0; i <= n; ++i)
            if (std::binary_search(pd.timeline.begin(), pd.timeline.end(), tl[i])) evAtStep[i] = e++;
        if (e != plan.nEv) return fail(CF_E_SHAPE, "Dupire: product dates before today are not supported");
        const int nS = int(m.spots.size()), nT = int(m.times.size());
        std::vector<double> X(nS), inv(nS, 0.0), Y(size_t(n) * nS), cAv(n), cBv(n), sqv(n), twv(n, 0.0);
        std::vector<int> colA(n), colB(n);
        for (int j = 0; j < nS; ++j) X[j] = std::log(m.spots[j]);
        for (int j = 0; j + 1 < nS; ++j) inv[j] = 1.0 / (X[j + 1] - X[j]);
        std::vector<double> row(nT);
        for (int i = 0; i < n; ++i)
        {
            const double sq = std::sqrt(tl[i + 1] - tl[i]);
            sqv[i] = sq;
            // interp_lin of every spot's vols at tl[i], with the time bracket found once per step
            const double* it = std::upper_bound(m.times.data(), m.times.data() + nT, tl[i]);
            if (it == m.times.data() + nT || it == m.times.data())
            {
                const size_t c = it == m.times.data() ? 0 : size_t(nT) - 1;
                for (int j = 0; j < nS; ++j) Y[size_t(i) * nS + j] = sq * m.vols[size_t(j) * nT + c];
            }
            else
            {
                const size_t k = size_t(it - m.times.data()) - 1;
                const double tw = (tl[i] - m.times[k]) / (m.times[k + 1] - m.times[k]);
                for (int j = 0; j < nS; ++j)
                {
                    const double* y = &m.vols[size_t(j) * nT];
                    Y[size_t(i) * nS + j] = sq * (y[k] + (y[k + 1] - y[k]) * tw);
                }
            }
            if (it == m.times.data() + nT || it == m.times.data())
            {
                colA[i] = colB[i] = it == m.times.data() ? 0 : nT - 1;
                cAv[i] = sq;
                cBv[i] = 0.0;
            }
            else
            {
                const int k = int(it - m.times.data()) - 1;
                const double t = (tl[i] - m.times[k]) / (m.times[k + 1] - m.times[k]);
                twv[i] = t;
                colA[i] = k;
                colB[i] = k + 1;
                cAv[i] = sq * (1.0 - t);
                cBv[i] = sq * t;
            }
        }
        const double x0 = std::log(m.spot);
        std::vector<float> Xf(nS);
        for (int j = 0; j < nS; ++j) Xf[j] = float(X[j] - x0);
        P.x0d = x0;
        P.s0f = float(std::exp(x0));
        frontSpot = std::exp(x0);  // path.front() spot when today is a product date
        P.nS = nS;
        P.nT = nT;
        // bucket index of the grid (a search hint; the kernel corrects it exactly)
        const int nB = 512;
        std::vector<int> bucket(nB, 0);
        const double w = nS > 1 ? (X[nS - 1] - X[0]) / nB : 1.0;
        for (int b = 0; b < nB; ++b)
            bucket[b] = int(std::upper_bound(X.begin(), X.end(), X[0] + b * w) - X.begin());
        P.nBuckets = nB;
        P.bX0d = X[0];
        P.bInvWd = 1.0 / w;
        P.bX0f = Xf[0];
        P.bInvWf = float(1.0 / w);
        oBucket = pk.vec(bucket);
        oX = pk.vec(X);
        oInv = pk.vec(inv);
        oY = pk.vec(Y);
        oXf = pk.vec(Xf);
        oInvf = pk.vec(to_f(inv));
        oYf = pk.vec(to_f(Y));
        oColA = pk.vec(colA);
        oColB = pk.vec(colB);
        oCA = pk.vec(cAv);
        oCB = pk.vec(cBv);
        oCAf = pk.vec(to_f(cAv));
        oCBf = pk.vec(to_f(cBv));
        // FP32 risk: integer time weights of the row-to-node gather, and the node slab's
        // flush interval: a slab word receives at most 4 warps x (steps touching its time
        // column) products below 2^50 per unit, and must stay below 2^63.
        std::vector<int> wA(n), wB(n), touch(nT, 0);
        for (int i = 0; i < n; ++i)
        {
            wA[i] = int(std::llround(std::ldexp(cAv[i], WEIGHT_SHIFT)));
            wB[i] = int(std::llround(std::ldexp(cBv[i], WEIGHT_SHIFT)));
            ++touch[colA[i]];
            if (colB[i] != colA[i]) ++touch[colB[i]];
        }
        const int sMax = *std::max_element(touch.begin(), touch.end());
        P.nodeFlushUnits = std::max(1, std::min(4, 2048 / std::max(1, sMax)));
        P.nodeDirect = sMax >= 2048 ? 1 : 0;
        oWA = pk.vec(wA);
        oWB = pk.vec(wB);
        oVols = pk.vec(m.vols);
        oSq = pk.vec(sqv);
        oTw = pk.vec(twv);
        // FP32 risk kernel (dupire_risk32): knots with sentinels, (xr, ir) per interval,
        // (y, d) per step and interval, and buckets narrower than 2/3 of the smallest knot
        // spacing.  Products whose dates are not monitoring dates plus a final maturity, grids
        // with more than 510 spots or with knots too close for 4096 buckets use the generic kernel.
        {
            std::vector<float> xs(size_t(nS) + 2), irv(2 * size_t(nS + 1), 0.0f), tdv(2 * size_t(n) * (nS + 1));
            xs[0] = -INFINITY;
            xs[nS + 1] = INFINITY;
            for (int j = 0; j < nS; ++j) xs[j + 1] = Xf[j];
            for (int lo = 1; lo < nS; ++lo)
            {
                irv[2 * lo] = Xf[lo - 1];
                irv[2 * lo + 1] = float(inv[lo - 1]);
            }
            for (int i = 0; i < n; ++i)
            {
                const double* y = &Y[size_t(i) * nS];
                float* o = &tdv[2 * size_t(i) * (nS + 1)];
                // (y - 2 d, d): the kernels evaluate y + d t as (y - 2 d) + d (t + 2) straight from
                // the quantised float t + 2
                o[0] = float(y[0]);
                for (int lo = 1; lo < nS; ++lo)
                {
                    const double d = y[lo] - y[lo - 1];
                    o[2 * lo] = float(y[lo - 1] - 2.0 * d);
                    o[2 * lo + 1] = float(d);
                }
                o[2 * nS] = float(y[nS - 1]);
            }
            const BucketGrid bg = bucket_grid(Xf);
            const std::vector<int>& bf = bg.first;
            bool evOk = evAtStep[n] == plan.nEv - 1;
            if (pd.kind == PROD_EUROPEAN)
                for (int i = 0; i < n; ++i) evOk = evOk && evAtStep[i] < 0;
            // node slab unit: a word receives per unit round at most 256 paths x (steps touching
            // its time column) contributions, each below 512 x (largest time weight) in value
            double wMax = 0.0;
            for (int i = 0; i < n; ++i) wMax = std::max(wMax, std::max(cAv[i], cBv[i]));
            const double perWord = 256.0 * sMax * 512.0 * std::max(wMax, 1e-300);
            const int shift = int(std::floor(std::log2(1073741824.0 / perWord)));  // one bit of margin
            P.nodeShiftF = std::min(FIX_HI_SHIFT, shift);
            // the reverse sweep's per-step node columns and weights (float, scaled by 2^nodeShiftF,
            // exact: a power of two)
            std::vector<int> scv(4 * size_t(n));
            for (int i = 0; i < n; ++i)
            {
                const float wa = std::ldexp(float(cAv[i]), P.nodeShiftF), wb = std::ldexp(float(cBv[i]), P.nodeShiftF);
                scv[4 * size_t(i)] = colA[i];
                scv[4 * size_t(i) + 1] = colB[i];
                std::memcpy(&scv[4 * size_t(i) + 2], &wa, 4);
                std::memcpy(&scv[4 * size_t(i) + 3], &wb, 4);
            }
            oSc = pk.vec(scv);
            P.fast32 = (pd.kind == PROD_UOC || pd.kind == PROD_EUROPEAN) && evOk && nS <= 510 && bg.ok &&
                       bg.oneCompare && shift >= 4;
            // FP32 AADriskMulti (multi_risk32.cu) uses the same tables and slab unit: its chunks
            // hold 256 paths of one bucket
            plan.multi32 = pd.kind == PROD_EUROPEANS && nS <= 510 && bg.ok && shift >= 4;
            P.nBucketsF = int(bf.size());
            P.bX0F = bg.x0;
            P.bInvWF = bg.invW;
            oXs = pk.vec(xs);
            oIr = pk.vec(irv);
            oTd = pk.vec(tdv);
            oBf = pk.vec(bf);
        }
        plan.nSteps = n;
        plan.yBytesD = Y.size() * 8;
        plan.yBytesF = Y.size() * 4;
    }
    P.nSteps = plan.nSteps;
    plan.timeline = tl;

    // product constants (mcPrd.h:235-288: smoothing from the first sample's spot)
    if (pd.kind == PROD_UOC)
    {
        const double smooth = frontSpot * pd.smooth;
        P.twoSmooth = 2 * smooth;
        P.barSmooth = pd.barrier + smooth;
        P.minusSmooth = pd.barrier - smooth;
        const double lb = P.minusSmooth > 0 ? std::log(P.minusSmooth) : -INFINITY;
        P.logBandD = lb - 1e-9;
        P.logBandF = float(m.kind == MODEL_DUPIRE ? lb - P.x0d - 1e-5 : lb - 1e-5);
    }

    if (pd.kind == PROD_CONTINGENT)
    {
        // coverages myDt (mcPrd.h:441-452); smoothing from the first spot (mcPrd.h:531-532)
        for (int e = 0; e + 1 < plan.nEv; ++e) ev[9 * plan.nEv + e] = pd.timeline[e + 1] - pd.timeline[e];
        P.coupon = pd.coupon;
        P.cbSmooth = frontSpot * pd.smooth;
    }
    std::vector<int> evPoint(std::max(1, plan.nEv), 0);
    for (int i = 0; i <= plan.nSteps; ++i)
        if (evAtStep[i] >= 0) evPoint[evAtStep[i]] = i;
    const size_t oEvPt = pk.vec(evPoint);
    const size_t oEv = pk.vec(evAtStep);
    const size_t oEvD = pk.vec(ev), oEvF = pk.vec(to_f(ev));
    std::vector<double> kf = pd.kflat;
    if (kf.empty()) kf.push_back(0.0);
    std::vector<int> po = pd.payOff;
    if (po.empty()) po = {0, 0};
    const size_t oK = pk.vec(kf), oKf = pk.vec(to_f(kf)), oPo = pk.vec(po);
    size_t oDir = 0;
    if (plan.nSteps <= sobol_max_dim())
    {
        auto& dirs = sobolDirs[plan.nSteps];  // regenerated once per dimension count
        if (dirs.empty()) dirs = sobol_dirs(plan.nSteps);
        oDir = pk.vec(dirs);
    }
    plan.sobolOk = plan.nSteps <= sobol_max_dim();

    int rc = plan.tables.ensure(pk.buf.size());
    if (rc) return rc;
    CF_CUDA(cudaMemcpyAsync(plan.tables.ptr, pk.buf.data(), pk.buf.size(), cudaMemcpyHostToDevice, stream));
    h2d += pk.buf.size();
    // the tables are read by kernels on any slot's stream: the upload completes here
    CF_CUDA(cudaStreamSynchronize(stream));
    unsigned char* d = static_cast<unsigned char*>(plan.tables.ptr);
    auto D = [&](size_t off) { return static_cast<const void*>(d + off); };
    if (m.kind == MODEL_BS)
    {
        P.bsD = (const double*)D(oBs);
        P.bsF = (const float*)D(oBsF);
    }
    else
    {
        P.Xd = (const double*)D(oX);
        P.invdXd = (const double*)D(oInv);
        P.Yd = (const double*)D(oY);
        P.Xf = (const float*)D(oXf);
        P.invdXf = (const float*)D(oInvf);
        P.Yf = (const float*)D(oYf);
        P.colA = (const int*)D(oColA);
        P.bucket = (const int*)D(oBucket);
        P.colB = (const int*)D(oColB);
        P.cAd = (const double*)D(oCA);
        P.cBd = (const double*)D(oCB);
        P.cAf = (const float*)D(oCAf);
        P.cBf = (const float*)D(oCBf);
        P.wAi = (const int*)D(oWA);
        P.wBi = (const int*)D(oWB);
        P.xsF = (const float*)D(oXs);
        P.irF = (const float*)D(oIr);
        P.tdF = (const float*)D(oTd);
        P.stepcF = (const int4*)D(oSc);
        P.bucketF = (const int*)D(oBf);
        P.volsD = (const double*)D(oVols);
        P.stepSqD = (const double*)D(oSq);
        P.stepTwD = (const double*)D(oTw);
    }
    P.evAtStep = (const int*)D(oEv);
    P.evPoint = (const int*)D(oEvPt);
    P.evD = (const double*)D(oEvD);
    P.evF = (const float*)D(oEvF);
    P.kD = (const double*)D(oK);
    P.kF = (const float*)D(oKf);
    P.evPayOff = (const int*)D(oPo);
    P.sobolDir = plan.sobolOk ? (const unsigned*)D(oDir) : nullptr;
    plan.evAtStep = evAtStep;
    P.evEvery = 1;
    for (int i = 1; i <= plan.nSteps; ++i)
        if (evAtStep[i] < 0) P.evEvery = 0;
    return CF_OK;
}

// ------------------------------------------------------------------------------------
// Context
// ------------------------------------------------------------------------------------
int Context::init(int dev)
{
    device = dev;
    CF_CUDA(cudaSetDevice(dev));
    CF_CUDA(cudaStreamCreateWithFlags(&ownStream, cudaStreamNonBlocking));
    stream = ownStream;
    CF_CUDA(cudaDeviceGetAttribute(&numSMs, cudaDevAttrMultiProcessorCount, dev));
    // slot buffers grow through the stream-ordered allocator: the device's pool keeps what they
    // free for reuse instead of returning it at every synchronisation
    {
        cudaMemPool_t pool;
        uint64_t keep = ~0ULL;
        if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess)
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    uint32_t A[256][12], B[256][12];
    mrg_jump_tables(A, B);
    int rc = jump.ensure(sizeof(A) + sizeof(B));
    if (rc) return rc;
    CF_CUDA(cudaMemcpy(jump.ptr, A, sizeof(A), cudaMemcpyHostToDevice));
    CF_CUDA(cudaMemcpy(static_cast<char*>(jump.ptr) + sizeof(A), B, sizeof(B), cudaMemcpyHostToDevice));
    jumpA = static_cast<const unsigned*>(jump.ptr);
    jumpB = jumpA + 256 * 12;
    // uniforms: mrg32k3a d / (m1 + 1) (mrg32k3a.h:52,78-79), Sobol s * 2.3283064365387e-10 (sobol.h:26)
    std::vector<float> tab(2 * size_t(INVN_PIECES) * 4);
    inv_normal_table(4294967088.0, tab.data());
    inv_normal_table(1.0 / 2.3283064365387e-10, tab.data() + size_t(INVN_PIECES) * 4);
    if ((rc = invn.ensure(tab.size() * sizeof(float)))) return rc;
    CF_CUDA(cudaMemcpy(invn.ptr, tab.data(), tab.size() * sizeof(float), cudaMemcpyHostToDevice));
    invnMrg = static_cast<const float*>(invn.ptr);
    invnSobol = invnMrg + size_t(INVN_PIECES) * 4;
    main.stream = stream;
    return CF_OK;
}

Context::~Context()
{
    cudaSetDevice(device);
    plans.clear();
    if (ownStream) cudaStreamDestroy(ownStream);
}

int Context::getPlan(const std::string& mid, const std::string& pid, Plan*& out)
{
    auto mi = models.find(mid);
    auto pi = products.find(pid);
    if (mi == models.end() || pi == products.end())
        return fail(CF_E_NOTFOUND, "Could not retrieve model and product: '" + mid + "', '" + pid + "'");
    auto key = std::make_pair(mid, pid);
    auto it = plans.find(key);
    if (it != plans.end() && it->second->mver == mi->second.version && it->second->pver == pi->second.version)
    {
        out = it->second.get();
        return CF_OK;
    }
    auto plan = std::make_shared<Plan>();
    if (it != plans.end())
    {
        // the model or product changed: the new plan takes over the stale plan's device tables
        // once no kernel can still read them (a device-wide wait, as freeing them would be)
        CF_CUDA(cudaDeviceSynchronize());
        plan->tables.swap(it->second->tables);
    }
    int rc = buildPlan(mi->second, pi->second, *plan);
    if (rc) return rc;
    plan->mver = mi->second.version;
    plan->pver = pi->second.version;
    out = plan.get();
    plans[key] = std::move(plan);
    return CF_OK;
}

// Enqueue one value (risk = false) or risk (risk = true, weights[nPay]) run on a slot: the
// weights upload, the accumulator reset, the kernel and the download of the accumulators
// into the slot's pinned buffer are all asynchronous on the slot's stream; slot.done is
// recorded after them.
int Context::enqueue(Slot& slot, Plan& plan, const cf_num_param& num, bool risk, const double* weights,
                     long long firstPath, double* pathOut, long long chunkPaths, int maxBlocksPerSM)
{
    if (num.numPath <= 0) return fail(CF_E_ARG, "numPath must be positive");
    if (firstPath < 0 || firstPath % 64) return fail(CF_E_ARG, "firstPath must be a non-negative multiple of 64");
    if (plan.model == MODEL_MULTI) return enqueueMd(slot, plan, num, risk, weights, firstPath);
    const bool sobol = num.useSobol != 0;
    if (sobol && !plan.sobolOk)
        return fail(CF_E_SHAPE, "Sobol dimension " + std::to_string(plan.nSteps) + " exceeds the " +
                                    std::to_string(sobol_max_dim()) + " dimensions of the direction numbers");
    const bool fp32 = num.precision == CF_FP32;
    cudaStream_t st = slot.stream;
    McParams p = plan.base;
    p.nPath = num.numPath;
    p.firstPath = firstPath;
    p.seed1 = unsigned(num.seed1);
    p.seed2 = unsigned(num.seed2);
    p.mrgJumpA = jumpA;
    p.mrgJumpB = jumpB;
    p.invnF = sobol ? invnSobol : invnMrg;
    p.nRisk = risk ? plan.nParam : 0;
    p.nAcc = p.nRisk + 2 * plan.nPay + 2;
    p.pathOut = risk ? nullptr : pathOut;
    // chunked runs (the serving loop's long requests): launches of chunkPaths paths each
    const long long totalPaths = p.nPath;
    const long long chunk = (!pathOut && chunkPaths >= 64 && chunkPaths < totalPaths) ? (chunkPaths & ~63LL) : totalPaths;
    const long long nChunk = (totalPaths + chunk - 1) / chunk;
    // weights (double and float copies), accumulators, the error flag and one round counter per
    // launch share one buffer
    const size_t wBytes = ((size_t(plan.nPay) * 12 + 255) & ~size_t(255));
    const size_t accBytes = size_t(p.nAcc) * 16;
    const size_t claimBytes = size_t(nChunk) * 8;
    int rc = slot.work.ensure(wBytes + accBytes + 16 + claimBytes + 256, st);
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
    p.claim = reinterpret_cast<unsigned long long*>(wbase + wBytes + accBytes + 16);
    CF_CUDA(cudaMemsetAsync(p.acc, 0, accBytes + 16 + claimBytes, st));

    McLaunch l{plan.model, plan.prod, sobol ? RNG_SOBOL : RNG_MRG, fp32 ? 1 : 0, risk ? 1 : 0, 0, 0, 0, 0};
    // FP32 Dupire risk runs dupire_risk32 when the plan has its tables and its node slab fits
    // an SM; everything else runs the generic mc_kernel.
    int stage = 0;
    size_t smem0 = 0, smem1 = 0;
    int occ0 = 0, occ1 = 0;
    l.fast = mc_use_fast32(plan.base, plan.prod, l.fp32, l.risk);
    if (l.fast)
    {
        // the local-vol rows (bulk copies) and the inverse-normal table go to shared memory when
        // that costs no occupancy
        p.stageY = 0;
        p.rowChunk = 0;
        mc_smem_bytes(l, p, 0, &smem0);
        if (smem0 > 200 * 1024 || mc_occupancy(l, smem0, &occ0) || occ0 < 1) l.fast = 0;
        else occ0 = r32_staging(l, p, occ0, &smem0);
    }
    if (!l.fast)
    {
        mc_smem_bytes(l, p, 0, &smem0);
        rc = mc_occupancy(l, smem0, &occ0);
        if (rc) return cuda_fail(cudaError_t(rc), "occupancy");
    }
    // Shared-memory staging of the interpolated local vols (a bulk copy through the TMA
    // unit): used only when it costs no occupancy; otherwise the table is read through L1.
    if (plan.model == MODEL_DUPIRE && !l.fast)
    {
        mc_smem_bytes(l, p, 1, &smem1);
        const char* env = std::getenv("CF_STAGE_Y");
        if (smem1 <= 200 * 1024)
        {
            rc = mc_occupancy(l, smem1, &occ1);
            if (rc) return cuda_fail(cudaError_t(rc), "occupancy");
            stage = occ1 >= occ0;  // only when it costs no occupancy (the kernel is latency-bound)
        }
        if (env && env[0] == '0') stage = 0;
        if (env && env[0] == '1' && occ1 > 0) stage = 1;
    }
    if (!l.fast) p.stageY = stage;
    l.smem = stage ? smem1 : smem0;
    const int occ = stage ? occ1 : occ0;
    if (occ < 1) return fail(CF_E_SHAPE, "kernel does not fit on an SM (shared memory " + std::to_string(l.smem) + ")");
    // chunked runs: the grid and the scratch are sized for one chunk, the launches below cover
    // the whole run
    p.nPath = chunk;
    const long long threadsNeeded = sobol ? (p.nPath / 32 + 1) * 32 : (p.nPath + 1) / 2;
    long long grid = (threadsNeeded + 127) / 128;
    const long long maxGrid = (long long)numSMs * (maxBlocksPerSM > 0 ? std::min(occ, maxBlocksPerSM) : occ);
    if (grid > maxGrid) grid = maxGrid;
    if (grid < 1) grid = 1;
    l.grid = int(grid);
    l.block = 128;
    if (risk)
    {
        // kernels index the scratch with 32-bit offsets: keep fields*(steps+1)*threads < 2^31
        // (sized for the full ring, the most fields a launch can need)
        const long long perThread = (long long)mc_scratch_fields(l, R32_RING) * (plan.nSteps + 1);
        const long long maxThreads = ((1LL << 31) - 1) / perThread;
        if (grid * 128 > maxThreads) grid = std::max(1LL, maxThreads / 128);
        l.grid = int(grid);
        p.scratchThreads = grid * 128;
        const long long rounds = mc_rounds(l, p.nPath, grid * 128);
        p.scratchFields = mc_scratch_fields(l, rounds);
        p.roundCap = rounds < R32_RING ? rounds : 0;
        const size_t bytes = mc_scratch_bytes(l, p, grid);
        if ((rc = slot.scratch.ensure(bytes, st))) return rc;
        p.scratch = slot.scratch.ptr;
    }
    int nLaunch = 0;
    for (long long off = 0; off < totalPaths; off += chunk)
    {
        McParams q = p;
        q.firstPath = firstPath + off;
        q.nPath = std::min(chunk, totalPaths - off);
        q.claim = p.claim + nLaunch;
        rc = launch_mc(l, q, st);
        if (rc) return cuda_fail(cudaError_t(rc), "mc_kernel launch");
        ++nLaunch;
    }
    p.nPath = totalPaths;  // the averages are over the whole run
    CF_CUDA(cudaMemcpyAsync(slot.hostAcc.ptr, p.acc, accBytes + 16, cudaMemcpyDeviceToHost, st));
    d2h += accBytes + 16;
    if (!slot.done) CF_CUDA(cudaEventCreateWithFlags(&slot.done, cudaEventDisableTiming));
    CF_CUDA(cudaEventRecord(slot.done, st));
    slot.last = p;
    slot.plan = &plan;
    slot.planRef = plan.weak_from_this().lock();
    slot.risk = risk;
    slot.multi = false;
    slot.launches = nLaunch;
    return CF_OK;
}

// Estimated device footprint of a run (scratch of the reverse sweep + accumulators), the
// admission currency of the serving loop.
size_t Context::footprint(const Plan& plan, const cf_num_param& num, bool risk) const
{
    const bool sobol = num.useSobol != 0, fp32 = num.precision == CF_FP32;
    const int NP = sobol ? 1 : 2;
    if (plan.model == MODEL_MULTI)
    {
        // multi-asset: per thread the Gaussians, the spots and the notionals of the reverse
        // sweep; at most 4 resident blocks of 128 threads per SM (the kernels are register-heavy)
        const long long needed = sobol ? (num.numPath / 32 + 1) * 32 : (num.numPath + 1) / 2;
        const long long threads = std::min<long long>(needed, (long long)numSMs * 4 * 128);
        const size_t dim = size_t(plan.nSteps) * plan.base.nA;
        size_t b = size_t(plan.mdTotal + 2 * plan.nPay + 2) * 16 + 4096;
        if (risk) b += (dim + NP * dim + NP * size_t(plan.nEv)) * size_t(threads) * (fp32 ? 4 : 8);
        return b;
    }
    // resident threads of the launch (the grid of enqueue), bounded by the occupancy limit
    McParams p = plan.base;
    p.nRisk = risk ? plan.nParam : 0;
    p.nAcc = p.nRisk + 2 * plan.nPay + 2;
    McLaunch l{plan.model, plan.prod, sobol ? RNG_SOBOL : RNG_MRG, fp32 ? 1 : 0, risk ? 1 : 0, 0, 0, 0, 0};
    l.fast = mc_use_fast32(plan.base, plan.prod, l.fp32, l.risk);
    size_t smem = 0;
    mc_smem_bytes(l, p, 0, &smem);
    int occ = 16;
    if (mc_occupancy(l, smem, &occ) || occ < 1) occ = 16;
    const long long needed = sobol ? (num.numPath / 32 + 1) * 32 : (num.numPath + 1) / 2;
    const long long threads = std::min<long long>(needed, (long long)numSMs * occ * 128);
    if (plan.prod == PROD_EUROPEANS && risk && multi32Use(plan, num))
    {
        // multi_risk32.cu: step records per path, bucket and spot per (maturity, path), entry
        // lists, bucket accumulators and the finished risks
        const size_t nP = size_t(num.numPath), nE = size_t(plan.nEv);
        return nP * size_t((plan.nSteps + 1) & ~1) * 8 + nE * nP * 14 +
               size_t(plan.nPay + plan.nEv) * size_t(plan.nParam) * 16 + size_t(plan.nPay) * size_t(plan.nParam) * 8 +
               size_t(plan.nPay + plan.nEv) * 96 + 8192;
    }
    const int fields = plan.prod == PROD_EUROPEANS ? 1 + 3 * NP : mc_scratch_fields(l, mc_rounds(l, num.numPath, threads));
    size_t b = size_t(plan.nParam + 2 * plan.nPay + 2) * 16 + size_t(plan.nPay) * 12 + 4096;
    if (risk) b += size_t(fields) * size_t(plan.nSteps + 1) * size_t(threads) * (fp32 ? 4 : 8);
    if (risk && l.fast) b += size_t((threads + 127) / 128) * size_t(plan.base.nS) * size_t(plan.base.nT) * 8 + 256;
    // multi: bucket accumulators plus the finished per-payoff risks
    if (plan.prod == PROD_EUROPEANS && risk) b += size_t(plan.nPay + plan.nEv) * size_t(plan.nParam) * 16 + size_t(plan.nPay) * size_t(plan.nParam) * 8;
    return b;
}

bool Context::ready(Slot& slot) const
{
    return !slot.done || cudaEventQuery(slot.done) != cudaErrorNotReady;
}

int Context::fetch(Slot& slot, double* values, double* stderrs, double* aggregate, double* risks)
{
    if (!slot.plan) return fail(CF_E_ARG, "nothing enqueued");
    CF_CUDA(cudaEventSynchronize(slot.done));
    if (slot.multi) return finishMulti(slot, values, risks, aggregate);
    const McParams& p = slot.last;
    const long long* acc = static_cast<const long long*>(slot.hostAcc.ptr);
    const int e = *reinterpret_cast<const int*>(acc + 2 * size_t(p.nAcc));
    if (e) return fail(CF_E_DEVICE, "kernel error flag " + std::to_string(e));
    if (slot.plan->model == MODEL_MULTI && slot.risk && risks)
    {
        // path-averaged adjoints of the derived quantities -> parameter risks through the
        // Jacobian of the model's initialisation
        const Plan& pl = *slot.plan;
        std::vector<double> der(size_t(p.nRisk));
        results_from_acc(acc, p.nRisk, p.nPay, p.nPath, values, stderrs, aggregate, der.data());
        for (int j = 0; j < pl.nParam; ++j) risks[j] = 0.0;
        for (int d = 0; d < p.nRisk; ++d)
            if (der[d] != 0.0)
            {
                const double* row = &pl.mdJac[size_t(d) * pl.nParam];
                for (int j = 0; j < pl.nParam; ++j) risks[j] += der[d] * row[j];
            }
        return CF_OK;
    }
    results_from_acc(acc, p.nRisk, p.nPay, p.nPath, values, stderrs, aggregate, slot.risk ? risks : nullptr);
    return CF_OK;
}

// Path averages of the exact accumulators (hi, lo pairs): payoff means and Monte Carlo
// standard errors, the aggregate's mean, the risks (parameter adjoints / nPath).
void results_from_acc(const long long* acc, int nRisk, int nPay, long long nPath, double* values, double* stderrs,
                      double* aggregate, double* risks)
{
    const double n = double(nPath);
    auto val = [&](int i) { return fix_value_host(acc[2 * size_t(i)], acc[2 * size_t(i) + 1]); };
    for (int k = 0; k < nPay; ++k)
    {
        const double s = val(nRisk + k), q = val(nRisk + nPay + k);
        const double mean = s / n;
        if (values) values[k] = mean;
        if (stderrs) stderrs[k] = std::sqrt(std::max(0.0, q / n - mean * mean) / n);
    }
    if (aggregate) aggregate[0] = val(nRisk + 2 * nPay) / n;
    if (risks)
        for (int j = 0; j < nRisk; ++j) risks[j] = val(j) / n;
}

double fix_value_host(long long hi, long long lo)
{
    return (double)hi * (1.0 / 1048576.0) + (double)lo * (1.0 / 1152921504606846976.0);
}

}  // namespace cf

// =====================================================================================
// C ABI
// =====================================================================================
using namespace cf;

#define CF_CTX()                                               \
    if (!ctx) return fail(CF_E_ARG, "null context");           \
    std::lock_guard<std::mutex> lock_(ctx->mu);                \
    cudaSetDevice(ctx->c.device);

extern "C" {

int cf_create(int device, cf_context** out)
{
    if (!out) return fail(CF_E_ARG, "null output");
    *out = nullptr;
    auto c = std::make_unique<cf_context>();
    const int rc = c->c.init(device);
    if (rc) return rc;
    *out = c.release();
    return CF_OK;
}

int cf_destroy(cf_context* ctx)
{
    delete ctx;
    return CF_OK;
}

int cf_last_error(char* buf, size_t size)
{
    if (!buf || !size) return CF_E_ARG;
    std::snprintf(buf, size, "%s", g_lastError.c_str());
    return CF_OK;
}

int cf_bucket_grid(const float* knots, int nKnots, int capacity, float* x0, float* invW, int* nBuckets, int* ok,
                   int* oneCompare, int* first)
{
    if (!knots || nKnots < 1 || !nBuckets) return fail(CF_E_ARG, "bucket grid: null argument or no knots");
    for (int j = 0; j + 1 < nKnots; ++j)
        if (!(knots[j] < knots[j + 1])) return fail(CF_E_ARG, "bucket grid: knots not strictly ascending");
    const BucketGrid g = bucket_grid(std::vector<float>(knots, knots + nKnots));
    *nBuckets = int(g.first.size());
    if (x0) *x0 = g.x0;
    if (invW) *invW = g.invW;
    if (ok) *ok = g.ok ? 1 : 0;
    if (oneCompare) *oneCompare = g.oneCompare ? 1 : 0;
    if (first)
    {
        if (capacity < *nBuckets) return fail(CF_E_SHAPE, "bucket grid: capacity below the bucket count");
        std::copy(g.first.begin(), g.first.end(), first);
    }
    return CF_OK;
}

int cf_set_stream(cf_context* ctx, void* stream)
{
    CF_CTX();
    ctx->c.stream = stream ? static_cast<cudaStream_t>(stream) : ctx->c.ownStream;
    ctx->c.main.stream = ctx->c.stream;
    return CF_OK;
}

int cf_transfer_stats(cf_context* ctx, uint64_t* h2dBytes, uint64_t* d2hBytes)
{
    CF_CTX();
    if (h2dBytes) *h2dBytes = ctx->c.h2d;
    if (d2hBytes) *d2hBytes = ctx->c.d2h;
    return CF_OK;
}

int cf_synchronize(cf_context* ctx)
{
    CF_CTX();
    CF_CUDA(cudaStreamSynchronize(ctx->c.stream));
    return CF_OK;
}

static int check_id(const char* id) { return id && *id ? CF_OK : fail(CF_E_ARG, "empty id"); }

int cf_put_black_scholes(cf_context* ctx, double spot, double vol, int qSpot, double rate, double div, const char* id)
{
    CF_CTX();
    if (check_id(id)) return CF_E_ARG;
    ModelDesc m;
    m.kind = MODEL_BS;
    m.spot = spot;
    m.vol = vol;
    m.qSpot = qSpot != 0;
    m.rate = rate;
    m.div = div;
    m.version = ++ctx->c.versionCounter;
    m.build();
    ctx->c.models[id] = std::move(m);
    return CF_OK;
}

int cf_put_dupire(cf_context* ctx, double spot, const double* spots, int nSpots, const double* times, int nTimes,
                  const double* vols, double maxDt, const char* id)
{
    CF_CTX();
    if (check_id(id)) return CF_E_ARG;
    if (!spots || !times || !vols || nSpots < 1 || nTimes < 1 || !(maxDt > 0))
        return fail(CF_E_ARG, "putDupire: bad grid");
    ModelDesc m;
    m.kind = MODEL_DUPIRE;
    m.spot = spot;
    m.spots.assign(spots, spots + nSpots);
    m.times.assign(times, times + nTimes);
    m.vols.assign(vols, vols + size_t(nSpots) * nTimes);
    m.maxDt = maxDt;
    m.version = ++ctx->c.versionCounter;
    m.build();
    ctx->c.models[id] = std::move(m);
    return CF_OK;
}

int cf_put_european(cf_context* ctx, double strike, double exerciseDate, double settlementDate, const char* id)
{
    CF_CTX();
    if (check_id(id)) return CF_E_ARG;
    ProductDesc p;
    p.kind = PROD_EUROPEAN;
    p.strike = strike;
    p.exercise = exerciseDate;
    p.settlement = settlementDate;
    p.version = ++ctx->c.versionCounter;
    p.build();
    ctx->c.products[id] = std::move(p);
    return CF_OK;
}

int cf_put_contingent(cf_context* ctx, double coupon, double maturity, double payFreq, double smooth, const char* id)
{
    CF_CTX();
    if (check_id(id)) return CF_E_ARG;
    if (!(payFreq > 0) || !(maturity > 0)) return fail(CF_E_ARG, "putContingent: bad maturity or frequency");
    ProductDesc p;
    p.kind = PROD_CONTINGENT;
    p.coupon = coupon;
    p.maturity = maturity;
    p.freq = payFreq;
    p.smooth = smooth <= 0 ? 0.0 : smooth;  // store.h:172
    p.version = ++ctx->c.versionCounter;
    p.build();
    ctx->c.products[id] = std::move(p);
    return CF_OK;
}

int cf_put_barrier(cf_context* ctx, double strike, double barrier, double maturity, double monitorFreq,
                   double smooth, int callPut, const char* id)
{
    CF_CTX();
    if (check_id(id)) return CF_E_ARG;
    if (!(monitorFreq > 0) || !(maturity > 0)) return fail(CF_E_ARG, "putBarrier: bad maturity or frequency");
    ProductDesc p;
    p.kind = PROD_UOC;
    p.strike = strike;
    p.barrier = barrier;
    p.maturity = maturity;
    p.freq = monitorFreq;
    p.smooth = smooth <= 0 ? kEps : smooth;  // store.h:153
    p.callPut = callPut ? 1 : 0;
    p.version = ++ctx->c.versionCounter;
    p.build();
    ctx->c.products[id] = std::move(p);
    return CF_OK;
}

int cf_put_europeans(cf_context* ctx, const double* maturities, const double* strikes, int n, const char* id)
{
    CF_CTX();
    if (check_id(id)) return CF_E_ARG;
    if (!maturities || !strikes || n < 1) return fail(CF_E_ARG, "putEuropeans: empty portfolio");
    ProductDesc p;
    p.kind = PROD_EUROPEANS;
    p.mats.assign(maturities, maturities + n);
    p.strikes.assign(strikes, strikes + n);
    p.version = ++ctx->c.versionCounter;
    p.build();
    ctx->c.products[id] = std::move(p);
    return CF_OK;
}

static int read_names(int n, const char* const* names, std::vector<std::string>& out)
{
    out.clear();
    if (n < 1 || !names) return fail(CF_E_ARG, "no assets");
    for (int i = 0; i < n; ++i)
    {
        if (!names[i] || !*names[i]) return fail(CF_E_ARG, "empty asset name");
        out.emplace_back(names[i]);
    }
    return CF_OK;
}

int cf_put_displaced(cf_context* ctx, int nA, const char* const* assets, const double* spots, const double* atms,
                     const double* skews, double discRate, const double* repoSpreads, int nDiv,
                     const double* divDates, const double* divs, const double* correl, double lambda, const char* id)
{
    CF_CTX();
    if (check_id(id)) return CF_E_ARG;
    ModelDesc m;
    m.kind = MODEL_MULTI;
    if (read_names(nA, assets, m.assets)) return CF_E_ARG;
    if (nA > 16) return fail(CF_E_SHAPE, "putDisplaced: at most 16 assets");
    if (!spots || !atms || !skews || !repoSpreads || !correl || nDiv < 0 || (nDiv > 0 && (!divDates || !divs)))
        return fail(CF_E_ARG, "putDisplaced: missing inputs");
    for (int d = 1; d < nDiv; ++d)
        if (!(divDates[d] > divDates[d - 1])) return fail(CF_E_ARG, "putDisplaced: dividend dates must increase");
    m.disc = discRate;
    m.lambda = lambda;
    m.aSpots.assign(spots, spots + nA);
    m.atms.assign(atms, atms + nA);
    m.skews.assign(skews, skews + nA);
    m.spreads.assign(repoSpreads, repoSpreads + nA);
    if (nDiv > 0)
    {
        m.divDates.assign(divDates, divDates + nDiv);
        m.divs.assign(divs, divs + size_t(nDiv) * nA);
    }
    m.correl.assign(correl, correl + size_t(nA) * nA);
    m.version = ++ctx->c.versionCounter;
    m.build();
    ctx->c.models[id] = std::move(m);
    return CF_OK;
}

int cf_put_baskets(cf_context* ctx, int nA, const char* const* assets, const double* weights, double maturity, int nK,
                   const double* strikes, const char* id)
{
    CF_CTX();
    if (check_id(id)) return CF_E_ARG;
    ProductDesc p;
    p.kind = PROD_BASKETS;
    if (read_names(nA, assets, p.assets)) return CF_E_ARG;
    if (!(maturity > 0)) return fail(CF_E_ARG, "putBaskets: maturity must be positive");
    if (!weights || !strikes || nK < 1) return fail(CF_E_ARG, "putBaskets: weights and strikes required");
    p.weights.assign(weights, weights + nA);
    p.maturity = maturity;
    p.strikes.assign(strikes, strikes + nK);
    p.version = ++ctx->c.versionCounter;
    p.build();
    ctx->c.products[id] = std::move(p);
    return CF_OK;
}

int cf_put_autocall(cf_context* ctx, int nA, const char* const* assets, const double* refs, double maturity, int periods,
                    double ko, double strike, double cpn, double smooth, const char* id)
{
    CF_CTX();
    if (check_id(id)) return CF_E_ARG;
    ProductDesc p;
    p.kind = PROD_AUTOCALL;
    if (read_names(nA, assets, p.assets)) return CF_E_ARG;
    if (!refs) return fail(CF_E_ARG, "putAutocall: one reference level per asset");
    if (!(maturity > 0) || periods < 1) return fail(CF_E_ARG, "putAutocall: positive maturity and periods");
    p.refs.assign(refs, refs + nA);
    p.maturity = maturity;
    p.periods = periods;
    p.ko = ko;
    p.strike = strike;
    p.cpn = cpn;
    p.smooth = smooth;
    p.version = ++ctx->c.versionCounter;
    p.build();
    ctx->c.products[id] = std::move(p);
    return CF_OK;
}

int cf_md_state(cf_context* ctx, const char* modelId, const char* productId, double* derived, int capacity, int* count,
                int* dynamics)
{
    CF_CTX();
    Plan* plan;
    int rc = ctx->c.getPlan(modelId ? modelId : "", productId ? productId : "", plan);
    if (rc) return rc;
    if (plan->model != MODEL_MULTI) return fail(CF_E_ARG, "not a multi-asset model");
    if (count) *count = plan->mdTotal;
    if (derived)
    {
        if (capacity < plan->mdTotal) return fail(CF_E_ARG, "cf_md_state: buffer too small");
        std::memcpy(derived, plan->mdDerived.data(), size_t(plan->mdTotal) * 8);
    }
    if (dynamics)
    {
        std::vector<int> dyn(plan->base.nA);
        CF_CUDA(cudaMemcpy(dyn.data(), plan->base.mdDyn, dyn.size() * 4, cudaMemcpyDeviceToHost));
        std::memcpy(dynamics, dyn.data(), dyn.size() * 4);
    }
    return CF_OK;
}

static int write_labels(const std::vector<std::string>& l, char* buf, size_t size, int* count, size_t* needed)
{
    std::string s;
    for (size_t i = 0; i < l.size(); ++i)
    {
        if (i) s += '\n';
        s += l[i];
    }
    if (count) *count = int(l.size());
    if (needed) *needed = s.size() + 1;
    if (!buf) return CF_OK;
    if (size < s.size() + 1) return fail(CF_E_SHAPE, "label buffer too small");
    std::memcpy(buf, s.c_str(), s.size() + 1);
    return CF_OK;
}

int cf_payoff_labels(cf_context* ctx, const char* productId, char* buf, size_t size, int* count, size_t* needed)
{
    CF_CTX();
    auto it = ctx->c.products.find(productId ? productId : "");
    if (it == ctx->c.products.end()) return fail(CF_E_NOTFOUND, "product not found");
    return write_labels(it->second.labels, buf, size, count, needed);
}

int cf_parameter_labels(cf_context* ctx, const char* modelId, char* buf, size_t size, int* count, size_t* needed)
{
    CF_CTX();
    auto it = ctx->c.models.find(modelId ? modelId : "");
    if (it == ctx->c.models.end()) return fail(CF_E_NOTFOUND, "model not found");
    return write_labels(it->second.labels(), buf, size, count, needed);
}

int cf_shapes(cf_context* ctx, const char* modelId, const char* productId, int* nPay, int* nParam, int* simDim)
{
    CF_CTX();
    Plan* plan;
    int rc = ctx->c.getPlan(modelId ? modelId : "", productId ? productId : "", plan);
    if (rc) return rc;
    if (nPay) *nPay = plan->nPay;
    if (nParam) *nParam = plan->nParam;
    if (simDim) *simDim = plan->model == MODEL_MULTI ? plan->nSteps * plan->base.nA : plan->nSteps;
    return CF_OK;
}

int cf_model_grid(cf_context* ctx, const char* modelId, int* nSpots, int* nTimes, double* spots, double* times)
{
    CF_CTX();
    auto it = ctx->c.models.find(modelId ? modelId : "");
    if (it == ctx->c.models.end()) return fail(CF_E_NOTFOUND, "dupireAADRisk() : Model not found");
    const ModelDesc& m = it->second;
    if (m.kind != MODEL_DUPIRE) return fail(CF_E_ARG, "dupireAADRisk() : Model not a Dupire");
    if (nSpots) *nSpots = int(m.spots.size());
    if (nTimes) *nTimes = int(m.times.size());
    if (spots) std::copy(m.spots.begin(), m.spots.end(), spots);
    if (times) std::copy(m.times.begin(), m.times.end(), times);
    return CF_OK;
}

int cf_value(cf_context* ctx, const char* modelId, const char* productId, const cf_num_param* num, double* values,
             double* stderrs)
{
    CF_CTX();
    if (!num || !values) return fail(CF_E_ARG, "null argument");
    Plan* plan;
    int rc = ctx->c.getPlan(modelId ? modelId : "", productId ? productId : "", plan);
    if (rc) return rc;
    if ((rc = ctx->c.enqueue(*plan, *num, false, nullptr))) return rc;
    return ctx->c.fetch(values, stderrs, nullptr, nullptr);
}

static int payoff_index(const Plan& plan, const ProductDesc& pd, const char* label, int* idx)
{
    *idx = 0;
    if (!label || !*label) return CF_OK;
    for (size_t i = 0; i < pd.labels.size(); ++i)
        if (pd.labels[i] == label)
        {
            *idx = int(i);
            return CF_OK;
        }
    (void)plan;
    return fail(CF_E_NOTFOUND, "AADriskOne() : payoff not found");
}

int cf_aad_risk_one(cf_context* ctx, const char* modelId, const char* productId, const cf_num_param* num,
                    const char* riskPayoff, double* payoffValues, double* riskPayoffValue, double* risks)
{
    CF_CTX();
    if (!num || !risks) return fail(CF_E_ARG, "null argument");
    Plan* plan;
    int rc = ctx->c.getPlan(modelId ? modelId : "", productId ? productId : "", plan);
    if (rc) return rc;
    int k;
    if ((rc = payoff_index(*plan, ctx->c.products[productId], riskPayoff, &k))) return rc;
    std::vector<double> w(plan->nPay, 0.0);
    w[k] = 1.0;
    return ctx->c.aggregateRisk(*plan, *num, w.data(), payoffValues, riskPayoffValue, risks);
}

int cf_aad_risk_aggregate(cf_context* ctx, const char* modelId, const char* productId, const double* notionals,
                          const cf_num_param* num, double* payoffValues, double* aggregateValue, double* risks)
{
    CF_CTX();
    if (!num || !risks || !notionals) return fail(CF_E_ARG, "null argument");
    Plan* plan;
    int rc = ctx->c.getPlan(modelId ? modelId : "", productId ? productId : "", plan);
    if (rc) return rc;
    return ctx->c.aggregateRisk(*plan, *num, notionals, payoffValues, aggregateValue, risks);
}

int cf_aad_risk_multi(cf_context* ctx, const char* modelId, const char* productId, const cf_num_param* num,
                      double* values, double* risks)
{
    CF_CTX();
    if (!num || !risks) return fail(CF_E_ARG, "null argument");
    Plan* plan;
    int rc = ctx->c.getPlan(modelId ? modelId : "", productId ? productId : "", plan);
    if (rc) return rc;
    return ctx->c.riskMulti(*plan, *num, values, risks);
}

int cf_simulate_paths(cf_context* ctx, const char* modelId, const char* productId, const cf_num_param* num,
                      double* payoffs)
{
    CF_CTX();
    if (!num || !payoffs) return fail(CF_E_ARG, "null argument");
    if (num->numPath <= 0) return fail(CF_E_ARG, "numPath must be positive");
    Plan* plan;
    int rc = ctx->c.getPlan(modelId ? modelId : "", productId ? productId : "", plan);
    if (rc) return rc;
    if (plan->model == MODEL_MULTI)
        return fail(CF_E_UNSUPPORTED, "mcSimul: per-path payoffs of the multi-asset model are not supported");
    Context& c = ctx->c;
    const size_t bytes = size_t(num->numPath) * size_t(plan->nPay) * 8;
    if ((rc = c.main.paths.ensure(bytes, c.stream))) return rc;
    double* dev = static_cast<double*>(c.main.paths.ptr);
    if ((rc = c.enqueue(*plan, *num, false, nullptr, dev))) return rc;
    if ((rc = c.fetch(nullptr, nullptr, nullptr, nullptr))) return rc;
    CF_CUDA(cudaMemcpyAsync(payoffs, dev, bytes, cudaMemcpyDeviceToHost, c.stream));
    CF_CUDA(cudaStreamSynchronize(c.stream));
    c.d2h += bytes;
    return CF_OK;
}

int cf_enqueue(cf_context* ctx, const char* modelId, const char* productId, const cf_num_param* num, int risk,
               const double* weights, int* launches)
{
    CF_CTX();
    if (!num) return fail(CF_E_ARG, "null argument");
    Plan* plan;
    int rc = ctx->c.getPlan(modelId ? modelId : "", productId ? productId : "", plan);
    if (rc) return rc;
    std::vector<double> w;
    if (risk && !weights)
    {
        w.assign(plan->nPay, 0.0);
        w[0] = 1.0;
        weights = w.data();
    }
    if ((rc = ctx->c.enqueue(*plan, *num, risk != 0, weights))) return rc;
    if (launches) *launches = ctx->c.main.launches;
    return CF_OK;
}

int cf_fetch_result(cf_context* ctx, double* values, double* stderrs, double* aggregate, double* risks)
{
    CF_CTX();
    return ctx->c.fetch(values, stderrs, aggregate, risks);
}

int cf_enqueue_shard(cf_context* ctx, const char* modelId, const char* productId, const cf_num_param* num,
                     int64_t firstPath, int risk, const double* weights, int* launches)
{
    CF_CTX();
    if (!num) return fail(CF_E_ARG, "null argument");
    Plan* plan;
    int rc = ctx->c.getPlan(modelId ? modelId : "", productId ? productId : "", plan);
    if (rc) return rc;
    // a shard's raw accumulators carry parameter adjoints for the single-asset models; the
    // multi-asset model's are adjoints of its derived quantities (mapped in fetch)
    if (risk && plan->model == MODEL_MULTI)
        return fail(CF_E_UNSUPPORTED, "sharded risk runs cover the Black-Scholes and Dupire models");
    std::vector<double> w;
    if (risk && !weights)
    {
        w.assign(plan->nPay, 0.0);
        w[0] = 1.0;
        weights = w.data();
    }
    ctx->c.main.stream = ctx->c.stream;
    if ((rc = ctx->c.enqueue(ctx->c.main, *plan, *num, risk != 0, weights, (long long)firstPath))) return rc;
    if (launches) *launches = ctx->c.main.launches;
    return CF_OK;
}

int cf_fetch_raw(cf_context* ctx, int64_t* acc, int capacity, int* nWords)
{
    CF_CTX();
    Slot& slot = ctx->c.main;
    if (!slot.plan || slot.multi) return fail(CF_E_ARG, "no value or risk run enqueued");
    CF_CUDA(cudaEventSynchronize(slot.done));
    const McParams& p = slot.last;
    const long long* h = static_cast<const long long*>(slot.hostAcc.ptr);
    if (*reinterpret_cast<const int*>(h + 2 * size_t(p.nAcc))) return fail(CF_E_DEVICE, "kernel error flag");
    if (nWords) *nWords = 2 * p.nAcc;
    if (acc)
    {
        if (capacity < 2 * p.nAcc) return fail(CF_E_ARG, "accumulator buffer too small");
        std::memcpy(acc, h, size_t(p.nAcc) * 16);
    }
    return CF_OK;
}

int cf_results_from_raw(const int64_t* acc, int nRisk, int nPay, int64_t nPath, double* values, double* stderrs,
                        double* aggregate, double* risks)
{
    if (!acc || nRisk < 0 || nPay < 1 || nPath < 1) return fail(CF_E_ARG, "bad accumulators");
    results_from_acc(reinterpret_cast<const long long*>(acc), nRisk, nPay, (long long)nPath, values, stderrs,
                     aggregate, risks);
    return CF_OK;
}

int cf_sobol_points(cf_context* ctx, int dim, int64_t firstPath, int nPaths, uint32_t* out)
{
    CF_CTX();
    if (dim < 1 || dim > sobol_max_dim() || nPaths < 0 || firstPath < 0 || !out)
        return fail(CF_E_ARG, "sobol: bad dimension or range");
    const auto dirs = sobol_dirs(dim);
    DevBuf d, o;
    int rc;
    if ((rc = d.ensure(dirs.size() * 4)) || (rc = o.ensure(size_t(nPaths) * dim * 4 + 4))) return rc;
    CF_CUDA(cudaMemcpyAsync(d.ptr, dirs.data(), dirs.size() * 4, cudaMemcpyHostToDevice, ctx->c.stream));
    rc = launch_sobol_points((const unsigned*)d.ptr, dim, firstPath, nPaths, (unsigned*)o.ptr, ctx->c.stream);
    if (rc) return cuda_fail(cudaError_t(rc), "sobol_points");
    CF_CUDA(cudaMemcpyAsync(out, o.ptr, size_t(nPaths) * dim * 4, cudaMemcpyDeviceToHost, ctx->c.stream));
    CF_CUDA(cudaStreamSynchronize(ctx->c.stream));
    d.release();
    o.release();
    return CF_OK;
}

int cf_mrg_state(cf_context* ctx, unsigned seed1, unsigned seed2, int dim, int64_t firstPath, uint32_t* state6)
{
    CF_CTX();
    if (dim < 1 || firstPath < 0 || !state6) return fail(CF_E_ARG, "mrg: bad argument");
    DevBuf o;
    int rc;
    if ((rc = o.ensure(32))) return rc;
    rc = launch_mrg_state(ctx->c.jumpA, ctx->c.jumpB, seed1, seed2, (unsigned long long)(firstPath / 2) * dim,
                          (unsigned*)o.ptr, ctx->c.stream);
    if (rc) return cuda_fail(cudaError_t(rc), "mrg_state");
    CF_CUDA(cudaMemcpyAsync(state6, o.ptr, 24, cudaMemcpyDeviceToHost, ctx->c.stream));
    CF_CUDA(cudaStreamSynchronize(ctx->c.stream));
    o.release();
    return CF_OK;
}

namespace {
int rng_draws(cf_context* ctx, int uniform, int useSobol, unsigned seed1, unsigned seed2, int dim, int64_t firstPath,
              int nPaths, double* out)
{
    if (dim < 1 || nPaths < 0 || firstPath < 0 || !out || (useSobol && dim > sobol_max_dim()))
        return fail(CF_E_ARG, uniform ? "uniforms: bad argument" : "gaussians: bad argument");
    DevBuf d, o;
    int rc;
    std::vector<uint32_t> dirs = useSobol ? sobol_dirs(dim) : std::vector<uint32_t>(1);
    if ((rc = d.ensure(dirs.size() * 4)) || (rc = o.ensure(size_t(nPaths) * dim * 8 + 8))) return rc;
    CF_CUDA(cudaMemcpyAsync(d.ptr, dirs.data(), dirs.size() * 4, cudaMemcpyHostToDevice, ctx->c.stream));
    rc = launch_gauss(useSobol, uniform, (const unsigned*)d.ptr, ctx->c.jumpA, ctx->c.jumpB, seed1, seed2, dim,
                      firstPath, nPaths, (double*)o.ptr, ctx->c.stream);
    if (rc) return cuda_fail(cudaError_t(rc), uniform ? "uniforms" : "gaussians");
    CF_CUDA(cudaMemcpyAsync(out, o.ptr, size_t(nPaths) * dim * 8, cudaMemcpyDeviceToHost, ctx->c.stream));
    CF_CUDA(cudaStreamSynchronize(ctx->c.stream));
    d.release();
    o.release();
    return CF_OK;
}
}  // namespace

int cf_gaussians(cf_context* ctx, int useSobol, unsigned seed1, unsigned seed2, int dim, int64_t firstPath, int nPaths,
                 double* out)
{
    CF_CTX();
    return rng_draws(ctx, 0, useSobol, seed1, seed2, dim, firstPath, nPaths, out);
}

int cf_uniforms(cf_context* ctx, int useSobol, unsigned seed1, unsigned seed2, int dim, int64_t firstPath, int nPaths,
                double* out)
{
    CF_CTX();
    return rng_draws(ctx, 1, useSobol, seed1, seed2, dim, firstPath, nPaths, out);
}

int cf_model_sim_dim(cf_context* ctx, const char* modelId, const double* productTimeline, int n, int* simDim)
{
    CF_CTX();
    if (!modelId || !simDim || n < 1 || !productTimeline) return fail(CF_E_ARG, "simDim: bad argument");
    const auto it = ctx->c.models.find(modelId);
    if (it == ctx->c.models.end()) return fail(CF_E_NOTFOUND, "simDim: model not found");
    const ModelDesc& m = it->second;
    const std::vector<double> tl(productTimeline, productTimeline + n);
    if (m.kind == MODEL_BS)  // mcMdlBS.h:149-195, 280-283: one step per product date after today
        *simDim = int(std::count_if(tl.begin(), tl.end(), [](double t) { return t > 0.0; }));
    else if (m.kind == MODEL_DUPIRE)  // mcMdlDupire.h:165-193, 220-223: the refined timeline's steps
        *simDim = int(fill_data(tl, m.maxDt, kHalfDay, {0.0}).size()) - 1;
    else
        return fail(CF_E_UNSUPPORTED, "simDim: multi-asset models take their dimension from a product");
    return CF_OK;
}

int cf_product_events(cf_context* ctx, const char* productId, double* times, int* needNumeraire, double* forwardMats,
                      double* discountMats, double* liborEnds, int capacity, int* count)
{
    CF_CTX();
    if (!productId || !count) return fail(CF_E_ARG, "product events: null argument");
    const auto it = ctx->c.products.find(productId);
    if (it == ctx->c.products.end()) return fail(CF_E_NOTFOUND, "product events: product not found");
    const ProductDesc& pd = it->second;
    const int n = int(pd.timeline.size());
    *count = n;
    if (!times) return CF_OK;
    if (capacity < n) return fail(CF_E_SHAPE, "product events: capacity too small");
    for (int e = 0; e < n; ++e)
    {
        times[e] = pd.timeline[e];
        if (needNumeraire) needNumeraire[e] = pd.needNum[e];
        if (forwardMats) forwardMats[e] = e < int(pd.fwdMat.size()) ? pd.fwdMat[e] : NAN;
        if (discountMats) discountMats[e] = e < int(pd.discMat.size()) ? pd.discMat[e] : NAN;
        if (liborEnds) liborEnds[e] = e < int(pd.libEnd.size()) ? pd.libEnd[e] : NAN;
    }
    return CF_OK;
}

}  // extern "C"
