// cfgpu.hpp -- C++17 drop-in for CompFinance's main.h / store.h entry points, on the C ABI
// of libcfgpu.so (cfgpu.h).
//
// Source-compatible with the reference's callers of main.h (xlExport.cpp-style code):
//   putBlackScholes / putDupire / putEuropean / putBarrier / putEuropeans   (store.h:38-205)
//   value / AADriskOne / AADriskAggregate / AADriskMulti                    (main.h:43-312)
//   dupireCalib / dupireSuperbucket                                         (main.h:414-569)
// with the same argument meaning, result members and std::runtime_error on failure.
// Models and products live on the GPU; `NumericalParam::parallel` is accepted and ignored.
// One process-wide context on device 0 (cfgpu::setDevice before the first call to change it).
#pragma once

#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "cfgpu.h"

namespace cfgpu {

// NumericalParam, main.h:33-40 (+ precision: CF_FP64 parity form or CF_FP32)
struct NumericalParam
{
    bool parallel = true;
    bool useSobol = false;
    int numPath = 0;
    int seed1 = 12345;
    int seed2 = 1234;
    int precision = CF_FP64;
};

// Row-major matrix with the reference's accessors (matrix.h:10-90).
template <class T>
struct matrix
{
    size_t myRows = 0, myCols = 0;
    std::vector<T> v;
    matrix() = default;
    matrix(size_t r, size_t c) : myRows(r), myCols(c), v(r * c) {}
    size_t rows() const { return myRows; }
    size_t cols() const { return myCols; }
    T* operator[](size_t r) { return &v[r * myCols]; }
    const T* operator[](size_t r) const { return &v[r * myCols]; }
    void resize(size_t r, size_t c) { myRows = r; myCols = c; v.assign(r * c, T()); }
    typename std::vector<T>::iterator begin() { return v.begin(); }
    typename std::vector<T>::iterator end() { return v.end(); }
};

namespace detail {

inline int& device()
{
    static int d = 0;
    return d;
}

inline std::string lastError()
{
    char buf[1024];
    cf_last_error(buf, sizeof buf);
    return buf;
}

inline void check(int rc, const char* where)
{
    if (rc != CF_OK) throw std::runtime_error(std::string(where) + " : " + lastError());
}

struct Ctx
{
    cf_context* h = nullptr;
    Ctx() { check(cf_create(device(), &h), "cfgpu context"); }
    ~Ctx() { cf_destroy(h); }
};

inline cf_context* ctx()
{
    static Ctx c;
    return c.h;
}

inline cf_num_param cnum(const NumericalParam& n)
{
    return cf_num_param{n.parallel ? 1 : 0, n.useSobol ? 1 : 0, n.numPath, n.seed1, n.seed2, n.precision};
}

inline std::vector<std::string> split(const std::string& s)
{
    std::vector<std::string> out;
    size_t a = 0;
    if (s.empty()) return out;
    while (true)
    {
        const size_t b = s.find('\n', a);
        out.push_back(s.substr(a, b == std::string::npos ? std::string::npos : b - a));
        if (b == std::string::npos) break;
        a = b + 1;
    }
    return out;
}

inline std::vector<std::string> labels(int (*fn)(cf_context*, const char*, char*, size_t, int*, size_t*),
                                       const std::string& id, const char* where)
{
    int n = 0;
    size_t need = 0;
    check(fn(ctx(), id.c_str(), nullptr, 0, &n, &need), where);
    std::string buf(need, '\0');
    check(fn(ctx(), id.c_str(), &buf[0], need, &n, &need), where);
    buf.resize(need ? need - 1 : 0);
    return split(buf);
}

struct Shapes
{
    int nPay, nParam, simDim;
};

inline Shapes shapes(const std::string& m, const std::string& p, const char* where)
{
    Shapes s{};
    check(cf_shapes(ctx(), m.c_str(), p.c_str(), &s.nPay, &s.nParam, &s.simDim), where);
    return s;
}

}  // namespace detail

inline void setDevice(int d) { detail::device() = d; }

// ---- store.h ---------------------------------------------------------------------------
inline void putBlackScholes(double spot, double vol, bool qSpot, double rate, double div, const std::string& store)
{
    detail::check(cf_put_black_scholes(detail::ctx(), spot, vol, qSpot ? 1 : 0, rate, div, store.c_str()),
                  "putBlackScholes()");
}

inline void putDupire(double spot, const std::vector<double>& spots, const std::vector<double>& times,
                      const matrix<double>& vols, double maxDt, const std::string& store)
{
    if (vols.rows() != spots.size() || vols.cols() != times.size())
        throw std::runtime_error("putDupire() : vols must be spots x times");
    detail::check(cf_put_dupire(detail::ctx(), spot, spots.data(), int(spots.size()), times.data(), int(times.size()),
                                vols.v.data(), maxDt, store.c_str()),
                  "putDupire()");
}

inline void putEuropean(double strike, double exerciseDate, double settlementDate, const std::string& store)
{
    detail::check(cf_put_european(detail::ctx(), strike, exerciseDate, settlementDate, store.c_str()), "putEuropean()");
}

inline void putBarrier(double strike, double barrier, double maturity, double monitorFreq, double smooth,
                       bool callPut, const std::string& store)
{
    detail::check(cf_put_barrier(detail::ctx(), strike, barrier, maturity, monitorFreq, smooth, callPut ? 1 : 0,
                                 store.c_str()),
                  "putBarrier()");
}

// store.h:165-180
inline void putContingent(double coupon, double maturity, double payFreq, double smooth, const std::string& store)
{
    detail::check(cf_put_contingent(detail::ctx(), coupon, maturity, payFreq, smooth, store.c_str()), "putContingent()");
}

inline void putEuropeans(const std::vector<double>& maturities, const std::vector<double>& strikes,
                         const std::string& store)
{
    if (maturities.size() != strikes.size()) throw std::runtime_error("putEuropeans() : size mismatch");
    detail::check(cf_put_europeans(detail::ctx(), maturities.data(), strikes.data(), int(maturities.size()),
                                   store.c_str()),
                  "putEuropeans()");
}

namespace detail {
inline std::vector<const char*> cnames(const std::vector<std::string>& v)
{
    std::vector<const char*> out;
    for (const auto& x : v) out.push_back(x.c_str());
    return out;
}
}  // namespace detail

// store.h:75-94 (MultiDisplaced): same arguments in the same order as the reference
inline void putDisplaced(const std::vector<std::string>& assets, const std::vector<double>& spots,
                         const std::vector<double>& atms, const std::vector<double>& skews, const double& discRate,
                         const std::vector<double>& repoSpreads, const std::vector<double>& divDates,
                         const matrix<double>& divs, const matrix<double>& correl, const double& lambda,
                         const std::string& store)
{
    const size_t n = assets.size();
    if (!n || spots.size() != n || atms.size() != n || skews.size() != n || repoSpreads.size() != n ||
        divs.rows() != divDates.size() || (divDates.size() && divs.cols() != n) || correl.rows() != n ||
        correl.cols() != n)
        throw std::runtime_error("putDisplaced() : inconsistent dimensions");
    const auto names = detail::cnames(assets);
    detail::check(cf_put_displaced(detail::ctx(), int(n), names.data(), spots.data(), atms.data(), skews.data(),
                                   discRate, repoSpreads.data(), int(divDates.size()), divDates.data(),
                                   divs.v.data(), correl.v.data(), lambda, store.c_str()),
                  "putDisplaced()");
}

// store.h:224-237
inline void putBaskets(const std::vector<std::string>& assets, const std::vector<double>& weights, double maturity,
                       const std::vector<double> strikes, const std::string& store)
{
    if (weights.size() != assets.size()) throw std::runtime_error("putBaskets() : one weight per asset");
    const auto names = detail::cnames(assets);
    detail::check(cf_put_baskets(detail::ctx(), int(assets.size()), names.data(), weights.data(), maturity,
                                 int(strikes.size()), strikes.data(), store.c_str()),
                  "putBaskets()");
}

// store.h:239-255
inline void putAutocall(const std::vector<std::string>& assets, const std::vector<double>& refs, double maturity,
                        int periods, double ko, double strike, double cpn, double smooth, const std::string& store)
{
    if (refs.size() != assets.size()) throw std::runtime_error("putAutocall() : one reference per asset");
    const auto names = detail::cnames(assets);
    detail::check(cf_put_autocall(detail::ctx(), int(assets.size()), names.data(), refs.data(), maturity, periods,
                                  ko, strike, cpn, smooth, store.c_str()),
                  "putAutocall()");
}

inline std::vector<std::string> getPayoffLabels(const std::string& productId)
{
    return detail::labels(cf_payoff_labels, productId, "getPayoffLabels()");
}

inline std::vector<std::string> getParameterLabels(const std::string& modelId)
{
    return detail::labels(cf_parameter_labels, modelId, "getModelParameters()");
}

// ---- main.h ----------------------------------------------------------------------------
struct ValueResults
{
    std::vector<std::string> identifiers;
    std::vector<double> values;
    std::vector<double> stderrs;  // Monte Carlo standard errors (not in the reference)
};

inline ValueResults value(const std::string& modelId, const std::string& productId, const NumericalParam& num)
{
    const auto s = detail::shapes(modelId, productId, "value() : Could not retrieve model and product");
    ValueResults r;
    r.values.resize(s.nPay);
    r.stderrs.resize(s.nPay);
    const cf_num_param n = detail::cnum(num);
    detail::check(cf_value(detail::ctx(), modelId.c_str(), productId.c_str(), &n, r.values.data(), r.stderrs.data()),
                  "value()");
    r.identifiers = getPayoffLabels(productId);
    return r;
}

struct RiskResults
{
    std::vector<std::string> payoffIds;
    std::vector<double> payoffValues;
    double riskPayoffValue = 0;
    std::vector<std::string> paramIds;
    std::vector<double> risks;
};

inline RiskResults AADriskOne(const std::string& modelId, const std::string& productId, const NumericalParam& num,
                              const std::string& riskPayoff = "")
{
    const auto s = detail::shapes(modelId, productId, "AADrisk() : Could not retrieve model and product");
    RiskResults r;
    r.payoffValues.resize(s.nPay);
    r.risks.resize(s.nParam);
    const cf_num_param n = detail::cnum(num);
    detail::check(cf_aad_risk_one(detail::ctx(), modelId.c_str(), productId.c_str(), &n, riskPayoff.c_str(),
                                  r.payoffValues.data(), &r.riskPayoffValue, r.risks.data()),
                  "AADriskOne()");
    r.payoffIds = getPayoffLabels(productId);
    r.paramIds = getParameterLabels(modelId);
    return r;
}

inline RiskResults AADriskAggregate(const std::string& modelId, const std::string& productId,
                                    const std::map<std::string, double>& notionals, const NumericalParam& num)
{
    const auto s = detail::shapes(modelId, productId, "AADriskAggregate() : Could not retrieve model and product");
    const auto labels = getPayoffLabels(productId);
    std::vector<double> w(s.nPay, 0.0);
    for (const auto& kv : notionals)
    {
        size_t k = 0;
        while (k < labels.size() && labels[k] != kv.first) ++k;
        if (k == labels.size()) throw std::runtime_error("AADriskAggregate() : payoff not found");
        w[k] = kv.second;
    }
    RiskResults r;
    r.payoffValues.resize(s.nPay);
    r.risks.resize(s.nParam);
    const cf_num_param n = detail::cnum(num);
    detail::check(cf_aad_risk_aggregate(detail::ctx(), modelId.c_str(), productId.c_str(), w.data(), &n,
                                        r.payoffValues.data(), &r.riskPayoffValue, r.risks.data()),
                  "AADriskAggregate()");
    r.payoffIds = labels;
    r.paramIds = getParameterLabels(modelId);
    return r;
}

// dupireAADRisk, main.h:364-411: AADriskAggregate of a Dupire model, split into the value,
// delta (risk to spot) and the vega matrix [spots][times] of the local-vol risks.
struct DupireRiskResults
{
    double value = 0;
    double delta = 0;
    matrix<double> vega;
};

inline DupireRiskResults dupireAADRisk(const std::string& modelId, const std::string& productId,
                                       const std::map<std::string, double>& notionals, const NumericalParam& num)
{
    int nS = 0, nT = 0;
    detail::check(cf_model_grid(detail::ctx(), modelId.c_str(), &nS, &nT, nullptr, nullptr), "dupireAADRisk()");
    const RiskResults agg = AADriskAggregate(modelId, productId, notionals, num);
    DupireRiskResults r;
    r.value = agg.riskPayoffValue;
    r.delta = agg.risks[0];
    r.vega.resize(size_t(nS), size_t(nT));
    std::copy(agg.risks.begin() + 1, agg.risks.end(), r.vega.begin());
    return r;
}

// RiskReports, main.h:260-266
struct RiskReports
{
    std::vector<std::string> payoffs;
    std::vector<std::string> params;
    std::vector<double> values;
    matrix<double> risks;  // params x payoffs
};

inline RiskReports AADriskMulti(const std::string& modelId, const std::string& productId, const NumericalParam& num)
{
    const auto s = detail::shapes(modelId, productId, "AADrisk() : Could not retrieve model and product");
    RiskReports r;
    r.values.resize(s.nPay);
    r.risks.resize(s.nParam, s.nPay);
    const cf_num_param n = detail::cnum(num);
    detail::check(cf_aad_risk_multi(detail::ctx(), modelId.c_str(), productId.c_str(), &n, r.values.data(),
                                    r.risks.v.data()),
                  "AADriskMulti()");
    r.payoffs = getPayoffLabels(productId);
    r.params = getParameterLabels(modelId);
    return r;
}

// bumpRisk, main.h:316-359: one-sided 1e-8 bumps of every parameter, repriced on the same
// random numbers (FP64), in the RiskReports layout.
inline RiskReports bumpRisk(const std::string& modelId, const std::string& productId, const NumericalParam& num)
{
    const auto s = detail::shapes(modelId, productId, "bumpRisk() : Could not retrieve model and product");
    RiskReports r;
    r.values.resize(s.nPay);
    r.risks.resize(size_t(s.nParam), size_t(s.nPay));
    const cf_num_param n = detail::cnum(num);
    detail::check(cf_bump_risk(detail::ctx(), modelId.c_str(), productId.c_str(), &n, CF_BUMP_AUTO, r.values.data(),
                               &*r.risks.begin()),
                  "bumpRisk()");
    r.payoffs = getPayoffLabels(productId);
    r.params = getParameterLabels(modelId);
    return r;
}

struct CalibResults
{
    std::vector<double> spots, times;
    matrix<double> lVols;  // spots x times
};

// dupireCalib (main.h:414-438): on a Merton implied surface, or any cf_ivs.
inline CalibResults dupireCalib(const std::vector<double>& inclSpots, double maxDs, const std::vector<double>& inclTimes,
                                double maxDt, const cf_ivs& ivs)
{
    CalibResults r;
    int nS = 0, nT = 0;
    detail::check(cf_dupire_calib(detail::ctx(), &ivs, inclSpots.data(), int(inclSpots.size()), maxDs, inclTimes.data(),
                                  int(inclTimes.size()), maxDt, &nS, &nT, nullptr, nullptr, nullptr),
                  "dupireCalib()");
    r.spots.resize(nS);
    r.times.resize(nT);
    r.lVols.resize(nS, nT);
    detail::check(cf_dupire_calib(detail::ctx(), &ivs, inclSpots.data(), int(inclSpots.size()), maxDs, inclTimes.data(),
                                  int(inclTimes.size()), maxDt, &nS, &nT, r.spots.data(), r.times.data(),
                                  r.lVols.v.data()),
                  "dupireCalib()");
    return r;
}

inline CalibResults dupireCalib(const std::vector<double>& inclSpots, double maxDs, const std::vector<double>& inclTimes,
                                double maxDt, double spot, double vol, double jmpIntens = 0.0, double jmpAverage = 0.0,
                                double jmpStd = 0.0)
{
    cf_ivs s{1, spot, {vol, jmpIntens, jmpAverage, jmpStd}};
    return dupireCalib(inclSpots, maxDs, inclTimes, maxDt, s);
}

// SuperbucketResults, main.h:442-449
struct SuperbucketResults
{
    double value = 0, delta = 0;
    std::vector<double> strikes, mats;
    matrix<double> vega;
};

inline SuperbucketResults dupireSuperbucketIvs(const cf_ivs& ivs, double maxDt, const std::string& productId,
                                               const std::map<std::string, double>& notionals,
                                               const std::vector<double>& inclSpots, double maxDs,
                                               const std::vector<double>& inclTimes, double maxDtVol,
                                               const std::vector<double>& strikes, const std::vector<double>& mats,
                                               const NumericalParam& num, bool referenceSeeding = false)
{
    const auto labels = getPayoffLabels(productId);
    std::vector<double> w(labels.size(), 0.0);
    for (const auto& kv : notionals)
    {
        size_t k = 0;
        while (k < labels.size() && labels[k] != kv.first) ++k;
        if (k == labels.size()) throw std::runtime_error("dupireSuperbucket() : payoff not found");
        w[k] = kv.second;
    }
    SuperbucketResults r;
    r.strikes = strikes;
    r.mats = mats;
    r.vega.resize(strikes.size(), mats.size());
    const cf_num_param n = detail::cnum(num);
    detail::check(cf_dupire_superbucket(detail::ctx(), &ivs, ivs.spot, maxDt, productId.c_str(), w.data(),
                                        inclSpots.data(), int(inclSpots.size()), maxDs, inclTimes.data(),
                                        int(inclTimes.size()), maxDtVol, strikes.data(), int(strikes.size()),
                                        mats.data(), int(mats.size()), &n, referenceSeeding ? 1 : 0, &r.value,
                                        &r.delta, r.vega.v.data(), nullptr),
                  "dupireSuperbucket()");
    return r;
}

// dupireSuperbucket with the reference's signature (main.h:453-473, Merton surface)
inline SuperbucketResults dupireSuperbucket(double spot, double maxDt, const std::string& productId,
                                            const std::map<std::string, double>& notionals,
                                            const std::vector<double>& inclSpots, double maxDs,
                                            const std::vector<double>& inclTimes, double maxDtVol,
                                            const std::vector<double>& strikes, const std::vector<double>& mats,
                                            double vol, double jmpIntens, double jmpAverage, double jmpStd,
                                            const NumericalParam& num)
{
    cf_ivs s{1, spot, {vol, jmpIntens, jmpAverage, jmpStd}};
    return dupireSuperbucketIvs(s, maxDt, productId, notionals, inclSpots, maxDs, inclTimes, maxDtVol, strikes, mats,
                                num);
}

// dupireSuperbucketBump, main.h:575-696 (Merton surface, the reference's signature): delta by
// the spot +1e-8, vega by each risk-view implied vol +1e-5, recalibrated and repriced.
inline SuperbucketResults dupireSuperbucketBump(double spot, double maxDt, const std::string& productId,
                                                const std::map<std::string, double>& notionals,
                                                const std::vector<double>& inclSpots, double maxDs,
                                                const std::vector<double>& inclTimes, double maxDtVol,
                                                const std::vector<double>& strikes, const std::vector<double>& mats,
                                                double vol, double jmpIntens, double jmpAverage, double jmpStd,
                                                const NumericalParam& num)
{
    const cf_ivs ivs{1, spot, {vol, jmpIntens, jmpAverage, jmpStd}};
    const auto labels = getPayoffLabels(productId);
    std::vector<double> w(labels.size(), 0.0);
    for (const auto& kv : notionals)
    {
        size_t k = 0;
        while (k < labels.size() && labels[k] != kv.first) ++k;
        if (k == labels.size()) throw std::runtime_error("dupireSuperbucketBump() : payoff not found");
        w[k] = kv.second;
    }
    SuperbucketResults r;
    r.strikes = strikes;
    r.mats = mats;
    r.vega.resize(strikes.size(), mats.size());
    const cf_num_param n = detail::cnum(num);
    detail::check(cf_dupire_superbucket_bump(detail::ctx(), &ivs, spot, maxDt, productId.c_str(), w.data(),
                                             inclSpots.data(), int(inclSpots.size()), maxDs, inclTimes.data(),
                                             int(inclTimes.size()), maxDtVol, strikes.data(), int(strikes.size()),
                                             mats.data(), int(mats.size()), &n, 0.0, &r.value, &r.delta,
                                             r.vega.v.data()),
                  "dupireSuperbucketBump()");
    return r;
}

}  // namespace cfgpu
