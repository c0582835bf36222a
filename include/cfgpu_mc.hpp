// cfgpu_mc.hpp -- C++17 drop-in for CompFinance's model / product / RNG objects and the
// simulators that take them (mcBase.h:40-989), on the C ABI of libcfgpu.so (cfgpu.h).
//
// Callers that build objects and call the simulators directly, e.g.
//
//     Dupire<double> mdl(spot, spots, times, vols, maxDt);
//     UOC<double> prd(120, 150, 3, 1.0 / 52, 0.01);
//     mrg32k3a rng(12345, 1234);
//     auto paths = mcSimul(prd, mdl, rng, nPath);                 // [nPath][nPay]
//     auto aad = mcSimulAAD(prdN, mdlN, rng, nPath);              // payoffs, aggregated, risks
//
// keep their source: the class shapes (Product<T>, Model<T>, RNG, Sample<T>, Scenario<T>,
// SampleDef), the concrete types' constructors, the simulators' signatures and result structs
// are the reference's.  What differs is where the work runs: every path is simulated and
// differentiated on the GPU (the hand-written adjoint kernels replace the tape), so
//  * the objects are descriptions: each lowers itself into the engine's store when a
//    simulator runs (lower()), reading its current parameters (Model::parameters() points at
//    them, as in the reference);
//  * Model::generatePath and Product::payoffs (the per-path virtual calls of mcBase.h:297-305)
//    are not part of these shapes: there is no host path loop;
//  * Number is a value type with the arithmetic an aggregator needs, not a tape node;
//    mcSimulAAD accepts affine aggregators of the payoffs (the reference's default and the
//    notional-weighted ones of main.h:176-254) and throws for others;
//  * the concrete types are the engine's: BlackScholes, Dupire; European, UOC, Europeans,
//    ContingentBond; mrg32k3a, Sobol.
// The simulators take an optional precision (CF_FP64, the parity form, by default; CF_FP32).
#pragma once

#include <algorithm>
#include <cmath>
#include <map>
#include <memory>
#include <numeric>
#include <random>
#include <stdexcept>
#include <string>
#include <vector>

#include "cfgpu.hpp"

namespace cfgpu {

using Time = double;

// ---- scenarios, mcBase.h:40-117 --------------------------------------------------------
struct SampleDef
{
    bool numeraire = true;
    struct RateDef
    {
        Time start;
        Time end;
        std::string curve;
        RateDef(const Time s, const Time e, const std::string& c) : start(s), end(e), curve(c) {}
    };
    std::vector<Time> discountMats;
    std::vector<RateDef> liborDefs;
    std::vector<std::vector<Time>> forwardMats;  // [asset][maturity]
};

template <class T>
struct Sample
{
    T numeraire;
    std::vector<T> discounts;
    std::vector<T> libors;
    std::vector<std::vector<T>> forwards;
    void allocate(const SampleDef& data)
    {
        discounts.resize(data.discountMats.size());
        libors.resize(data.liborDefs.size());
        forwards.resize(data.forwardMats.size());
        for (size_t a = 0; a < forwards.size(); ++a) forwards[a].resize(data.forwardMats[a].size());
    }
    void initialize()
    {
        numeraire = T(1.0);
        std::fill(discounts.begin(), discounts.end(), T(1.0));
        std::fill(libors.begin(), libors.end(), T(0.0));
        for (auto& f : forwards) std::fill(f.begin(), f.end(), T(100.0));
    }
};

template <class T>
using Scenario = std::vector<Sample<T>>;

template <class T>
inline void allocatePath(const std::vector<SampleDef>& defline, Scenario<T>& path)
{
    path.resize(defline.size());
    for (size_t i = 0; i < defline.size(); ++i) path[i].allocate(defline[i]);
}

template <class T>
inline void initializePath(Scenario<T>& path)
{
    for (auto& s : path) s.initialize();
}

// ---- Number ------------------------------------------------------------------------------
// The value type of the AAD instantiations (Model<Number>, Product<Number>, aggregators).  The
// engine's adjoint kernels replace the tape, so a Number carries a value only.
class Number
{
    double myValue = 0.0;

public:
    Number() = default;
    Number(double v) : myValue(v) {}
    double value() const { return myValue; }
    double& value() { return myValue; }
    explicit operator double() const { return myValue; }
    Number& operator+=(const Number& o) { myValue += o.myValue; return *this; }
    Number& operator-=(const Number& o) { myValue -= o.myValue; return *this; }
    Number& operator*=(const Number& o) { myValue *= o.myValue; return *this; }
    Number& operator/=(const Number& o) { myValue /= o.myValue; return *this; }
    friend Number operator+(Number a, const Number& b) { return a += b; }
    friend Number operator-(Number a, const Number& b) { return a -= b; }
    friend Number operator*(Number a, const Number& b) { return a *= b; }
    friend Number operator/(Number a, const Number& b) { return a /= b; }
    friend Number operator-(const Number& a) { return Number(-a.myValue); }
    friend bool operator<(const Number& a, const Number& b) { return a.myValue < b.myValue; }
    friend bool operator>(const Number& a, const Number& b) { return a.myValue > b.myValue; }
    friend bool operator==(const Number& a, const Number& b) { return a.myValue == b.myValue; }
};

namespace detail {
inline double val(double x) { return x; }
inline double val(const Number& x) { return x.value(); }

inline std::string newId(const char* kind)
{
    static unsigned long long counter = 0;
    return std::string("\x02") + kind + std::to_string(++counter);
}

inline const std::vector<std::string>& spotName()
{
    static const std::vector<std::string> n = {"spot"};
    return n;
}
}  // namespace detail

// ---- products, mcBase.h:122-152 ----------------------------------------------------------
template <class T>
class Product
{
    mutable std::string myStoreId;

public:
    Product() = default;
    Product(const Product&) {}  // a copy is a product of its own: it gets its own store id
    Product& operator=(const Product&) { return *this; }
    // The id under which lower() puts this product into the engine's store (one per object).
    const std::string& storeId() const
    {
        if (myStoreId.empty()) myStoreId = detail::newId("prd");
        return myStoreId;
    }
    virtual const std::vector<Time>& timeline() const = 0;
    virtual const std::vector<SampleDef>& defline() const = 0;
    virtual const size_t numAssets() const { return 1; }
    virtual const std::vector<std::string>& assetNames() const { return detail::spotName(); }
    virtual const std::vector<std::string>& payoffLabels() const = 0;
    virtual std::unique_ptr<Product<T>> clone() const = 0;
    virtual ~Product() {}
    // The device form (no counterpart in the reference): puts this product into the engine's
    // store under `id`.
    virtual void lower(const std::string& id) const = 0;
};

// The engine-side half of the concrete products: timeline, defline and labels read back from the
// store (the engine builds them by the reference's rules, mcPrd.h).
template <class T>
class StoredProduct : public Product<T>
{
    mutable std::vector<Time> myTimeline;
    mutable std::vector<SampleDef> myDefline;
    mutable std::vector<std::string> myLabels;
    mutable bool myReady = false;

    void ready() const
    {
        if (myReady) return;
        const std::string& myId = this->storeId();
        this->lower(myId);
        int n = 0;
        detail::check(cf_product_events(detail::ctx(), myId.c_str(), nullptr, nullptr, nullptr, nullptr, nullptr, 0, &n),
                      "Product::timeline()");
        std::vector<double> t(n), fm(n), dm(n), le(n);
        std::vector<int> nn(n);
        detail::check(cf_product_events(detail::ctx(), myId.c_str(), t.data(), nn.data(), fm.data(), dm.data(), le.data(),
                                        n, &n),
                      "Product::defline()");
        myTimeline = t;
        myDefline.assign(n, SampleDef());
        for (int e = 0; e < n; ++e)
        {
            myDefline[e].numeraire = nn[e] != 0;
            if (!std::isnan(dm[e])) myDefline[e].discountMats.push_back(dm[e]);
            if (!std::isnan(le[e])) myDefline[e].liborDefs.emplace_back(t[e], le[e], "libor");
            if (!std::isnan(fm[e])) myDefline[e].forwardMats.push_back({fm[e]});
        }
        myLabels = getPayoffLabels(myId);
        myReady = true;
    }

public:
    const std::vector<Time>& timeline() const override { ready(); return myTimeline; }
    const std::vector<SampleDef>& defline() const override { ready(); return myDefline; }
    const std::vector<std::string>& payoffLabels() const override { ready(); return myLabels; }
};

// European, mcPrd.h:29-126
template <class T>
class European : public StoredProduct<T>
{
    double myStrike;
    Time myExerciseDate, mySettlementDate;

public:
    European(const double strike, const Time exerciseDate, const Time settlementDate)
        : myStrike(strike), myExerciseDate(exerciseDate), mySettlementDate(settlementDate) {}
    European(const double strike, const Time exerciseDate) : European(strike, exerciseDate, exerciseDate) {}
    std::unique_ptr<Product<T>> clone() const override { return std::make_unique<European<T>>(*this); }
    void lower(const std::string& id) const override { putEuropean(myStrike, myExerciseDate, mySettlementDate, id); }
};

// UOC (smoothed up-and-out), mcPrd.h:128-289
template <class T>
class UOC : public StoredProduct<T>
{
    double myStrike, myBarrier;
    Time myMaturity, myMonitorFreq;
    double mySmooth;
    bool myCallPut;

public:
    UOC(const double strike, const double barrier, const Time maturity, const Time monitorFreq, const double smooth,
        const bool callPut = false)
        : myStrike(strike), myBarrier(barrier), myMaturity(maturity), myMonitorFreq(monitorFreq), mySmooth(smooth),
          myCallPut(callPut) {}
    std::unique_ptr<Product<T>> clone() const override { return std::make_unique<UOC<T>>(*this); }
    void lower(const std::string& id) const override
    {
        putBarrier(myStrike, myBarrier, myMaturity, myMonitorFreq, mySmooth, myCallPut, id);
    }
};

// Europeans (portfolio of calls by maturity), mcPrd.h:291-400
template <class T>
class Europeans : public StoredProduct<T>
{
    std::map<Time, std::vector<double>> myOptions;

public:
    Europeans(const std::map<Time, std::vector<double>>& options) : myOptions(options) {}
    std::unique_ptr<Product<T>> clone() const override { return std::make_unique<Europeans<T>>(*this); }
    void lower(const std::string& id) const override
    {
        std::vector<double> mats, strikes;
        for (const auto& o : myOptions)
            for (double k : o.second)
            {
                mats.push_back(o.first);
                strikes.push_back(k);
            }
        putEuropeans(mats, strikes, id);
    }
};

// ContingentBond, mcPrd.h:404-574
template <class T>
class ContingentBond : public StoredProduct<T>
{
    Time myMaturity;
    double myCpn;
    Time myPayFreq;
    double mySmooth;

public:
    ContingentBond(const Time maturity, const double cpn, const Time payFreq, const double smooth)
        : myMaturity(maturity), myCpn(cpn), myPayFreq(payFreq), mySmooth(smooth) {}
    std::unique_ptr<Product<T>> clone() const override { return std::make_unique<ContingentBond<T>>(*this); }
    void lower(const std::string& id) const override { putContingent(myCpn, myMaturity, myPayFreq, mySmooth, id); }
};

// ---- models, mcBase.h:157-223 ------------------------------------------------------------
template <class T>
class Model
{
    mutable std::string myStoreId;

public:
    Model() = default;
    Model(const Model&) {}  // a copy (a bumped clone, say) is a model of its own: its own store id
    Model& operator=(const Model&) { return *this; }
    // The id under which lower() puts this model into the engine's store (one per object).
    const std::string& storeId() const
    {
        if (myStoreId.empty()) myStoreId = detail::newId("mdl");
        return myStoreId;
    }
    virtual const size_t numAssets() const { return 1; }
    virtual const std::vector<std::string>& assetNames() const { return detail::spotName(); }
    // The product's timeline; the engine simulates on the model's refinement of it.
    virtual void allocate(const std::vector<Time>& prdTimeline, const std::vector<SampleDef>& prdDefline) = 0;
    virtual void init(const std::vector<Time>& prdTimeline, const std::vector<SampleDef>& prdDefline) = 0;
    virtual size_t simDim() const = 0;
    virtual std::unique_ptr<Model<T>> clone() const = 0;
    virtual ~Model() {}
    virtual const std::vector<T*>& parameters() = 0;
    virtual const std::vector<std::string>& parameterLabels() const = 0;
    size_t numParams() const { return const_cast<Model*>(this)->parameters().size(); }
    // The device form (no counterpart in the reference): puts this model, with its current
    // parameters, into the engine's store under `id`.
    virtual void lower(const std::string& id) const = 0;
};

template <class T>
class StoredModel : public Model<T>
{
    std::vector<Time> myPrdTimeline;
    mutable std::vector<std::string> myLabels;

public:
    void allocate(const std::vector<Time>& prdTimeline, const std::vector<SampleDef>&) override
    {
        myPrdTimeline = prdTimeline;
    }
    void init(const std::vector<Time>&, const std::vector<SampleDef>&) override {}
    size_t simDim() const override
    {
        if (myPrdTimeline.empty()) throw std::runtime_error("Model::simDim() : allocate() the model first");
        const std::string& id = this->storeId();
        this->lower(id);
        int d = 0;
        detail::check(cf_model_sim_dim(detail::ctx(), id.c_str(), myPrdTimeline.data(), int(myPrdTimeline.size()), &d),
                      "Model::simDim()");
        return size_t(d);
    }
    const std::vector<std::string>& parameterLabels() const override
    {
        if (myLabels.empty())
        {
            const std::string& id = this->storeId();
            this->lower(id);
            myLabels = getParameterLabels(id);
        }
        return myLabels;
    }
};

// BlackScholes, mcMdlBS.h:28-350: parameters spot, vol, rate, div
template <class T>
class BlackScholes : public StoredModel<T>
{
    T mySpot, myVol, myRate, myDiv;
    bool mySpotMeasure;
    std::vector<T*> myParameters;

public:
    template <class U>
    BlackScholes(const U spot, const U vol, const bool spotMeasure = false, const U rate = U(0.0), const U div = U(0.0))
        : mySpot(spot), myVol(vol), myRate(rate), myDiv(div), mySpotMeasure(spotMeasure),
          myParameters{&mySpot, &myVol, &myRate, &myDiv} {}
    BlackScholes(const BlackScholes& o)
        : StoredModel<T>(o), mySpot(o.mySpot), myVol(o.myVol), myRate(o.myRate), myDiv(o.myDiv),
          mySpotMeasure(o.mySpotMeasure), myParameters{&mySpot, &myVol, &myRate, &myDiv} {}
    std::unique_ptr<Model<T>> clone() const override { return std::make_unique<BlackScholes<T>>(*this); }
    const std::vector<T*>& parameters() override { return myParameters; }
    void lower(const std::string& id) const override
    {
        putBlackScholes(detail::val(mySpot), detail::val(myVol), mySpotMeasure, detail::val(myRate),
                        detail::val(myDiv), id);
    }
};

// Dupire, mcMdlDupire.h:29-280: parameters spot, then the local vols [spot][time]
template <class T>
class Dupire : public StoredModel<T>
{
    T mySpot;
    std::vector<double> mySpots;
    std::vector<Time> myTimes;
    matrix<T> myVols;
    Time myMaxDt;
    std::vector<T*> myParameters;

    void link()
    {
        myParameters.assign(1, &mySpot);
        for (auto& v : myVols.v) myParameters.push_back(&v);
    }

public:
    template <class U>
    Dupire(const U spot, const std::vector<double> spots, const std::vector<Time> times, const matrix<U> vols,
           const Time maxDt = 0.25)
        : mySpot(spot), mySpots(spots), myTimes(times), myVols(vols.rows(), vols.cols()), myMaxDt(maxDt)
    {
        if (vols.rows() != spots.size() || vols.cols() != times.size())
            throw std::runtime_error("Dupire() : vols must be spots x times");
        std::copy(vols.v.begin(), vols.v.end(), myVols.v.begin());
        link();
    }
    Dupire(const Dupire& o)
        : StoredModel<T>(o), mySpot(o.mySpot), mySpots(o.mySpots), myTimes(o.myTimes), myVols(o.myVols),
          myMaxDt(o.myMaxDt)
    {
        link();
    }
    const std::vector<double>& spots() const { return mySpots; }
    const std::vector<Time>& times() const { return myTimes; }
    const matrix<T>& vols() const { return myVols; }
    std::unique_ptr<Model<T>> clone() const override { return std::make_unique<Dupire<T>>(*this); }
    const std::vector<T*>& parameters() override { return myParameters; }
    void lower(const std::string& id) const override
    {
        matrix<double> v(myVols.rows(), myVols.cols());
        for (size_t k = 0; k < v.v.size(); ++k) v.v[k] = detail::val(myVols.v[k]);
        putDupire(detail::val(mySpot), mySpots, myTimes, v, myMaxDt, id);
    }
};

// ---- random number generators, mcBase.h:228-246 --------------------------------------------
// The device generators (sobol.h, mrg32k3a.h): the simulators run them on the GPU from path 0,
// as the reference's clone + init does.  nextU / nextG return the vectors of consecutive paths,
// computed on the device; skipTo(b) moves to path b.
class RNG
{
public:
    virtual void init(const size_t simDim) = 0;
    virtual void nextU(std::vector<double>& uVec) = 0;
    virtual void nextG(std::vector<double>& gaussVec) = 0;
    virtual std::unique_ptr<RNG> clone() const = 0;
    virtual ~RNG() {}
    virtual void skipTo(const unsigned b) = 0;
    // The device form (no counterpart in the reference)
    virtual bool sobol() const = 0;
    virtual unsigned seed1() const { return 0; }
    virtual unsigned seed2() const { return 0; }
};

class DeviceRNG : public RNG
{
protected:
    size_t myDim = 0;
    long long myPath = 0;

    void draw(int uniform, std::vector<double>& out)
    {
        if (!myDim) throw std::runtime_error("RNG : init() the generator first");
        if (out.size() < myDim) out.resize(myDim);
        auto fn = uniform ? cf_uniforms : cf_gaussians;
        detail::check(fn(detail::ctx(), sobol() ? 1 : 0, seed1(), seed2(), int(myDim), myPath, 1, out.data()),
                      uniform ? "RNG::nextU()" : "RNG::nextG()");
        ++myPath;
    }

public:
    void init(const size_t simDim) override
    {
        myDim = simDim;
        myPath = 0;
    }
    void nextU(std::vector<double>& uVec) override { draw(1, uVec); }
    void nextG(std::vector<double>& gaussVec) override { draw(0, gaussVec); }
    void skipTo(const unsigned b) override { myPath = b; }
};

// mrg32k3a, mrg32k3a.h:25-394 (antithetic: the second path of each pair negates the first)
class mrg32k3a : public DeviceRNG
{
    unsigned myA, myB;

public:
    mrg32k3a(const unsigned a = 12345, const unsigned b = 12346) : myA(a), myB(b) {}
    std::unique_ptr<RNG> clone() const override { return std::make_unique<mrg32k3a>(*this); }
    bool sobol() const override { return false; }
    unsigned seed1() const override { return myA; }
    unsigned seed2() const override { return myB; }
};

// Sobol, sobol.h:30-152
class Sobol : public DeviceRNG
{
public:
    std::unique_ptr<RNG> clone() const override { return std::make_unique<Sobol>(*this); }
    bool sobol() const override { return true; }
};

// ---- simulators, mcBase.h:249-989 ----------------------------------------------------------
template <class T>
inline bool checkCompatiblity(const Product<T>& prd, const Model<T>& mdl)
{
    return prd.assetNames() == mdl.assetNames();
}

namespace detail {
template <class T>
struct Lowered
{
    std::string mid, pid;
    cf_num_param num;
    int nPay, nParam;
    Lowered(const Product<T>& prd, const Model<T>& mdl, const RNG& rng, size_t nPath, int precision)
    {
        if (!checkCompatiblity(prd, mdl)) throw std::runtime_error("Model and product are not compatible");
        if (nPath < 1 || nPath > size_t(0x7fffffff)) throw std::runtime_error("mcSimul : bad number of paths");
        mid = mdl.storeId();
        pid = prd.storeId();
        mdl.lower(mid);  // with the model's current parameters
        prd.lower(pid);
        num = cf_num_param{1, rng.sobol() ? 1 : 0, int(nPath), int(rng.seed1()), int(rng.seed2()), precision};
        int dim = 0;
        check(cf_shapes(ctx(), mid.c_str(), pid.c_str(), &nPay, &nParam, &dim), "mcSimul()");
    }
    std::vector<std::vector<double>> paths() const
    {
        std::vector<double> flat(size_t(num.numPath) * size_t(nPay));
        check(cf_simulate_paths(ctx(), mid.c_str(), pid.c_str(), &num, flat.data()), "mcSimul()");
        std::vector<std::vector<double>> out(size_t(num.numPath), std::vector<double>(size_t(nPay)));
        for (size_t i = 0; i < out.size(); ++i)
            std::copy(flat.begin() + i * nPay, flat.begin() + (i + 1) * nPay, out[i].begin());
        return out;
    }
};

// The weights w and constant c of an affine aggregator, f(v) = c + w.v, read off f at 0 and at
// the unit vectors, and checked on a seeded random vector.
template <class F>
inline std::vector<double> affineWeights(const F& aggFun, size_t nPay, double& c)
{
    std::vector<Number> v(nPay, Number(0.0));
    c = val(aggFun(v));
    std::vector<double> w(nPay);
    for (size_t k = 0; k < nPay; ++k)
    {
        v[k] = Number(1.0);
        w[k] = val(aggFun(v)) - c;
        v[k] = Number(0.0);
    }
    std::mt19937_64 gen(20181);
    std::uniform_real_distribution<double> U(-1.0, 1.0);
    double lin = c, scale = std::fabs(c);
    for (size_t k = 0; k < nPay; ++k)
    {
        const double r = U(gen);
        v[k] = Number(r);
        lin += w[k] * r;
        scale += std::fabs(w[k] * r);
    }
    if (std::fabs(val(aggFun(v)) - lin) > 1e-12 * std::max(scale, 1.0))
        throw std::runtime_error("mcSimulAAD() : the aggregator must be an affine function of the payoffs "
                                 "(the device adjoint is taken of a weighted sum)");
    return w;
}
}  // namespace detail

// mcSimul / mcParallelSimul, mcBase.h:267-400: the payoffs of every path [nPath][nPay]
inline std::vector<std::vector<double>> mcSimul(const Product<double>& prd, const Model<double>& mdl, const RNG& rng,
                                                const size_t nPath, int precision = CF_FP64)
{
    return detail::Lowered<double>(prd, mdl, rng, nPath, precision).paths();
}

inline std::vector<std::vector<double>> mcParallelSimul(const Product<double>& prd, const Model<double>& mdl,
                                                        const RNG& rng, const size_t nPath, int precision = CF_FP64)
{
    return mcSimul(prd, mdl, rng, nPath, precision);
}

// AADSimulResults, mcBase.h:405-422
struct AADSimulResults
{
    AADSimulResults(const size_t nPath, const size_t nPay, const size_t nParam)
        : payoffs(nPath, std::vector<double>(nPay)), aggregated(nPath), risks(nParam) {}
    std::vector<std::vector<double>> payoffs;  // [nPath][nPay]
    std::vector<double> aggregated;            // [nPath]
    std::vector<double> risks;                 // [nParam], of the aggregate, averaged over paths
};

const auto defaultAggregator = [](const std::vector<Number>& v) { return v[0]; };

// mcSimulAAD / mcParallelSimulAAD, mcBase.h:427-753, for affine aggregators (see the header
// comment); payoffs and aggregated from the valuation kernel on the same random numbers.
template <class F = decltype(defaultAggregator)>
inline AADSimulResults mcSimulAAD(const Product<Number>& prd, const Model<Number>& mdl, const RNG& rng,
                                  const size_t nPath, const F& aggFun = defaultAggregator, int precision = CF_FP64)
{
    const detail::Lowered<Number> L(prd, mdl, rng, nPath, precision);
    double c = 0.0;
    const std::vector<double> w = detail::affineWeights(aggFun, size_t(L.nPay), c);
    AADSimulResults r(nPath, size_t(L.nPay), size_t(L.nParam));
    std::vector<double> values(L.nPay);
    double agg = 0.0;
    detail::check(cf_aad_risk_aggregate(detail::ctx(), L.mid.c_str(), L.pid.c_str(), w.data(), &L.num, values.data(),
                                        &agg, r.risks.data()),
                  "mcSimulAAD()");
    r.payoffs = L.paths();
    for (size_t i = 0; i < nPath; ++i)
    {
        double a = c;
        for (int k = 0; k < L.nPay; ++k) a += w[k] * r.payoffs[i][k];
        r.aggregated[i] = a;
    }
    return r;
}

template <class F = decltype(defaultAggregator)>
inline AADSimulResults mcParallelSimulAAD(const Product<Number>& prd, const Model<Number>& mdl, const RNG& rng,
                                          const size_t nPath, const F& aggFun = defaultAggregator,
                                          int precision = CF_FP64)
{
    return mcSimulAAD(prd, mdl, rng, nPath, aggFun, precision);
}

// AADMultiSimulResults, mcBase.h:758-771
struct AADMultiSimulResults
{
    AADMultiSimulResults(const size_t nPath, const size_t nPay, const size_t nParam)
        : payoffs(nPath, std::vector<double>(nPay)), risks(nParam, nPay) {}
    std::vector<std::vector<double>> payoffs;  // [nPath][nPay]
    matrix<double> risks;                      // [nParam][nPay], averaged over paths
};

// mcSimulAADMulti / mcParallelSimulAADMulti, mcBase.h:775-989
inline AADMultiSimulResults mcSimulAADMulti(const Product<Number>& prd, const Model<Number>& mdl, const RNG& rng,
                                            const size_t nPath, int precision = CF_FP64)
{
    const detail::Lowered<Number> L(prd, mdl, rng, nPath, precision);
    AADMultiSimulResults r(nPath, size_t(L.nPay), size_t(L.nParam));
    std::vector<double> values(L.nPay);
    detail::check(cf_aad_risk_multi(detail::ctx(), L.mid.c_str(), L.pid.c_str(), &L.num, values.data(),
                                    r.risks.v.data()),
                  "mcSimulAADMulti()");
    r.payoffs = L.paths();
    return r;
}

inline AADMultiSimulResults mcParallelSimulAADMulti(const Product<Number>& prd, const Model<Number>& mdl,
                                                    const RNG& rng, const size_t nPath, int precision = CF_FP64)
{
    return mcSimulAADMulti(prd, mdl, rng, nPath, precision);
}

}  // namespace cfgpu
