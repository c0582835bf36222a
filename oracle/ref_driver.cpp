// Command-driven harness around the reference's own entry points (main.h), used only
// to write golden fixtures and to pin the CPU restatement in oracle/oracle.cpp.
// Built by oracle/build_ref.py into oracle/_ref/ref_driver; reads commands on stdin and
// prints one line per result, doubles as C99 hex floats so nothing is lost in transit.
//
// Internal state of the reference classes (simulation timelines, RNG state words) is
// read through member pointers formed in explicit template instantiations, where access
// checking does not apply ([temp.spec]/6); nothing in the reference is modified for it.

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <functional>
#include <future>
#include <iomanip>
#include <iostream>
#include <map>
#include <memory>
#include <mutex>
#include <numeric>
#include <queue>
#include <sstream>
#include <string>
#include <thread>
#include <type_traits>
#include <unordered_map>
#include <vector>

#include "main.h"

template <class Tag, typename Tag::type M>
struct Expose
{
    friend typename Tag::type member(Tag) { return M; }
};
#define EXPOSE(NAME, CLS, TYPE, MEMBER)                          \
    struct NAME { typedef TYPE CLS::*type; friend type member(NAME); }; \
    template struct Expose<NAME, &CLS::MEMBER>;
EXPOSE(MrgXn, mrg32k3a, double, myXn)
EXPOSE(MrgXn1, mrg32k3a, double, myXn1)
EXPOSE(MrgXn2, mrg32k3a, double, myXn2)
EXPOSE(MrgYn, mrg32k3a, double, myYn)
EXPOSE(MrgYn1, mrg32k3a, double, myYn1)
EXPOSE(MrgYn2, mrg32k3a, double, myYn2)
EXPOSE(MrgAnti, mrg32k3a, bool, myAnti)
typedef Dupire<double> DupireD;
typedef BlackScholes<double> BSD;
EXPOSE(DupTimeline, DupireD, std::vector<double>, myTimeline)
EXPOSE(DupCommon, DupireD, std::vector<bool>, myCommonSteps)
EXPOSE(DupIv, DupireD, matrix<double>, myInterpVols)
EXPOSE(BsTimeline, BSD, std::vector<double>, myTimeline)
EXPOSE(BsStds, BSD, std::vector<double>, myStds)
EXPOSE(BsDrifts, BSD, std::vector<double>, myDrifts)
EXPOSE(BsNums, BSD, std::vector<double>, myNumeraires)
typedef MultiDisplaced<double> MdD;
EXPOSE(MdTimeline, MdD, std::vector<double>, myTimeline)
EXPOSE(MdChol, MdD, matrix<double>, myChol)
EXPOSE(MdStds, MdD, matrix<double>, myStds)
EXPOSE(MdDrifts, MdD, matrix<double>, myDrifts)
EXPOSE(MdFfs, MdD, matrix<double>, myDynFwdFacts)
EXPOSE(MdNums, MdD, std::vector<double>, myNumeraires)

template <class M>
static std::vector<double> flat(const M& m)
{
    return std::vector<double>(m.begin(), m.begin() + m.rows() * m.cols());
}

static std::vector<string> rdnames(std::istream& is, size_t n)
{
    std::vector<string> v(n);
    for (auto& s : v) is >> s;
    return v;
}

static std::vector<double> mrgState(const mrg32k3a& r)
{
    return {r.*member(MrgXn()), r.*member(MrgXn1()), r.*member(MrgXn2()),
            r.*member(MrgYn()), r.*member(MrgYn1()), r.*member(MrgYn2()),
            double(r.*member(MrgAnti()))};
}

using std::string;

static void put(const char* tag, const std::vector<double>& v)
{
    std::printf("%s %zu", tag, v.size());
    for (double d : v) std::printf(" %a", d);
    std::printf("\n");
}

static void puts_labels(const char* tag, const std::vector<string>& v)
{
    std::printf("%s %zu", tag, v.size());
    for (const auto& s : v) std::printf("|%s", s.c_str());
    std::printf("\n");
}

template <class T>
static std::vector<T> readv(std::istream& in, size_t n)
{
    std::vector<T> v(n);
    for (auto& x : v) in >> x;
    return v;
}

static double rd(std::istream& in)
{
    string s;
    in >> s;
    return std::strtod(s.c_str(), nullptr);  // accepts decimal and hex floats
}

static std::vector<double> rdv(std::istream& in, size_t n)
{
    std::vector<double> v(n);
    for (auto& x : v) x = rd(in);
    return v;
}

// Implied-vol surface iv(K,T) = a + b ln^2(K/sref)/sqrt(T) + c ln(K/sref), the synthetic
// surface of the superbucket workload (not a Merton surface).
struct ParamIVS : public IVS
{
    double a, b, c, sref;
    ParamIVS(double spot, double a_, double b_, double c_, double sref_)
        : IVS(spot), a(a_), b(b_), c(c_), sref(sref_) {}
    double impliedVol(const double strike, const Time mat) const override
    {
        const double l = std::log(strike / sref);
        return a + b * l * l / std::sqrt(mat) + c * l;
    }
};

static NumericalParam rdnum(std::istream& in)
{
    NumericalParam num;
    int sob, par;
    in >> sob >> num.numPath >> num.seed1 >> num.seed2 >> par;
    num.useSobol = sob != 0;
    num.parallel = par != 0;
    return num;
}

static double now_s()
{
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

int main()
{
    std::ios::sync_with_stdio(false);
    string cmd;
    bool poolStarted = false;
    auto ensurePool = [&]() {
        if (!poolStarted)
        {
            ThreadPool::getInstance()->start();
            poolStarted = true;
        }
    };
    while (std::cin >> cmd)
    {
        if (cmd == "sobol_u")  // D npts : first npts points of nextU
        {
            size_t D, n;
            std::cin >> D >> n;
            Sobol s;
            s.init(D);
            std::vector<double> u(D);
            for (size_t i = 0; i < n; ++i)
            {
                s.nextU(u);
                put("sobol_u", u);
            }
        }
        else if (cmd == "sobol_skip")  // D b : skipTo(b) then one nextU and nextG
        {
            size_t D;
            unsigned b;
            std::cin >> D >> b;
            Sobol s;
            s.init(D);
            s.skipTo(b);
            std::vector<double> u(D);
            s.nextU(u);
            put("sobol_skip_u", u);
            s.skipTo(b);
            s.nextG(u);
            put("sobol_skip_g", u);
        }
        else if (cmd == "sobol_dirhash")  // per-dimension FNV-1a hash of the 32 direction numbers
        {
            const unsigned* const* dir = getjkDir();
            // The tables hold 1101 dimensions (sobol.cpp), although sobol.h:93 says 1111.
            std::vector<double> h(1101);
            for (size_t d = 0; d < 1101; ++d)
            {
                unsigned long long x = 1469598103934665603ULL;
                for (int i = 0; i < 32; ++i)
                {
                    unsigned v = dir[i][d];
                    for (int k = 0; k < 4; ++k)
                    {
                        x ^= (v >> (8 * k)) & 0xffu;
                        x *= 1099511628211ULL;
                    }
                }
                h[d] = double(x & 0xffffffffffffULL);  // 48 bits: exact in a double
            }
            put("sobol_dirhash", h);
        }
        else if (cmd == "mrg_u" || cmd == "mrg_g")  // s1 s2 D n : n vectors, with state after each
        {
            unsigned s1, s2;
            size_t D, n;
            std::cin >> s1 >> s2 >> D >> n;
            mrg32k3a r(s1, s2);
            r.init(D);
            std::vector<double> u(D);
            for (size_t i = 0; i < n; ++i)
            {
                if (cmd == "mrg_u") r.nextU(u); else r.nextG(u);
                put(cmd.c_str(), u);
                put("mrg_state", mrgState(r));
            }
        }
        else if (cmd == "mrg_skip")  // s1 s2 D b : skipTo(b), state, then nextU
        {
            unsigned s1, s2, b;
            size_t D;
            std::cin >> s1 >> s2 >> D >> b;
            mrg32k3a r(s1, s2);
            r.init(D);
            r.skipTo(b);
            put("mrg_state", mrgState(r));
            std::vector<double> u(D);
            r.nextU(u);
            put("mrg_skip_u", u);
        }
        else if (cmd == "invnorm" || cmd == "normcdf" || cmd == "normdens")
        {
            size_t n;
            std::cin >> n;
            auto x = rdv(std::cin, n);
            std::vector<double> y(n);
            for (size_t i = 0; i < n; ++i)
                y[i] = cmd == "invnorm" ? invNormalCdf(x[i])
                     : cmd == "normcdf" ? normalCdf(x[i]) : normalDens(x[i]);
            put(cmd.c_str(), y);
        }
        else if (cmd == "fill")  // n x... maxDx minDx nadd add...
        {
            size_t n, na;
            std::cin >> n;
            auto x = rdv(std::cin, n);
            double maxDx = rd(std::cin), minDx = rd(std::cin);
            std::cin >> na;
            auto add = rdv(std::cin, na);
            auto f = na ? fillData(x, maxDx, minDx, add.data(), add.data() + na)
                        : fillData(x, maxDx, minDx);
            put("fill", f);
        }
        else if (cmd == "bs")  // id spot vol qspot rate div
        {
            string id;
            std::cin >> id;
            double spot = rd(std::cin), vol = rd(std::cin);
            int q;
            std::cin >> q;
            double rate = rd(std::cin), div = rd(std::cin);
            putBlackScholes(spot, vol, q != 0, rate, div, id);
        }
        else if (cmd == "dupire")  // id spot maxDt nS spots nT times vols(nS x nT)
        {
            string id;
            std::cin >> id;
            double spot = rd(std::cin), maxDt = rd(std::cin);
            size_t nS, nT;
            std::cin >> nS;
            auto spots = rdv(std::cin, nS);
            std::cin >> nT;
            auto times = rdv(std::cin, nT);
            matrix<double> vols(nS, nT);
            for (size_t i = 0; i < nS; ++i)
                for (size_t j = 0; j < nT; ++j) vols[i][j] = rd(std::cin);
            putDupire(spot, spots, times, vols, maxDt, id);
        }
        else if (cmd == "european")  // id K Tex Tset
        {
            string id;
            std::cin >> id;
            double K = rd(std::cin), te = rd(std::cin), ts = rd(std::cin);
            putEuropean(K, te, ts, id);
        }
        else if (cmd == "contingent")  // id coupon maturity payFreq smooth
        {
            string id;
            std::cin >> id;
            double cpn = rd(std::cin), mat = rd(std::cin), fq = rd(std::cin), sm = rd(std::cin);
            putContingent(cpn, mat, fq, sm, id);
        }
        else if (cmd == "uoc")  // id K B T freq smooth callput
        {
            string id;
            std::cin >> id;
            double K = rd(std::cin), B = rd(std::cin), T = rd(std::cin), f = rd(std::cin),
                   sm = rd(std::cin);
            int cp;
            std::cin >> cp;
            putBarrier(K, B, T, f, sm, cp != 0, id);
        }
        else if (cmd == "europeans")  // id n mats... strikes...
        {
            string id;
            size_t n;
            std::cin >> id >> n;
            auto mats = rdv(std::cin, n);
            auto strikes = rdv(std::cin, n);
            putEuropeans(mats, strikes, id);
        }
        else if (cmd == "displaced")  // id nA names spots atms skews disc spreads nDiv divDates divs correl lambda
        {
            string id;
            size_t nA, nD;
            std::cin >> id >> nA;
            auto names = rdnames(std::cin, nA);
            auto spots = rdv(std::cin, nA), atms = rdv(std::cin, nA), skews = rdv(std::cin, nA);
            double disc = rd(std::cin);
            auto spreads = rdv(std::cin, nA);
            std::cin >> nD;
            auto divDates = rdv(std::cin, nD);
            matrix<double> divs(nD, nA), correl(nA, nA);
            for (size_t i = 0; i < nD; ++i)
                for (size_t j = 0; j < nA; ++j) divs[i][j] = rd(std::cin);
            for (size_t i = 0; i < nA; ++i)
                for (size_t j = 0; j < nA; ++j) correl[i][j] = rd(std::cin);
            double lambda = rd(std::cin);
            putDisplaced(names, spots, atms, skews, disc, spreads, divDates, divs, correl, lambda, id);
        }
        else if (cmd == "baskets")  // id nA names weights maturity nK strikes
        {
            string id;
            size_t nA, nK;
            std::cin >> id >> nA;
            auto names = rdnames(std::cin, nA);
            auto w = rdv(std::cin, nA);
            double mat = rd(std::cin);
            std::cin >> nK;
            auto k = rdv(std::cin, nK);
            putBaskets(names, w, mat, k, id);
        }
        else if (cmd == "autocall")  // id nA names refs maturity periods ko strike cpn smooth
        {
            string id;
            size_t nA;
            int periods;
            std::cin >> id >> nA;
            auto names = rdnames(std::cin, nA);
            auto refs = rdv(std::cin, nA);
            double mat = rd(std::cin);
            std::cin >> periods;
            double ko = rd(std::cin), k = rd(std::cin), cpn = rd(std::cin), sm = rd(std::cin);
            putAutocall(names, refs, mat, periods, ko, k, cpn, sm, id);
        }
        else if (cmd == "labels")  // mid pid
        {
            string mid, pid;
            std::cin >> mid >> pid;
            puts_labels("payoff_labels", *getPayoffLabels(pid));
            puts_labels("param_labels", getModel<double>(mid)->parameterLabels());
            puts_labels("product_timeline", {});
            put("product_timeline", getProduct<double>(pid)->timeline());
            // simulation timeline of the model for this product
            auto m = getModel<double>(mid)->clone();
            auto* p = getProduct<double>(pid);
            m->allocate(p->timeline(), p->defline());
            m->init(p->timeline(), p->defline());
            if (auto* d = dynamic_cast<Dupire<double>*>(m.get()))
            {
                put("sim_timeline", d->*member(DupTimeline()));
                const auto& c = d->*member(DupCommon());
                put("common_steps", std::vector<double>(c.begin(), c.end()));
                const auto& iv = d->*member(DupIv());
                put("interp_vols", std::vector<double>(iv.begin(), iv.begin() + iv.rows() * iv.cols()));
            }
            if (auto* d = dynamic_cast<MultiDisplaced<double>*>(m.get()))
            {
                put("sim_timeline", d->*member(MdTimeline()));
                put("md_chol", flat(d->*member(MdChol())));
                put("md_stds", flat(d->*member(MdStds())));
                put("md_drifts", flat(d->*member(MdDrifts())));
                put("md_ffs", flat(d->*member(MdFfs())));
                put("md_numeraires", d->*member(MdNums()));
                put("md_alphas", d->alphas());
                std::vector<double> dyn;
                for (auto x : d->dynamics()) dyn.push_back(double(int(x)));
                put("md_dynamics", dyn);
            }
            if (auto* b = dynamic_cast<BlackScholes<double>*>(m.get()))
            {
                put("sim_timeline", b->*member(BsTimeline()));
                put("bs_stds", b->*member(BsStds()));
                put("bs_drifts", b->*member(BsDrifts()));
                put("bs_numeraires", b->*member(BsNums()));
            }
        }
        else if (cmd == "value")  // mid pid num
        {
            string mid, pid;
            std::cin >> mid >> pid;
            auto num = rdnum(std::cin);
            if (num.parallel) ensurePool();
            double t0 = now_s();
            auto r = value(mid, pid, num);
            double t1 = now_s();
            put("values", r.values);
            put("seconds", {t1 - t0});
        }
        else if (cmd == "paths")  // mid pid num : per-path payoff matrix (serial mcSimul)
        {
            string mid, pid;
            std::cin >> mid >> pid;
            auto num = rdnum(std::cin);
            std::unique_ptr<RNG> rng;
            if (num.useSobol) rng = std::make_unique<Sobol>();
            else rng = std::make_unique<mrg32k3a>(num.seed1, num.seed2);
            auto res = mcSimul(*getProduct<double>(pid), *getModel<double>(mid), *rng, num.numPath);
            std::vector<double> flat;
            for (auto& row : res) flat.insert(flat.end(), row.begin(), row.end());
            put("paths", flat);
        }
        else if (cmd == "risk")  // mid pid num payoffIdx
        {
            string mid, pid;
            std::cin >> mid >> pid;
            auto num = rdnum(std::cin);
            size_t k;
            std::cin >> k;
            if (num.parallel) ensurePool();
            const string lab = (*getPayoffLabels(pid))[k];
            double t0 = now_s();
            auto r = AADriskOne(mid, pid, num, lab);
            double t1 = now_s();
            put("values", r.payoffValues);
            put("risk_value", {r.riskPayoffValue});
            put("risks", r.risks);
            put("seconds", {t1 - t0});
        }
        else if (cmd == "riskagg")  // mid pid num n (idx weight)...
        {
            string mid, pid;
            std::cin >> mid >> pid;
            auto num = rdnum(std::cin);
            size_t n;
            std::cin >> n;
            std::map<string, double> nots;
            for (size_t i = 0; i < n; ++i)
            {
                size_t k;
                std::cin >> k;
                nots[(*getPayoffLabels(pid))[k]] = rd(std::cin);
            }
            if (num.parallel) ensurePool();
            auto r = AADriskAggregate(mid, pid, nots, num);
            put("values", r.payoffValues);
            put("risk_value", {r.riskPayoffValue});
            put("risks", r.risks);
        }
        else if (cmd == "bump")  // mid pid num : bumpRisk (main.h:316-359), one-sided 1e-8 bumps
        {
            string mid, pid;
            std::cin >> mid >> pid;
            auto num = rdnum(std::cin);
            if (num.parallel) ensurePool();
            double t0 = now_s();
            auto r = bumpRisk(mid, pid, num);
            double t1 = now_s();
            put("values", r.values);
            put("risks", std::vector<double>(r.risks.begin(),
                r.risks.begin() + r.risks.rows() * r.risks.cols()));
            put("shape", {double(r.risks.rows()), double(r.risks.cols())});
            put("seconds", {t1 - t0});
        }
        else if (cmd == "riskmulti")  // mid pid num
        {
            string mid, pid;
            std::cin >> mid >> pid;
            auto num = rdnum(std::cin);
            if (num.parallel) ensurePool();
            double t0 = now_s();
            auto r = AADriskMulti(mid, pid, num);
            double t1 = now_s();
            put("values", r.values);
            put("risks", std::vector<double>(r.risks.begin(),
                r.risks.begin() + r.risks.rows() * r.risks.cols()));
            put("shape", {double(r.risks.rows()), double(r.risks.cols())});
            put("seconds", {t1 - t0});
        }
        else if (cmd == "calib" || cmd == "superbucket" || cmd == "superbucket_bump")
        {
            // ivs: "param spot a b c sref" or "merton spot vol intens avejmp stdjmp"
            string kind;
            std::cin >> kind;
            std::unique_ptr<IVS> ivs;
            double spot = rd(std::cin);
            double mv = 0, mi = 0, ma = 0, ms = 0;
            if (kind == "param")
            {
                double a = rd(std::cin), b = rd(std::cin), c = rd(std::cin), s = rd(std::cin);
                ivs = std::make_unique<ParamIVS>(spot, a, b, c, s);
            }
            else
            {
                mv = rd(std::cin); mi = rd(std::cin); ma = rd(std::cin); ms = rd(std::cin);
                ivs = std::make_unique<MertonIVS>(spot, mv, mi, ma, ms);
            }
            size_t n;
            std::cin >> n;
            auto inclSpots = rdv(std::cin, n);
            double maxDs = rd(std::cin);
            std::cin >> n;
            auto inclTimes = rdv(std::cin, n);
            double maxDtVol = rd(std::cin);
            if (cmd == "calib")
            {
                auto r = dupireCalib(*ivs, inclSpots, maxDs, inclTimes, maxDtVol);
                put("calib_spots", r.spots);
                put("calib_times", r.times);
                put("calib_lvols", std::vector<double>(r.lVols.begin(),
                    r.lVols.begin() + r.lVols.rows() * r.lVols.cols()));
                continue;
            }
            // superbucket: maxDt pid nNot (idx w)... nStrikes strikes nMats mats num
            double maxDt = rd(std::cin);
            string pid;
            std::cin >> pid;
            size_t nn;
            std::cin >> nn;
            std::map<string, double> nots;
            for (size_t i = 0; i < nn; ++i)
            {
                size_t k;
                std::cin >> k;
                nots[(*getPayoffLabels(pid))[k]] = rd(std::cin);
            }
            std::cin >> n;
            auto strikes = rdv(std::cin, n);
            std::cin >> n;
            auto mats = rdv(std::cin, n);
            auto num = rdnum(std::cin);
            if (num.parallel) ensurePool();
            double t0 = now_s();
            if (cmd == "superbucket_bump")  // merton only, as main.h:575-696
            {
                auto r = dupireSuperbucketBump(spot, maxDt, pid, nots, inclSpots, maxDs, inclTimes,
                                               maxDtVol, strikes, mats, mv, mi, ma, ms, num);
                put("sb_value", {r.value});
                put("sb_delta", {r.delta});
                put("sb_vega", std::vector<double>(r.vega.begin(),
                    r.vega.begin() + r.vega.rows() * r.vega.cols()));
            }
            else if (kind == "merton")
            {
                auto r = dupireSuperbucket(spot, maxDt, pid, nots, inclSpots, maxDs, inclTimes,
                                           maxDtVol, strikes, mats, mv, mi, ma, ms, num);
                put("sb_value", {r.value});
                put("sb_delta", {r.delta});
                put("sb_vega", std::vector<double>(r.vega.begin(),
                    r.vega.begin() + r.vega.rows() * r.vega.cols()));
            }
            else
            {
                // The same checkpointed chain as main.h's dupireSuperbucket, on a non-Merton surface:
                // value calibration, MC adjoints to local vols, then the calibration adjoint.
                Number::tape->rewind();
                auto calib = dupireCalib(*ivs, inclSpots, maxDs, inclTimes, maxDtVol);
                putDupire(spot, calib.spots, calib.times, calib.lVols, maxDt, "sb_model");
                auto mc = dupireAADRisk("sb_model", pid, nots, num);
                Number::tape->clear();
                RiskView<Number> view(strikes, mats);
                auto ncal = dupireCalib(*ivs, inclSpots, maxDs, inclTimes, maxDtVol, view);
                for (size_t i = 0; i < mc.vega.rows(); ++i)
                    for (size_t j = 0; j < mc.vega.cols(); ++j)
                        ncal.lVols[i][j].adjoint() = mc.vega[i][j];
                Number::propagateAdjoints(std::prev(Number::tape->end()), Number::tape->begin());
                std::vector<double> vega;
                for (auto it = view.begin(); it != view.end(); ++it) vega.push_back(it->adjoint());
                Number::tape->clear();
                put("sb_value", {mc.value});
                put("sb_delta", {mc.delta});
                put("sb_microbucket", std::vector<double>(mc.vega.begin(),
                    mc.vega.begin() + mc.vega.rows() * mc.vega.cols()));
                put("sb_vega", vega);
                // the calibrated model the Monte Carlo adjoints were taken on
                put("sb_spots", calib.spots);
                put("sb_times", calib.times);
                put("sb_lvols", std::vector<double>(calib.lVols.begin(),
                    calib.lVols.begin() + calib.lVols.rows() * calib.lVols.cols()));
            }
            double t1 = now_s();
            put("seconds", {t1 - t0});
        }
        else if (cmd == "analytics")  // spot strike vol mat rate div barrier
        {
            double s = rd(std::cin), k = rd(std::cin), v = rd(std::cin), t = rd(std::cin),
                   r = rd(std::cin), d = rd(std::cin), b = rd(std::cin);
            double bs = blackScholes(s, k, v, t);
            put("analytics", {bs, blackScholesIvol(s, k, bs, t), BlackScholesKO(s, r, d, k, b, t, v),
                              merton(s, k, v, t, 0.5, -0.1, 0.15)});
        }
        else if (cmd == "threads")
        {
            ensurePool();
            put("threads", {double(ThreadPool::getInstance()->numThreads() + 1)});
        }
        else
        {
            std::fprintf(stderr, "ref_driver: unknown command %s\n", cmd.c_str());
            return 1;
        }
        std::fflush(stdout);
    }
    if (poolStarted) ThreadPool::getInstance()->stop();
    return 0;
}
