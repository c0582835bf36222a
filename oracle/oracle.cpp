// CPU restatement of the reference's Monte Carlo valuation and AAD-risk path.
//
// TEST INFRASTRUCTURE ONLY (see oracle.h): the checker of the CUDA engine and the timed
// CPU baseline.  Each function cites the reference file:line whose behaviour it restates.
// Compiled with -ffp-contract=off so that the double arithmetic matches the reference's.

#include "oracle.h"

#include <algorithm>
#include <stdexcept>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <thread>
#include <type_traits>
#include <vector>

namespace {

using std::vector;

constexpr double kEps = 1.0e-08;                  // gaussians.h:8, utility.h:9
constexpr double kHalfDay = 0.00136986301369863;  // mcMdlDupire.h:26
constexpr double kOneHour = 0.000114469;          // mcPrd.h:26, mcMdlDupire.h:333
constexpr double kOneDay = 0.003773585;           // mcPrd.h:27
constexpr double kOneOver2Pow32 = 2.3283064365387E-10;  // sobol.h:26 (truncated constant)

// ---------------------------------------------------------------------------------------
// Gaussian functions, gaussians.h:13-87
// ---------------------------------------------------------------------------------------
double normalDens(double x)
{
    return x < -10.0 || 10.0 < x ? 0.0 : std::exp(-0.5 * x * x) / 2.506628274631;
}

double normalCdf(double x)  // Zelen-Severo
{
    if (x < -10.0) return 0.0;
    if (x > 10.0) return 1.0;
    if (x < 0.0) return 1.0 - normalCdf(-x);
    const double t = 1.0 / (1.0 + 0.2316419 * x);
    const double pol =
        t * (0.319381530 + t * (-0.356563782 + t * (1.781477937 + t * (-1.821255978 + t * 1.330274429))));
    return 1.0 - normalDens(x) * pol;
}

double invNormalCdf(double p)  // Beasley-Springer-Moro
{
    const bool sup = p > 0.5;
    const double up = sup ? 1.0 - p : p;
    const double x = up - 0.5;
    if (std::fabs(x) < 0.42)
    {
        double r = x * x;
        r = x * (((-25.44106049637 * r + 41.39119773534) * r + -18.61500062529) * r + 2.50662823884) /
            ((((3.13082909833 * r + -21.06224101826) * r + 23.08336743743) * r + -8.47351093090) * r + 1.0);
        return sup ? -r : r;
    }
    double r = std::log(-std::log(up));
    r = 0.3374754822726147 +
        r * (0.9761690190917186 +
             r * (0.1607979714918209 +
                  r * (0.0276438810333863 +
                       r * (0.0038405729373609 +
                            r * (0.0003951896511919 +
                                 r * (0.0000321767881768 + r * (0.0000002888167364 + r * 0.0000003960315187)))))));
    return sup ? r : -r;
}

// ---------------------------------------------------------------------------------------
// A small reverse-mode tape (restates the role of AADTape.h / AADExpr.h: parameters and
// model initialisation are recorded once above a mark, each path is recorded after it,
// swept back to the mark, and the accumulated above-mark adjoints are swept to the start
// once at the end).  Adjoints may be vectors (multi-payoff risk, AADNode.h:85-102).
// ---------------------------------------------------------------------------------------
struct Node
{
    int a0, a1;
    double d0, d1;
};

struct Tape
{
    vector<Node> nodes;
    vector<double> adj;
    size_t mark = 0;
    int width = 1;
    void clear() { nodes.clear(); adj.clear(); mark = 0; }
    int push(int a0, double d0, int a1, double d1)
    {
        nodes.push_back({a0, a1, d0, d1});
        return int(nodes.size()) - 1;
    }
    void sizeAdj() { adj.assign(nodes.size() * width, 0.0); }
    // Propagate adjoints of nodes [lo, hi) backwards (hi-1 down to lo).
    void sweep(size_t hi, size_t lo)
    {
        for (size_t k = hi; k-- > lo;)
        {
            const Node& n = nodes[k];
            const double* ak = &adj[k * width];
            if (n.a0 >= 0)
                for (int w = 0; w < width; ++w) adj[size_t(n.a0) * width + w] += n.d0 * ak[w];
            if (n.a1 >= 0)
                for (int w = 0; w < width; ++w) adj[size_t(n.a1) * width + w] += n.d1 * ak[w];
        }
    }
};

thread_local Tape* gTape = nullptr;

struct Var
{
    double v;
    int i;  // node index, -1 = constant
    Var() : v(0.0), i(-1) {}
    Var(double x) : v(x), i(-1) {}
    Var(double x, int idx) : v(x), i(idx) {}
};

inline Var leaf(double x) { return Var(x, gTape->push(-1, 0.0, -1, 0.0)); }
inline Var un(double v, const Var& a, double da)
{
    if (a.i < 0) return Var(v);
    return Var(v, gTape->push(a.i, da, -1, 0.0));
}
inline Var bin(double v, const Var& a, double da, const Var& b, double db)
{
    if (a.i < 0 && b.i < 0) return Var(v);
    return Var(v, gTape->push(a.i, da, b.i, db));
}
inline Var operator+(const Var& a, const Var& b) { return bin(a.v + b.v, a, 1.0, b, 1.0); }
inline Var operator-(const Var& a, const Var& b) { return bin(a.v - b.v, a, 1.0, b, -1.0); }
inline Var operator*(const Var& a, const Var& b) { return bin(a.v * b.v, a, b.v, b, a.v); }
inline Var operator/(const Var& a, const Var& b) { return bin(a.v / b.v, a, 1.0 / b.v, b, -a.v / b.v / b.v); }
inline Var operator+(const Var& a, double b) { return un(a.v + b, a, 1.0); }
inline Var operator+(double b, const Var& a) { return un(b + a.v, a, 1.0); }
inline Var operator-(const Var& a, double b) { return un(a.v - b, a, 1.0); }
inline Var operator-(double b, const Var& a) { return un(b - a.v, a, -1.0); }
inline Var operator*(const Var& a, double b) { return un(a.v * b, a, b); }
inline Var operator*(double b, const Var& a) { return un(b * a.v, a, b); }
inline Var operator/(const Var& a, double b) { return un(a.v / b, a, 1.0 / b); }
inline Var operator/(double b, const Var& a) { return un(b / a.v, a, -b / a.v / a.v); }
inline Var operator-(const Var& a) { return un(-a.v, a, -1.0); }
inline Var& operator+=(Var& a, const Var& b) { return a = a + b; }
inline Var& operator*=(Var& a, const Var& b) { return a = a * b; }
inline Var exp(const Var& a) { const double e = std::exp(a.v); return un(e, a, e); }
inline Var log(const Var& a) { return un(std::log(a.v), a, 1.0 / a.v); }
inline Var sqrt(const Var& a) { const double s = std::sqrt(a.v); return un(s, a, 0.5 / s); }
inline Var vmax(const Var& a, double d) { return un(std::max(a.v, d), a, a.v > d ? 1.0 : 0.0); }  // AADExpr.h:571-583
inline Var normalCdf(const Var& a) { return un(normalCdf(a.v), a, normalDens(a.v)); }           // AADExpr.h:434-447
inline double exp(double a) { return std::exp(a); }
inline double log(double a) { return std::log(a); }
inline double sqrt(double a) { return std::sqrt(a); }
inline double val(const Var& a) { return a.v; }
inline double val(double a) { return a; }
inline double vmax(double a, double d) { return std::max(a, d); }

// ---------------------------------------------------------------------------------------
// Utilities: fillData (utility.h:11-79), interp (interp.h:26-63), interp2D (interp.h:66-109)
// ---------------------------------------------------------------------------------------
vector<double> fillData(const vector<double>& original, double maxDx, double minDx,
                        const double* addB = nullptr, const double* addE = nullptr)
{
    vector<double> added;
    const size_t nAdd = addB && addE ? size_t(addE - addB) : 0;
    if (nAdd)
        std::set_union(original.begin(), original.end(), addB, addE, std::back_inserter(added),
                       [minDx](double x, double y) { return x < y - minDx; });
    const vector<double>& seq = nAdd ? added : original;
    vector<double> filled;
    auto it = seq.begin();
    filled.push_back(*it);
    ++it;
    while (it != seq.end())
    {
        const double cur = filled.back(), nxt = *it;
        if (nxt - cur > maxDx)
        {
            const int add = int((nxt - cur) / maxDx - kEps) + 1;
            const double spacing = (nxt - cur) / add;
            double t = cur + spacing;
            while (t < nxt - minDx)
            {
                filled.push_back(t);
                t += spacing;
            }
        }
        filled.push_back(*it);
        ++it;
    }
    return filled;
}

template <bool Smooth, class T>
T interp(const double* x, size_t n, const T* y, double x0)
{
    const double* it = std::upper_bound(x, x + n, x0);
    if (it == x + n) return y[n - 1];
    if (it == x) return y[0];
    const size_t k = size_t(it - x) - 1;
    const double t = (x0 - x[k]) / (x[k + 1] - x[k]);
    if (Smooth) return y[k] + (y[k + 1] - y[k]) * t * t * (3.0 - 2 * t);
    return y[k] + (y[k + 1] - y[k]) * t;
}

// Interpolation in a model variable x0 (Dupire spot axis): t carries the derivative.
template <class T>
T interpVar(const double* x, size_t n, const T* y, const T& x0)
{
    const double* it = std::upper_bound(x, x + n, val(x0));
    if (it == x + n) return y[n - 1];
    if (it == x) return y[0];
    const size_t k = size_t(it - x) - 1;
    const T t = (x0 - x[k]) / (x[k + 1] - x[k]);
    return y[k] + (y[k + 1] - y[k]) * t;
}

template <class T>
T interp2DSmooth(const vector<double>& x, const vector<double>& y, const vector<T>& z, double x0, double y0)
{
    const size_t n = x.size(), m = y.size();
    const size_t n2 = size_t(std::upper_bound(x.begin(), x.end(), x0) - x.begin());
    if (n2 == n) return interp<true>(y.data(), m, &z[(n2 - 1) * m], y0);
    if (n2 == 0) return interp<true>(y.data(), m, &z[0], y0);
    const size_t n1 = n2 - 1;
    const T z1 = interp<true>(y.data(), m, &z[n1 * m], y0);
    const T z2 = interp<true>(y.data(), m, &z[n2 * m], y0);
    const double t = (x0 - x[n1]) / (x[n2] - x[n1]);
    return z1 + (z2 - z1) * t * t * (3.0 - 2 * t);
}

// ---------------------------------------------------------------------------------------
// RNGs: Sobol (sobol.h:30-152) with direction numbers regenerated from the Joe-Kuo
// initialisation data, and mrg32k3a (mrg32k3a.h:25-394) in the reference's double arithmetic.
// ---------------------------------------------------------------------------------------
struct JKInit
{
    int s, a;
    unsigned m[13];
};
const JKInit kJK[] = {
#include "../compfinance_gb300/data/sobol_joe_kuo.inc"
};

const vector<unsigned>& sobolDirs()  // [32][CF_SOBOL_MAX_DIM]
{
    static vector<unsigned> dirs = [] {
        vector<unsigned> d(32 * CF_SOBOL_MAX_DIM);
        for (int dim = 0; dim < CF_SOBOL_MAX_DIM; ++dim)
        {
            const JKInit& e = kJK[dim];
            uint64_t m[32];
            if (e.s == 0)
                for (int k = 0; k < 32; ++k) m[k] = 1;
            else
            {
                for (int k = 0; k < e.s; ++k) m[k] = e.m[k];
                for (int k = e.s; k < 32; ++k)
                {
                    uint64_t v = m[k - e.s] ^ (m[k - e.s] << e.s);
                    for (int j = 1; j < e.s; ++j)
                        if ((e.a >> (e.s - 1 - j)) & 1) v ^= m[k - j] << j;
                    m[k] = v;
                }
            }
            for (int k = 0; k < 32; ++k) d[size_t(k) * CF_SOBOL_MAX_DIM + dim] = unsigned(m[k] << (31 - k));
        }
        return d;
    }();
    return dirs;
}

struct Rng
{
    virtual ~Rng() {}
    virtual void nextG(double* g) = 0;
    virtual void skipTo(uint64_t path) = 0;  // position before path `path` (serial stream)
};

struct Sobol : Rng
{
    int dim;
    vector<unsigned> state;
    uint64_t index = 0;
    explicit Sobol(int d) : dim(d), state(d, 0u) {}
    void next()  // sobol.h:77-100
    {
        uint64_t n = index;
        int j = 0;
        while (n & 1) { n >>= 1; ++j; }
        const unsigned* dn = &sobolDirs()[size_t(j) * CF_SOBOL_MAX_DIM];
        for (int i = 0; i < dim; ++i) state[i] ^= dn[i];
        ++index;
    }
    void nextG(double* g) override
    {
        next();
        for (int i = 0; i < dim; ++i) g[i] = invNormalCdf(kOneOver2Pow32 * state[i]);
    }
    void skipTo(uint64_t b) override  // sobol.h:119-151: state = XOR of dirs over gray(b)
    {
        std::fill(state.begin(), state.end(), 0u);
        const uint64_t gray = b ^ (b >> 1);
        for (int i = 0; i < 32; ++i)
            if ((gray >> i) & 1)
            {
                const unsigned* dn = &sobolDirs()[size_t(i) * CF_SOBOL_MAX_DIM];
                for (int k = 0; k < dim; ++k) state[k] ^= dn[k];
            }
        index = b;
    }
};

struct Mrg : Rng
{
    static constexpr double m1 = 4294967087, m2 = 4294944443, a12 = 1403580, a13 = 810728,
                            a21 = 527612, a23 = 1370589, m1p1 = 4294967088;
    double A, B;
    int dim;
    double x0, x1, x2, y0, y1, y2;
    bool anti = false;
    vector<double> cachedG;
    Mrg(unsigned a, unsigned b, int d) : A(a), B(b), dim(d), cachedG(d) { reset(); }
    void reset()
    {
        x0 = x1 = x2 = A;
        y0 = y1 = y2 = B;
        anti = false;
    }
    double nextNumber()  // mrg32k3a.h:55-81
    {
        double x = a12 * x1 - a13 * x2;
        x -= long(x / m1) * m1;
        if (x < 0) x += m1;
        x2 = x1; x1 = x0; x0 = x;
        double y = a21 * y0 - a23 * y2;
        y -= long(y / m2) * m2;
        if (y < 0) y += m2;
        y2 = y1; y1 = y0; y0 = y;
        return x > y ? (x - y) / m1p1 : (x - y + m1) / m1p1;
    }
    void nextG(double* g) override  // mrg32k3a.h:150-184: antithetic pairs
    {
        if (anti)
        {
            for (int i = 0; i < dim; ++i) g[i] = -cachedG[i];
            anti = false;
        }
        else
        {
            for (int i = 0; i < dim; ++i) g[i] = cachedG[i] = invNormalCdf(nextNumber());
            anti = true;
        }
    }
    static void mulmat(const uint64_t a[9], const uint64_t b[9], uint64_t mod, uint64_t r[9])
    {
        uint64_t t[9];
        for (int j = 0; j < 3; ++j)
            for (int k = 0; k < 3; ++k)
            {
                uint64_t s = 0;
                for (int l = 0; l < 3; ++l) s = (s + (a[3 * j + l] * b[3 * l + k]) % mod) % mod;
                t[3 * j + k] = s;
            }
        std::memcpy(r, t, sizeof(t));
    }
    void skipNumbers(uint64_t n)  // mrg32k3a.h:306-394 (64-bit count)
    {
        const uint64_t M1 = 4294967087ULL, M2 = 4294944443ULL;
        uint64_t Ab[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1}, Bb[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
        uint64_t Ai[9] = {0, 1403580, M1 - 810728, 1, 0, 0, 0, 1, 0};
        uint64_t Bi[9] = {527612, 0, M2 - 1370589, 1, 0, 0, 0, 1, 0};
        while (n)
        {
            if (n & 1) { mulmat(Ab, Ai, M1, Ab); mulmat(Bb, Bi, M2, Bb); }
            mulmat(Ai, Ai, M1, Ai);
            mulmat(Bi, Bi, M2, Bi);
            n >>= 1;
        }
        const uint64_t X[3] = {uint64_t(x0), uint64_t(x1), uint64_t(x2)};
        const uint64_t Y[3] = {uint64_t(y0), uint64_t(y1), uint64_t(y2)};
        double nx[3], ny[3];
        for (int j = 0; j < 3; ++j)
        {
            uint64_t s = 0, t = 0;
            for (int l = 0; l < 3; ++l)
            {
                s = (s + (Ab[3 * j + l] * X[l]) % M1) % M1;
                t = (t + (Bb[3 * j + l] * Y[l]) % M2) % M2;
            }
            nx[j] = double(s);
            ny[j] = double(t);
        }
        x0 = nx[0]; x1 = nx[1]; x2 = nx[2];
        y0 = ny[0]; y1 = ny[1]; y2 = ny[2];
    }
    // Serial semantics: path b starts at uniform index floor(b/2)*dim; an odd b is the
    // antithetic twin of b-1 (mrg32k3a.h:192-238 with 64-bit counts).
    void skipTo(uint64_t b) override
    {
        reset();
        skipNumbers((b / 2) * uint64_t(dim));
        if (b & 1)
        {
            for (int i = 0; i < dim; ++i) cachedG[i] = invNormalCdf(nextNumber());
            anti = true;
        }
    }
};

// ---------------------------------------------------------------------------------------
// Scenario layout shared by models and products: one sample per product event date with
// the quantities the products read (mcBase.h:45-117): numeraire, one forward, one discount.
// ---------------------------------------------------------------------------------------
template <class T>
struct Sample
{
    T numeraire, forward, discount, libor;
};

struct ProductDef
{
    vector<double> timeline;
    vector<double> fwdMat;   // forward maturity per event (forwardMats[0][0])
    vector<double> discMat;  // discount maturity per event, NaN when none
    vector<int> needNum;
    vector<double> libEnd;   // libor(t, libEnd) per event, NaN when none
    vector<std::string> labels;
};

std::string fmt2(double x)
{
    char b[64];
    std::snprintf(b, sizeof b, "%.2f", x);
    return b;
}

// Product timelines and deflines: mcPrd.h:43-80 (European), 149-211 (UOC), 305-340 (Europeans).
ProductDef productDef(const orc_product& p)
{
    ProductDef d;
    if (p.kind == 0)
    {
        d.timeline = {p.exercise};
        d.fwdMat = {p.settlement};
        d.discMat = {p.settlement};
        d.needNum = {1};
        d.labels = {p.settlement == p.exercise ? "call " + fmt2(p.strike) + " " + fmt2(p.exercise)
                                               : "call " + fmt2(p.strike) + " " + fmt2(p.exercise) + " " +
                                                     fmt2(p.settlement)};
    }
    else if (p.kind == 1)
    {
        d.timeline.push_back(0.0);
        double t = p.freq;
        while (p.maturity - t > kOneHour)
        {
            d.timeline.push_back(t);
            t += p.freq;
        }
        d.timeline.push_back(p.maturity);
        for (double x : d.timeline)
        {
            d.fwdMat.push_back(x);
            d.discMat.push_back(NAN);
            d.needNum.push_back(0);
        }
        d.needNum.back() = 1;
        const double sm = p.smooth <= 0 ? kEps : p.smooth;  // store.h:153
        const std::string l1 = std::string(p.callput ? "put " : "call ") + fmt2(p.maturity) + " " + fmt2(p.strike);
        d.labels = {l1 + " up and out " + fmt2(p.barrier) + " monitoring freq " + fmt2(p.freq) + " smooth " + fmt2(sm),
                    l1};
    }
    else if (p.kind == 3)
    {
        // mcPrd.h:426-480: today, every payFreq while more than a day remains, maturity; spot
        // on every date, libor(Ti, Ti+1) on every date but the last, numeraire after today
        d.timeline.push_back(0.0);
        double t = p.freq;
        while (p.maturity - t > kOneDay)
        {
            d.timeline.push_back(t);
            t += p.freq;
        }
        d.timeline.push_back(p.maturity);
        const size_t n = d.timeline.size();
        for (size_t i = 0; i < n; ++i)
        {
            d.fwdMat.push_back(d.timeline[i]);
            d.discMat.push_back(NAN);
            d.needNum.push_back(i > 0);
            d.libEnd.push_back(i + 1 < n ? d.timeline[i + 1] : NAN);
        }
        d.labels = {"contingent bond " + fmt2(p.maturity) + " " + fmt2(p.coupon)};
    }
    else
    {
        std::map<double, vector<double>> opts;  // store.h:184-205
        for (int i = 0; i < p.n; ++i) opts[p.mats[i]].push_back(p.strikes[i]);
        for (auto& kv : opts)
        {
            d.timeline.push_back(kv.first);
            d.fwdMat.push_back(kv.first);
            d.discMat.push_back(NAN);
            d.needNum.push_back(1);
            for (double k : kv.second) d.labels.push_back("call " + fmt2(kv.first) + " " + fmt2(k));
        }
    }
    return d;
}

// Per-run product data of the payoffs: Europeans, per event the strikes in insertion order
// (mcPrd.h:374-399); ContingentBond, the coverages of the periods (myDt, mcPrd.h:441-452).
vector<vector<double>> europeansStrikes(const orc_product& p)
{
    if (p.kind == 3)
    {
        const ProductDef d = productDef(p);
        vector<double> cov;
        for (size_t i = 0; i + 1 < d.timeline.size(); ++i) cov.push_back(d.timeline[i + 1] - d.timeline[i]);
        return {cov};
    }
    std::map<double, vector<double>> opts;
    for (int i = 0; i < p.n; ++i) opts[p.mats[i]].push_back(p.strikes[i]);
    vector<vector<double>> s;
    for (auto& kv : opts) s.push_back(kv.second);
    return s;
}

template <class T>
void payoffs(const orc_product& p, const vector<vector<double>>& estr, const Sample<T>* path, size_t nEv, T* out)
{
    if (p.kind == 0)  // mcPrd.h:113-125
    {
        const Sample<T>& s = path[0];
        out[0] = vmax(s.forward - p.strike, 0.0) * s.discount / s.numeraire;
    }
    else if (p.kind == 1)  // mcPrd.h:235-288
    {
        const double sm = p.smooth <= 0 ? kEps : p.smooth;
        const double smooth = val(path[0].forward) * sm, twoSmooth = 2 * smooth,
                     barSmooth = p.barrier + smooth, minusSmooth = p.barrier - smooth;
        T alive(1.0);
        for (size_t e = 0; e < nEv; ++e)
        {
            const T& spot = path[e].forward;
            if (val(spot) > barSmooth)
            {
                alive = T(0.0);
                break;
            }
            else if (val(spot) > minusSmooth)
                alive *= (barSmooth - spot) / twoSmooth;
        }
        const T& fin = path[nEv - 1].forward;
        const T euro = p.callput ? vmax(p.strike - fin, 0.0) / path[nEv - 1].numeraire
                                 : vmax(fin - p.strike, 0.0) / path[nEv - 1].numeraire;
        out[0] = alive * euro;
        out[1] = euro;
    }
    else if (p.kind == 3)  // mcPrd.h:522-573
    {
        const double smooth = val(path[0].forward) * (p.smooth <= 0 ? 0.0 : p.smooth), twoSmooth = 2 * smooth;
        T pay(0.0);
        for (size_t i = 0; i + 1 < nEv; ++i)
        {
            const T& s0 = path[i].forward;
            const T& s1 = path[i + 1].forward;
            T digital;
            if (val(s1) - val(s0) > smooth) digital = T(1.0);
            else if (val(s1) - val(s0) < -smooth) digital = T(0.0);
            else digital = (s1 - s0 + smooth) / twoSmooth;
            pay += digital * (path[i].libor + p.coupon) * estr[0][i] / path[i + 1].numeraire;
        }
        pay += 1.0 / path[nEv - 1].numeraire;
        out[0] = pay;
    }
    else  // mcPrd.h:374-399
    {
        size_t k = 0;
        for (size_t e = 0; e < nEv; ++e)
            for (double K : estr[e]) out[k++] = vmax(path[e].forward - K, 0.0) / path[e].numeraire;
    }
}

// ---------------------------------------------------------------------------------------
// Models.  Black-Scholes: mcMdlBS.h:149-350.  Dupire: mcMdlDupire.h:165-280.
// ---------------------------------------------------------------------------------------
template <class T>
struct ModelRun
{
    const orc_model* m;
    const ProductDef* pd;
    // parameters (on tape when T = Var)
    vector<T> params;
    // simulation timeline
    vector<double> tl;
    vector<int> common;  // Dupire: step index is a product date
    // BS precomputations
    vector<T> stds, drifts, nums, discs, ffs, libs;
    bool todayOn = false;
    // Dupire precomputations
    vector<double> logSpots;
    vector<T> iv;  // [nSteps][nS]

    void allocate(const orc_model& mm, const ProductDef& p)
    {
        m = &mm;
        pd = &p;
        if (mm.kind == 0)
        {
            tl = {0.0};
            for (double t : p.timeline)
                if (t > 0.0) tl.push_back(t);
            todayOn = p.timeline[0] == 0.0;
        }
        else
        {
            const double sys = 0.0;
            tl = fillData(p.timeline, mm.maxdt, kHalfDay, &sys, &sys + 1);
            common.resize(tl.size());
            for (size_t i = 0; i < tl.size(); ++i)
                common[i] = std::binary_search(p.timeline.begin(), p.timeline.end(), tl[i]);
            logSpots.resize(mm.nS);
            for (int i = 0; i < mm.nS; ++i) logSpots[i] = std::log(mm.spots[i]);
        }
    }
    size_t simDim() const { return tl.size() - 1; }
    size_t numParams() const { return m->kind == 0 ? 4 : 1 + size_t(m->nS) * m->nT; }

    // Parameters: BS {spot, vol, rate, div}; Dupire {spot, vols spot-major}.
    void putParams(bool onTape)
    {
        params.clear();
        auto mk = [&](double x) { return onTape ? T(leafOf(x)) : T(x); };
        params.push_back(mk(m->spot));
        if (m->kind == 0)
        {
            params.push_back(mk(m->vol));
            params.push_back(mk(m->rate));
            params.push_back(mk(m->div));
        }
        else
            for (int i = 0; i < m->nS * m->nT; ++i) params.push_back(mk(m->vols[i]));
    }
    static T leafOf(double x);

    void init()
    {
        const size_t n = simDim();
        if (m->kind == 0)
        {
            const T& vol = params[1];
            const T mu = params[2] - params[3];
            stds.resize(n);
            drifts.resize(n);
            for (size_t i = 0; i < n; ++i)
            {
                const double dt = tl[i + 1] - tl[i];
                stds[i] = vol * std::sqrt(dt);
                drifts[i] = m->spot_measure ? (mu + 0.5 * vol * vol) * dt : (mu - 0.5 * vol * vol) * dt;
            }
            const size_t ne = pd->timeline.size();
            nums.assign(ne, T(1.0));
            discs.assign(ne, T(1.0));
            ffs.assign(ne, T(1.0));
            libs.assign(ne, T(0.0));
            for (size_t e = 0; e < ne; ++e)
            {
                const double t = pd->timeline[e];
                if (pd->needNum[e])
                    nums[e] = m->spot_measure ? exp(params[3] * t) / params[0] : exp(params[2] * t);
                if (!std::isnan(pd->discMat[e])) discs[e] = exp(-params[2] * (pd->discMat[e] - t));
                ffs[e] = exp(mu * (pd->fwdMat[e] - t));
                if (!pd->libEnd.empty() && !std::isnan(pd->libEnd[e]))  // mcMdlBS.h:266-272
                {
                    const double dt = pd->libEnd[e] - t;
                    libs[e] = (exp(params[2] * dt) - 1.0) / dt;
                }
            }
        }
        else
        {
            const int nS = m->nS, nT = m->nT;
            iv.resize(n * nS);
            for (size_t i = 0; i < n; ++i)
            {
                const double sq = std::sqrt(tl[i + 1] - tl[i]);
                for (int j = 0; j < nS; ++j)
                    iv[i * nS + j] = sq * interp<false>(m->times, nT, &params[1 + size_t(j) * nT], tl[i]);
            }
        }
    }

    // generatePath; path has one Sample per product date.
    void generatePath(const double* g, Sample<T>* path) const
    {
        if (m->kind == 0)
        {
            T spot = params[0];
            size_t idx = 0;
            auto fill = [&](size_t e, const T& s) {
                path[e].numeraire = pd->needNum[e] ? (m->spot_measure ? nums[e] * s : nums[e]) : T(1.0);
                path[e].forward = s * ffs[e];
                path[e].discount = discs[e];
                path[e].libor = libs[e];
            };
            if (todayOn) fill(idx++, spot);
            for (size_t i = 0; i < simDim(); ++i)
            {
                spot = spot * exp(drifts[i] + stds[i] * g[i]);
                fill(idx++, spot);
            }
        }
        else
        {
            const int nS = m->nS;
            T logspot = log(params[0]);
            size_t idx = 0;
            if (common[0])
            {
                path[idx].numeraire = T(1.0);
                path[idx].discount = T(1.0);
                path[idx].libor = T(0.0);
                path[idx++].forward = exp(logspot);
            }
            for (size_t i = 0; i < simDim(); ++i)
            {
                const T vol = interpVar(logSpots.data(), nS, &iv[i * nS], logspot);
                logspot += vol * (-0.5 * vol + g[i]);
                if (common[i + 1])
                {
                    path[idx].numeraire = T(1.0);
                    path[idx].discount = T(1.0);
                    path[idx].libor = T(0.0);
                    path[idx++].forward = exp(logspot);
                }
            }
        }
    }
};

template <>
double ModelRun<double>::leafOf(double x) { return x; }
template <>
Var ModelRun<Var>::leafOf(double x) { return leaf(x); }

std::unique_ptr<Rng> makeRng(int sobol, unsigned s1, unsigned s2, int dim)
{
    if (sobol) return std::unique_ptr<Rng>(new Sobol(dim));
    return std::unique_ptr<Rng>(new Mrg(s1, s2, dim));
}

int nPayoffs(const orc_product& p) { return p.kind == 0 || p.kind == 3 ? 1 : p.kind == 1 ? 2 : p.n; }

// Serial path loop (mcBase.h:267-308) over paths [first, first+count).
void runPaths(const orc_model& m, const orc_product& p, int sobol, unsigned s1, unsigned s2, uint64_t first,
              uint64_t count, double* sum, double* sumsq, double* perPath)
{
    const ProductDef pd = productDef(p);
    const auto estr = europeansStrikes(p);
    ModelRun<double> mr;
    mr.allocate(m, pd);
    mr.putParams(false);
    mr.init();
    const int dim = int(mr.simDim());
    auto rng = makeRng(sobol, s1, s2, dim);
    if (first) rng->skipTo(first);
    vector<double> g(dim);
    vector<Sample<double>> path(pd.timeline.size());
    const int nPay = nPayoffs(p);
    vector<double> pay(nPay);
    for (uint64_t i = 0; i < count; ++i)
    {
        rng->nextG(g.data());
        mr.generatePath(g.data(), path.data());
        payoffs(p, estr, path.data(), path.size(), pay.data());
        for (int k = 0; k < nPay; ++k)
        {
            if (sum) sum[k] += pay[k];
            if (sumsq) sumsq[k] += pay[k] * pay[k];
            if (perPath) perPath[i * nPay + k] = pay[k];
        }
    }
}

// Tape-based risk over paths [first, first+count) on the calling thread's tape
// (mcBase.h:427-532, 775-854).  width = 1 with weights, or nPay for multi-risk.
//
// refMarkQuirk reproduces a property of the reference's multi-adjoint loop: its final sweep
// starts AT the mark (mcBase.h:847, inclusive bounds of AADExpr.h:1068-1079), so the first
// node recorded after the mark by the last path is propagated a second time.  The emulation
// is exact when that first statement is a single tape node (Dupire: log(spot),
// mcMdlDupire.h:248); the reference's expression templates fold a whole statement into
// one node, which this fine-grained tape does not.
void runRiskTape(const orc_model& m, const orc_product& p, int sobol, unsigned s1, unsigned s2, uint64_t first,
                 uint64_t count, const double* weights, bool multi, double* paySum, double* aggSum,
                 double* riskSum /* nParam * width, accumulated */, bool refMarkQuirk = false)
{
    Tape tape;
    gTape = &tape;
    const ProductDef pd = productDef(p);
    const auto estr = europeansStrikes(p);
    ModelRun<Var> mr;
    mr.allocate(m, pd);
    mr.putParams(true);
    mr.init();
    tape.mark = tape.nodes.size();
    const int nPay = nPayoffs(p);
    tape.width = multi ? nPay : 1;
    const int dim = int(mr.simDim());
    auto rng = makeRng(sobol, s1, s2, dim);
    if (first) rng->skipTo(first);
    vector<double> g(dim);
    vector<Sample<Var>> path(pd.timeline.size());
    vector<Var> pay(nPay);
    tape.adj.assign(tape.mark * tape.width, 0.0);  // above-mark adjoints accumulate over paths
    for (uint64_t i = 0; i < count; ++i)
    {
        tape.nodes.resize(tape.mark);
        rng->nextG(g.data());
        mr.generatePath(g.data(), path.data());
        payoffs(p, estr, path.data(), path.size(), pay.data());
        for (int k = 0; k < nPay; ++k) paySum[k] += pay[k].v;
        Var agg(0.0);
        if (!multi)
        {
            for (int k = 0; k < nPay; ++k)
                if (weights[k] != 0.0) agg = agg + pay[k] * weights[k];
            *aggSum += agg.v;
        }
        tape.adj.resize(tape.nodes.size() * tape.width, 0.0);
        if (multi)
        {
            for (int k = 0; k < nPay; ++k)
                if (pay[k].i >= 0) tape.adj[size_t(pay[k].i) * tape.width + k] += 1.0;
        }
        else if (agg.i >= 0)
            tape.adj[size_t(agg.i)] += 1.0;
        tape.sweep(tape.nodes.size(), tape.mark);
        if (refMarkQuirk && i + 1 == count && tape.nodes.size() > tape.mark)
            tape.sweep(tape.mark + 1, tape.mark);
        tape.adj.resize(tape.mark * tape.width);
    }
    // mark -> start
    tape.nodes.resize(tape.mark);
    tape.sweep(tape.mark, 0);
    const size_t nParam = mr.numParams();
    for (size_t j = 0; j < nParam; ++j)
        for (int w = 0; w < tape.width; ++w)
            riskSum[j * tape.width + w] += tape.adj[size_t(mr.params[j].i) * tape.width + w];
    gTape = nullptr;
}

// Split [0, n) into nThreads contiguous, even-aligned ranges (antithetic pairs stay together).
vector<std::pair<uint64_t, uint64_t>> ranges(uint64_t n, int nThreads)
{
    vector<std::pair<uint64_t, uint64_t>> r;
    uint64_t per = (n + nThreads - 1) / nThreads;
    per += per & 1;
    for (uint64_t s = 0; s < n; s += per) r.push_back({s, std::min(per, n - s)});
    return r;
}

// ---------------------------------------------------------------------------------------
// Hand-written per-path adjoint of the Dupire path (no tape): the timed CPU baseline.
// Same derivatives as the tape: x_{i+1} = x_i + v_i(-v_i/2 + g_i), v_i = interp(Y[i], x_i).
// ---------------------------------------------------------------------------------------
void runRiskFastDupire(const orc_model& m, const orc_product& p, int sobol, unsigned s1, unsigned s2,
                       uint64_t first, uint64_t count, const double* w, double* paySum, double* aggSum,
                       double* risk /* 1 + nS*nT */)
{
    const ProductDef pd = productDef(p);
    const auto estr = europeansStrikes(p);
    ModelRun<double> mr;
    mr.allocate(m, pd);
    mr.putParams(false);
    mr.init();
    const int n = int(mr.simDim()), nS = m.nS, nT = m.nT;
    const double* X = mr.logSpots.data();
    vector<double> invdX(nS > 1 ? nS - 1 : 1);
    for (int k = 0; k + 1 < nS; ++k) invdX[k] = 1.0 / (X[k + 1] - X[k]);
    // time interpolation coefficients of each step (init: iv[i][j] = sqrt(dt) * interp_t)
    vector<int> cA(n), cB(n);
    vector<double> wA(n), wB(n);
    for (int i = 0; i < n; ++i)
    {
        const double sq = std::sqrt(mr.tl[i + 1] - mr.tl[i]);
        const double* it = std::upper_bound(m.times, m.times + nT, mr.tl[i]);
        if (it == m.times + nT) { cA[i] = nT - 1; cB[i] = nT - 1; wA[i] = sq; wB[i] = 0; }
        else if (it == m.times) { cA[i] = 0; cB[i] = 0; wA[i] = sq; wB[i] = 0; }
        else
        {
            const int k = int(it - m.times) - 1;
            const double t = (mr.tl[i] - m.times[k]) / (m.times[k + 1] - m.times[k]);
            cA[i] = k; cB[i] = k + 1; wA[i] = sq * (1.0 - t); wB[i] = sq * t;
        }
    }
    vector<double> aY(size_t(n) * nS, 0.0);
    auto rng = makeRng(sobol, s1, s2, n);
    if (first) rng->skipTo(first);
    vector<double> g(n), xs(n + 1), S(pd.timeline.size()), aS(pd.timeline.size());
    vector<int> evStep(pd.timeline.size());
    {
        size_t idx = 0;
        for (int i = 0; i <= n; ++i)
            if (mr.common[i]) evStep[idx++] = i;
    }
    const int nPay = nPayoffs(p);
    vector<double> pay(nPay);
    vector<Sample<double>> path(pd.timeline.size());
    double aSpot = 0.0;
    for (uint64_t pth = 0; pth < count; ++pth)
    {
        rng->nextG(g.data());
        double x = std::log(m.spot);
        xs[0] = x;
        for (int i = 0; i < n; ++i)
        {
            const double v = interp<false>(X, nS, &mr.iv[size_t(i) * nS], x);
            x += v * (-0.5 * v + g[i]);
            xs[i + 1] = x;
        }
        for (size_t e = 0; e < evStep.size(); ++e)
        {
            S[e] = std::exp(xs[evStep[e]]);
            path[e] = {1.0, S[e], 1.0};
        }
        payoffs(p, estr, path.data(), path.size(), pay.data());
        double agg = 0.0;
        for (int k = 0; k < nPay; ++k)
        {
            paySum[k] += pay[k];
            agg += w[k] * pay[k];
        }
        *aggSum += agg;
        // product adjoint: dAgg/dS_e
        std::fill(aS.begin(), aS.end(), 0.0);
        const size_t nEv = S.size();
        if (p.kind == 0)
        {
            if (S[0] > p.strike) aS[0] = w[0];
        }
        else if (p.kind == 1)
        {
            const double sm = p.smooth <= 0 ? kEps : p.smooth;
            const double smooth = S[0] * sm, two = 2 * smooth, bs = p.barrier + smooth, ms = p.barrier - smooth;
            double alive = 1.0;
            bool dead = false;
            vector<double> before(nEv, 1.0);
            for (size_t e = 0; e < nEv; ++e)
            {
                before[e] = alive;
                if (S[e] > bs) { dead = true; break; }
                if (S[e] > ms) alive *= (bs - S[e]) / two;
            }
            const double fin = S[nEv - 1];
            const double euro = p.callput ? std::max(p.strike - fin, 0.0) : std::max(fin - p.strike, 0.0);
            const double dEuro = p.callput ? (p.strike - fin > 0.0 ? -1.0 : 0.0) : (fin - p.strike > 0.0 ? 1.0 : 0.0);
            const double aEuro = dead ? w[1] : w[0] * alive + w[1];
            aS[nEv - 1] += aEuro * dEuro;
            if (!dead)
            {
                double aAlive = w[0] * euro;
                for (size_t e = nEv; e-- > 0;)
                    if (S[e] > ms)
                    {
                        const double f = (bs - S[e]) / two;
                        aS[e] += aAlive * before[e] * (-1.0 / two);
                        aAlive *= f;
                    }
            }
        }
        else
        {
            size_t k = 0;
            for (size_t e = 0; e < nEv; ++e)
                for (double K : estr[e])
                {
                    if (S[e] - K > 0.0) aS[e] += w[k];
                    ++k;
                }
        }
        // reverse sweep over steps
        double ax = 0.0;
        size_t e = nEv;
        for (int i = n; i >= 0; --i)
        {
            if (e > 0 && evStep[e - 1] == i)
            {
                --e;
                ax += aS[e] * S[e];
            }
            if (i == 0) break;
            const int s = i - 1;
            const double xi = xs[s];
            const double* Y = &mr.iv[size_t(s) * nS];
            const double* it = std::upper_bound(X, X + nS, xi);
            double v, slope = 0.0, t = 0.0;
            int k;
            if (it == X + nS) { k = nS - 1; v = Y[k]; }
            else if (it == X) { k = 0; v = Y[0]; }
            else
            {
                k = int(it - X) - 1;
                t = (xi - X[k]) / (X[k + 1] - X[k]);
                v = Y[k] + (Y[k + 1] - Y[k]) * t;
                slope = (Y[k + 1] - Y[k]) * invdX[k];
            }
            const double q = g[s] - v;
            const double av = ax * q;
            ax += av * slope;
            if (it == X + nS || it == X) aY[size_t(s) * nS + k] += av;
            else
            {
                aY[size_t(s) * nS + k] += av * (1.0 - t);
                aY[size_t(s) * nS + k + 1] += av * t;
            }
        }
        aSpot += ax / m.spot;
    }
    risk[0] += aSpot;
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < nS; ++j)
        {
            const double a = aY[size_t(i) * nS + j];
            if (a == 0.0) continue;
            risk[1 + size_t(j) * nT + cA[i]] += a * wA[i];
            if (wB[i] != 0.0) risk[1 + size_t(j) * nT + cB[i]] += a * wB[i];
        }
}

// ---------------------------------------------------------------------------------------
// Calibration: IVS::call / localVol (ivs.h:103-138), dupireCalibMaturity / dupireCalib
// (mcMdlDupire.h:285-388), blackScholes / blackScholesIvol / merton (analytics.h:8-91).
// ---------------------------------------------------------------------------------------
template <class T>
T blackScholes(double spot, double strike, const T& vol, double mat)
{
    const T std_ = vol * std::sqrt(mat);
    if (val(std_) <= kEps) return T(std::max(0.0, spot - strike));
    const T d2 = std::log(spot / strike) / std_ - 0.5 * std_;
    const T d1 = d2 + std_;
    return spot * normalCdf(d1) - strike * normalCdf(d2);
}

double blackScholesIvol(double spot, double strike, double prem, double mat)
{
    if (prem <= std::max(0.0, spot - strike) + kEps) return 0.0;
    double u = 0.5;
    while (blackScholes(spot, strike, u, mat) < prem) u *= 2;
    double l = 0.05;
    while (blackScholes(spot, strike, l, mat) > prem) l /= 2;
    double pu = blackScholes(spot, strike, u, mat);
    double pl = blackScholes(spot, strike, l, mat);
    while (u - l > 1.e-12)
    {
        const double mid = 0.5 * (u + l);
        const double pm = blackScholes(spot, strike, mid, mat);
        if (pm > prem) { u = mid; pu = pm; }
        else { l = mid; pl = pm; }
    }
    return l + (prem - pl) / (pu - pl) * (u - l);
}

double merton(double spot, double strike, double vol, double mat, double intens, double meanJmp, double stdJmp)
{
    const double varJmp = stdJmp * stdJmp, mv2 = meanJmp + 0.5 * varJmp, comp = intens * (std::exp(mv2) - 1),
                 var = vol * vol, intensT = intens * mat;
    unsigned fact = 1;
    double iT = 1.0, result = 0.0;
    for (size_t n = 0; n < 10; ++n)
    {
        const double s = spot * std::exp(n * mv2 - comp * mat);
        const double v = std::sqrt(var + n * varJmp / mat);
        const double prob = std::exp(-intensT) * iT / fact;
        result += prob * blackScholes(s, strike, v, mat);
        fact *= unsigned(n + 1);
        iT *= intensT;
    }
    return result;
}

double impliedVol(const orc_ivs& s, double K, double T)
{
    if (s.kind == 0)
    {
        const double l = std::log(K / s.p[3]);
        return s.p[0] + s.p[1] * l * l / std::sqrt(T) + s.p[2] * l;
    }
    return blackScholesIvol(s.spot, K, merton(s.spot, K, s.p[0], T, s.p[1], s.p[2], s.p[3]), T);
}

template <class T>
struct RiskViewT
{
    bool empty = true;
    vector<double> strikes, mats;
    vector<T> spreads;
    T spread(double K, double t) const
    {
        return empty ? T(0.0) : interp2DSmooth(strikes, mats, spreads, K, t);
    }
};

template <class T>
T ivsCall(const orc_ivs& s, double K, double mat, const RiskViewT<T>* rv)
{
    return blackScholes<T>(s.spot, K, impliedVol(s, K, mat) + (rv ? rv->spread(K, mat) : T(0.0)), mat);
}

template <class T>
T localVol(const orc_ivs& s, double K, double mat, const RiskViewT<T>* rv)
{
    const T c00 = ivsCall(s, K, mat, rv);
    const T c01 = ivsCall(s, K, mat - 1.0e-04, rv);
    const T c02 = ivsCall(s, K, mat + 1.0e-04, rv);
    const T ct = (c02 - c01) * 0.5e04;
    const T c10 = ivsCall(s, K - 1.0e-04, mat, rv);
    const T c20 = ivsCall(s, K + 1.0e-04, mat, rv);
    const T ckk = (c10 + c20 - 2.0 * c00) * 1.0e08;
    return sqrt(2.0 * ct / ckk) / K;
}

// d blackScholes / d vol by the tape's rules (normalCdf' = normalDens, AADExpr.h:434-447), on a
// tape of its own.
double bsVegaTape(double spot, double K, double vol, double mat)
{
    Tape* outer = gTape;
    Tape t;
    gTape = &t;
    const Var v = leaf(vol);
    const Var c = blackScholes<Var>(spot, K, v, mat);
    t.sizeAdj();
    if (c.i >= 0)
    {
        t.adj[size_t(c.i)] = 1.0;
        t.sweep(t.nodes.size(), 0);
    }
    const double d = t.adj[size_t(v.i)];
    gTape = outer;
    return d;
}

// IVS::localVol (ivs.h:119-138) on the tape with each of its five calls recorded as one node of
// its implied vol (plus the risk view's spread): value c and partial d c / d vol, the oracle's
// own (own, ownV receive them) or given ones.  Dupire's formula and its partials are then taken at
// those values.  The points are, in this order, (K,T), (K,T-h), (K,T+h), (K-h,T), (K+h,T), h = 1e-4.
Var localVolPoints(const orc_ivs& s, double K, double mat, const RiskViewT<Var>* rv, const double* given,
                   const double* givenV, double* own, double* ownV, int* volNode)
{
    const double Kp[5] = {K, K, K, K - 1.0e-04, K + 1.0e-04};
    const double Tp[5] = {mat, mat - 1.0e-04, mat + 1.0e-04, mat, mat};
    Var c[5];
    for (int k = 0; k < 5; ++k)
    {
        const Var vol = impliedVol(s, Kp[k], Tp[k]) + rv->spread(Kp[k], Tp[k]);
        const double cv = blackScholes<double>(s.spot, Kp[k], vol.v, Tp[k]);
        const double dv = bsVegaTape(s.spot, Kp[k], vol.v, Tp[k]);
        if (own) own[k] = cv;
        if (ownV) ownV[k] = dv;
        c[k] = un(given ? given[k] : cv, vol, givenV ? givenV[k] : dv);
        if (volNode) volNode[k] = vol.i;
    }
    const Var ct = (c[2] - c[1]) * 0.5e04;
    const Var ckk = (c[3] + c[4] - 2.0 * c[0]) * 1.0e08;
    return sqrt(2.0 * ct / ckk) / K;
}

struct CalibGrid
{
    vector<double> spots, times;
};

CalibGrid calibGrid(const double* inclSpots, int nIS, double maxDs, const double* inclTimes, int nIT, double maxDtVol)
{
    CalibGrid g;
    g.spots = fillData(vector<double>(inclSpots, inclSpots + nIS), maxDs, 0.01);
    g.times = fillData(vector<double>(inclTimes, inclTimes + nIT), maxDtVol, kOneHour, &maxDtVol, &maxDtVol + 1);
    return g;
}

// The five calls and vegas of each node for localVolPoints, at [(j nS + i) 5, +5) of each array
// (node: spot i, time j); null arrays: the oracle's own values, not recorded.
struct CalibPoints
{
    const double *calls, *vegas;
    double *ownCalls, *ownVegas;
    int* volNode;  // tape node of each point's implied vol
};

// lvols spot-major [nS][nT]; with points (T = Var) each node through localVolPoints
template <class T>
vector<T> calibrate(const orc_ivs& s, const CalibGrid& g, const RiskViewT<T>& rv, const CalibPoints* points = nullptr)
{
    const size_t nS = g.spots.size(), nT = g.times.size();
    vector<T> lv(nS * nT);
    for (size_t j = 0; j < nT; ++j)
    {
        const double mat = g.times[j];
        const double atm = ivsCall<double>(s, s.spot, mat, nullptr);
        const double sd = atm * 2.506628274631;
        int il = 0;
        while (il < int(nS) && g.spots[il] < s.spot - 2.5 * sd) ++il;
        int ih = int(nS) - 1;
        while (ih >= 0 && g.spots[ih] > s.spot + 2.5 * sd) --ih;
        for (int i = il; i <= ih; ++i)
        {
            if constexpr (std::is_same_v<T, Var>)
                if (points)
                {
                    const size_t c5 = (j * nS + size_t(i)) * 5;
                    auto at = [&](auto* a) { return a ? a + c5 : nullptr; };
                    lv[i * nT + j] = localVolPoints(s, g.spots[i], mat, &rv, at(points->calls), at(points->vegas),
                                                    at(points->ownCalls), at(points->ownVegas), at(points->volNode));
                    continue;
                }
            lv[i * nT + j] = localVol<T>(s, g.spots[i], mat, &rv);
        }
        for (int i = 0; i < il; ++i) lv[i * nT + j] = lv[il * nT + j];
        for (int i = ih + 1; i < int(nS); ++i) lv[i * nT + j] = lv[ih * nT + j];
    }
    return lv;
}

}  // namespace

// =======================================================================================
// C API
// =======================================================================================

namespace {

// ---------------------------------------------------------------------------------------
// Multiple correlated assets, displaced Black-Scholes dynamics with proportional dividends
// (mcMdlMultiDisplaced.h:28-717, Cholesky of choldc.h:8-49), with the products Baskets
// and Autocall (mcPrdMulti.h:181-439).  Generic in T (double, or Var on the tape).
// ---------------------------------------------------------------------------------------
enum MdDyn { MD_LOG = 0, MD_NORMAL = 1, MD_SUR = 2, MD_SUB = 3 };
inline double mSqrt(double x) { return std::sqrt(x); }
inline Var mSqrt(const Var& x) { return sqrt(x); }

// Product timeline and numeraire flags (mcPrdMulti.h:201-216, 301-316).
vector<double> mTimeline(const orc_mproduct& p)
{
    if (p.kind == 0) return {p.maturity};
    vector<double> tl;
    double t = 0.0;
    const double dt = p.maturity / p.periods;
    for (int k = 0; k < p.periods; ++k)
    {
        t += dt;
        tl.push_back(t);
    }
    return tl;
}

int mPayoffs(const orc_mproduct& p) { return p.kind == 0 ? p.nK : 1; }
size_t mParams(const orc_mmodel& m)
{
    const size_t n = size_t(m.nA);
    return 1 + 2 * n + n * size_t(m.nDiv) + 2 * n + n * (n - 1) / 2 + 1;
}

template <class T>
struct MdRun
{
    const orc_mmodel* m;
    vector<double> ptl;  // product timeline
    vector<double> tl;   // simulation timeline: today + product dates after today
    bool todayOn = false;
    vector<T> params;
    // parameters, by role (copies of params entries)
    T disc, lambda;
    vector<T> spot, spread, atm, skew, divs, correl;  // divs [nDiv][nA], correl [nA][nA] lower
    // init outputs
    vector<T> chol, stds, drifts, ffs, alphas, nums;
    vector<int> dyn;

    void allocate(const orc_mmodel& mm, const orc_mproduct& p)  // mcMdlMultiDisplaced.h:367-405
    {
        m = &mm;
        ptl = mTimeline(p);
        tl = {0.0};
        for (double t : ptl)
            if (t > 0.0) tl.push_back(t);
        todayOn = ptl[0] == 0.0;
    }
    size_t nSteps() const { return tl.size() - 1; }

    // Parameter order of the reference (mcMdlMultiDisplaced.h:146-209).
    void putParams(bool onTape)
    {
        const int n = m->nA;
        params.clear();
        auto mk = [&](double x) {
            params.push_back(onTape ? T(leafOf(x)) : T(x));
            return params.back();
        };
        disc = mk(m->disc);
        spot.clear(); spread.clear(); atm.clear(); skew.clear(); divs.clear();
        for (int a = 0; a < n; ++a) spot.push_back(mk(m->spots[a]));
        for (int a = 0; a < n; ++a) spread.push_back(mk(m->spreads[a]));
        for (int d = 0; d < m->nDiv; ++d)
            for (int a = 0; a < n; ++a) divs.push_back(mk(m->divs[size_t(d) * n + a]));
        for (int a = 0; a < n; ++a) atm.push_back(mk(m->atms[a]));
        for (int a = 0; a < n; ++a) skew.push_back(mk(m->skews[a]));
        correl.assign(size_t(n) * n, T(0.0));
        for (int i = 1; i < n; ++i)
            for (int j = 0; j < i; ++j) correl[size_t(i) * n + j] = mk(m->correl[size_t(i) * n + j]);
        lambda = mk(m->lambda);
    }
    static T leafOf(double x);

    void init()  // mcMdlMultiDisplaced.h:407-566
    {
        const int n = m->nA;
        vector<T> repo(n), beta(n);
        for (int a = 0; a < n; ++a) repo[a] = disc - spread[a];
        alphas.assign(n, T(0.0));
        dyn.assign(n, MD_LOG);
        for (int a = 0; a < n; ++a)  // displacement from ATM and skew (mcMdlMultiDisplaced.h:418-444)
        {
            beta[a] = atm[a] + 2 * skew[a];
            if (std::fabs(val(skew[a])) < 1.0e-05)
            {
                dyn[a] = MD_LOG;
                alphas[a] = T(0.0);
            }
            else if (std::fabs(val(beta[a])) < 1.0e-05)
            {
                dyn[a] = MD_NORMAL;
                alphas[a] = -2 * spot[a] * skew[a];
                beta[a] = T(0.0);
            }
            else if (val(beta[a]) > 0)
            {
                dyn[a] = MD_SUR;
                alphas[a] = -2 * spot[a] / beta[a] * skew[a];
            }
            else
            {
                dyn[a] = MD_SUB;
                beta[a] = -1.0 * beta[a];
                alphas[a] = -2 * spot[a] / beta[a] * skew[a];
            }
        }
        // symmetric correl with unit diagonal, lambda shift, Cholesky (choldc.h:8-49)
        vector<T> used(size_t(n) * n);
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j)
            {
                const T raw = i == j ? T(1.0) : i > j ? correl[size_t(i) * n + j] : correl[size_t(j) * n + i];
                used[size_t(i) * n + j] = lambda * (1.0 - raw) + raw;
            }
        chol.assign(size_t(n) * n, T(0.0));
        for (int i = 0; i < n; ++i)
            for (int j = 0; j <= i; ++j)
            {
                T sum = used[size_t(i) * n + j];
                for (int k = 0; k < j; ++k) sum = sum - chol[size_t(i) * n + k] * chol[size_t(j) * n + k];
                if (i == j)
                {
                    if (val(sum) < -1.0e-15) throw std::runtime_error("choldc : matrix not positive definite");
                    if (val(sum) < 1.0e-15) sum = T(0.0);
                    chol[size_t(i) * n + i] = mSqrt(sum);
                }
                else
                    chol[size_t(i) * n + j] = std::fabs(val(chol[size_t(j) * n + j])) < 1.0e-15
                                                  ? T(0.0) : sum / chol[size_t(j) * n + j];
            }
        // per step: dividend-adjusted forward factors, stds and drifts
        const size_t ns = nSteps();
        stds.resize(ns * n);
        drifts.resize(ns * n);
        ffs.resize(ns * n);
        for (size_t i = 0; i < ns; ++i)
        {
            const double t1 = tl[i], t2 = tl[i + 1], dt = t2 - t1;
            for (int a = 0; a < n; ++a)  // mcMdlMultiDisplaced.h:343-364
            {
                T divProd(1.0);
                int d = int(std::lower_bound(m->divDates, m->divDates + m->nDiv, t1) - m->divDates);
                while (d < m->nDiv && m->divDates[d] < t2)
                {
                    divProd = divProd * (1.0 - divs[size_t(d) * n + a]);
                    ++d;
                }
                ffs[i * n + a] = divProd * exp(repo[a] * dt);
                T& sd = stds[i * n + a];
                T& dr = drifts[i * n + a];
                switch (dyn[a])
                {
                case MD_LOG: sd = beta[a] * std::sqrt(dt); dr = -0.5 * sd * sd; break;
                case MD_NORMAL: sd = alphas[a] * std::sqrt(dt); dr = T(0.0); break;
                case MD_SUR: sd = beta[a] * std::sqrt(dt); dr = -0.5 * beta[a] * beta[a] * dt; break;
                default: sd = -beta[a] * std::sqrt(dt); dr = -0.5 * beta[a] * beta[a] * dt; break;
                }
            }
        }
        // numeraires exp(r t) on the product dates (all of them ask for one); the forward
        // factors of the samples (spot(t) = forward(t, t)) are exp(repo * 0) = 1
        nums.resize(ptl.size());
        for (size_t e = 0; e < ptl.size(); ++e) nums[e] = exp(disc * ptl[e]);
    }

    // generatePath (mcMdlMultiDisplaced.h:612-662): spots[e][a] on the product dates
    void generatePath(const double* g, T* spotsOut) const
    {
        const int n = m->nA;
        vector<T> s(spot.begin(), spot.end());
        size_t idx = 0;
        if (todayOn)
        {
            for (int a = 0; a < n; ++a) spotsOut[a] = s[a];
            ++idx;
        }
        for (size_t i = 0; i < nSteps(); ++i)
        {
            const double* w = g + i * n;
            for (int a = 0; a < n; ++a)
            {
                T cw(0.0);
                for (int b = 0; b <= a; ++b) cw = cw + chol[size_t(a) * n + b] * w[b];
                const T fwd = s[a] * ffs[i * n + a];
                const T& sd = stds[i * n + a];
                const T& dr = drifts[i * n + a];
                switch (dyn[a])
                {
                case MD_LOG: s[a] = fwd * exp(dr + sd * cw); break;
                case MD_NORMAL: s[a] = fwd + sd * cw; break;
                case MD_SUR: s[a] = (fwd + alphas[a]) * exp(dr + sd * cw) - alphas[a]; break;
                default: s[a] = (fwd - alphas[a]) * exp(dr + sd * cw) + alphas[a]; break;
                }
            }
            for (int a = 0; a < n; ++a) spotsOut[idx * n + a] = s[a];
            ++idx;
        }
    }
};

template <>
double MdRun<double>::leafOf(double x) { return x; }
template <>
Var MdRun<Var>::leafOf(double x) { return leaf(x); }

template <class T>
T tmin(const T& a, double b);
template <>
double tmin(const double& a, double b) { return std::min(a, b); }
template <>
Var tmin(const Var& a, double b) { return un(std::min(a.v, b), a, a.v < b ? 1.0 : 0.0); }
inline bool lessV(double a, double b) { return a < b; }
inline bool lessV(const Var& a, const Var& b) { return a.v < b.v; }

// Payoffs (mcPrdMulti.h:266-276 Baskets, 368-416 Autocall); spots [nEv][nA], nums [nEv].
template <class T>
void mPayoffsOf(const orc_mproduct& p, const T* sp, const vector<T>& nums, T* out)
{
    const int n = p.nA;
    if (p.kind == 0)
    {
        T basket(0.0);
        for (int a = 0; a < n; ++a) basket = basket + p.weights[a] * sp[a];
        for (int k = 0; k < p.nK; ++k) out[k] = vmax(basket - p.strikes[k], 0.0) / nums[0];
        return;
    }
    const double dt = p.maturity / p.periods;
    const double smooth = std::max(p.smooth, kEps);
    T alive(1.0), pay(0.0);
    vector<T> perf(n);
    auto worstOf = [&](int e) {
        for (int a = 0; a < n; ++a) perf[a] = sp[size_t(e) * n + a] / p.refs[a];
        size_t w = 0;
        for (int a = 1; a < n; ++a)
            if (lessV(perf[a], perf[w])) w = a;
        return perf[w];
    };
    for (int e = 0; e < p.periods - 1; ++e)
    {
        const T worst = worstOf(e);
        pay = pay + alive * p.cpn * dt / nums[e];
        const T surv = alive * tmin(vmax((p.ko + smooth - worst) / 2 / smooth, 0.0), 1.0);
        const T dead = alive - surv;
        pay = pay + dead / nums[e];
        alive = surv;
    }
    const int e = p.periods - 1;
    const T worst = worstOf(e);
    pay = pay + alive * p.cpn * dt / nums[e];
    pay = pay + alive / nums[e];
    pay = pay - alive * vmax(p.strike - worst, 0.0) / p.strike / nums[e];
    out[0] = pay;
}

// Path loop for values (mcBase.h:267-308) and the tape-based risk (mcBase.h:427-532, 775-854).
void mRun(const orc_mmodel& m, const orc_mproduct& p, int sobol, unsigned s1, unsigned s2, uint64_t nPath,
          const double* weights, int mode /* 0 value, 1 aggregate risk, 2 multi risk */, double* paySum,
          double* paySq, double* aggSum, double* riskSum)
{
    const int nPay = mPayoffs(p), n = m.nA;
    const size_t nEv = mTimeline(p).size();
    if (mode == 0)
    {
        MdRun<double> mr;
        mr.allocate(m, p);
        mr.putParams(false);
        mr.init();
        const int dim = int(mr.nSteps()) * n;
        auto rng = makeRng(sobol, s1, s2, dim);
        vector<double> g(dim), sp(nEv * n), pay(nPay);
        for (uint64_t i = 0; i < nPath; ++i)
        {
            rng->nextG(g.data());
            mr.generatePath(g.data(), sp.data());
            mPayoffsOf(p, sp.data(), mr.nums, pay.data());
            for (int k = 0; k < nPay; ++k)
            {
                paySum[k] += pay[k];
                paySq[k] += pay[k] * pay[k];
            }
        }
        return;
    }
    Tape tape;
    gTape = &tape;
    MdRun<Var> mr;
    mr.allocate(m, p);
    mr.putParams(true);
    mr.init();
    tape.mark = tape.nodes.size();
    tape.width = mode == 2 ? nPay : 1;
    tape.adj.assign(tape.mark * tape.width, 0.0);
    const int dim = int(mr.nSteps()) * n;
    auto rng = makeRng(sobol, s1, s2, dim);
    vector<double> g(dim);
    vector<Var> sp(nEv * n), pay(nPay);
    for (uint64_t i = 0; i < nPath; ++i)
    {
        tape.nodes.resize(tape.mark);
        rng->nextG(g.data());
        mr.generatePath(g.data(), sp.data());
        mPayoffsOf(p, sp.data(), mr.nums, pay.data());
        for (int k = 0; k < nPay; ++k) paySum[k] += pay[k].v;
        Var agg(0.0);
        if (mode == 1)
        {
            for (int k = 0; k < nPay; ++k)
                if (weights[k] != 0.0) agg = agg + pay[k] * weights[k];
            *aggSum += agg.v;
        }
        tape.adj.resize(tape.nodes.size() * tape.width, 0.0);
        if (mode == 2)
        {
            for (int k = 0; k < nPay; ++k)
                if (pay[k].i >= 0) tape.adj[size_t(pay[k].i) * tape.width + k] += 1.0;
        }
        else if (agg.i >= 0)
            tape.adj[size_t(agg.i)] += 1.0;
        tape.sweep(tape.nodes.size(), tape.mark);
        tape.adj.resize(tape.mark * tape.width);
    }
    tape.nodes.resize(tape.mark);
    tape.sweep(tape.mark, 0);
    for (size_t j = 0; j < mr.params.size(); ++j)
        for (int w = 0; w < tape.width; ++w)
            if (mr.params[j].i >= 0) riskSum[j * tape.width + w] += tape.adj[size_t(mr.params[j].i) * tape.width + w];
    gTape = nullptr;
}

}  // namespace

extern "C" {

int orc_shapes(const orc_model* m, const orc_product* p, int* nPay, int* nParam, int* simDim)
{
    const ProductDef pd = productDef(*p);
    ModelRun<double> mr;
    mr.allocate(*m, pd);
    if (nPay) *nPay = nPayoffs(*p);
    if (nParam) *nParam = int(mr.numParams());
    if (simDim) *simDim = int(mr.simDim());
    return 0;
}

int orc_paths(const orc_model* m, const orc_product* p, int sobol, int nPath, unsigned s1, unsigned s2, double* out)
{
    runPaths(*m, *p, sobol, s1, s2, 0, uint64_t(nPath), nullptr, nullptr, out);
    return 0;
}

int orc_value(const orc_model* m, const orc_product* p, int sobol, int nPath, unsigned s1, unsigned s2, int nThreads,
              double* values, double* stderrs)
{
    const int nPay = nPayoffs(*p);
    if (nThreads <= 1)
    {
        vector<double> sum(nPay, 0.0), sq(nPay, 0.0);
        // path-order accumulation, like main.h:69-74
        runPaths(*m, *p, sobol, s1, s2, 0, uint64_t(nPath), sum.data(), sq.data(), nullptr);
        for (int k = 0; k < nPay; ++k)
        {
            values[k] = sum[k] / nPath;
            if (stderrs)
            {
                const double var = std::max(0.0, sq[k] / nPath - values[k] * values[k]);
                stderrs[k] = std::sqrt(var / nPath);
            }
        }
        return 0;
    }
    auto rg = ranges(uint64_t(nPath), nThreads);
    vector<vector<double>> sums(rg.size(), vector<double>(nPay, 0.0)), sqs(rg.size(), vector<double>(nPay, 0.0));
    vector<std::thread> th;
    for (size_t t = 0; t < rg.size(); ++t)
        th.emplace_back([&, t] {
            runPaths(*m, *p, sobol, s1, s2, rg[t].first, rg[t].second, sums[t].data(), sqs[t].data(), nullptr);
        });
    for (auto& x : th) x.join();
    for (int k = 0; k < nPay; ++k)
    {
        double s = 0, q = 0;
        for (size_t t = 0; t < rg.size(); ++t) { s += sums[t][k]; q += sqs[t][k]; }
        values[k] = s / nPath;
        if (stderrs) stderrs[k] = std::sqrt(std::max(0.0, q / nPath - values[k] * values[k]) / nPath);
    }
    return 0;
}

int orc_risk(const orc_model* m, const orc_product* p, int sobol, int nPath, unsigned s1, unsigned s2,
             const double* weights, double* values, double* aggValue, double* risks)
{
    const int nPay = nPayoffs(*p);
    int nParam;
    orc_shapes(m, p, nullptr, &nParam, nullptr);
    vector<double> paySum(nPay, 0.0), riskSum(nParam, 0.0);
    double agg = 0.0;
    runRiskTape(*m, *p, sobol, s1, s2, 0, uint64_t(nPath), weights, false, paySum.data(), &agg, riskSum.data());
    for (int k = 0; k < nPay; ++k) values[k] = paySum[k] / nPath;
    *aggValue = agg / nPath;
    for (int j = 0; j < nParam; ++j) risks[j] = riskSum[j] / nPath;
    return 0;
}

int orc_risk_multi(const orc_model* m, const orc_product* p, int sobol, int nPath, unsigned s1, unsigned s2,
                   int refMarkQuirk, double* values, double* risks)
{
    const int nPay = nPayoffs(*p);
    int nParam;
    orc_shapes(m, p, nullptr, &nParam, nullptr);
    vector<double> paySum(nPay, 0.0), riskSum(size_t(nParam) * nPay, 0.0);
    double agg = 0.0;
    runRiskTape(*m, *p, sobol, s1, s2, 0, uint64_t(nPath), nullptr, true, paySum.data(), &agg, riskSum.data(),
                refMarkQuirk != 0);
    for (int k = 0; k < nPay; ++k) values[k] = paySum[k] / nPath;
    for (size_t j = 0; j < riskSum.size(); ++j) risks[j] = riskSum[j] / nPath;
    return 0;
}

int orc_risk_fast(const orc_model* m, const orc_product* p, int sobol, int nPath, unsigned s1, unsigned s2,
                  const double* weights, int nThreads, double* values, double* aggValue, double* risks)
{
    if (m->kind != 1 || p->kind == 3) return orc_risk(m, p, sobol, nPath, s1, s2, weights, values, aggValue, risks);
    const int nPay = nPayoffs(*p);
    const size_t nParam = 1 + size_t(m->nS) * m->nT;
    auto rg = ranges(uint64_t(nPath), std::max(1, nThreads));
    vector<vector<double>> pay(rg.size(), vector<double>(nPay, 0.0)), rk(rg.size(), vector<double>(nParam, 0.0));
    vector<double> agg(rg.size(), 0.0);
    vector<std::thread> th;
    for (size_t t = 0; t < rg.size(); ++t)
        th.emplace_back([&, t] {
            runRiskFastDupire(*m, *p, sobol, s1, s2, rg[t].first, rg[t].second, weights, pay[t].data(), &agg[t],
                              rk[t].data());
        });
    for (auto& x : th) x.join();
    for (int k = 0; k < nPay; ++k)
    {
        double s = 0;
        for (auto& v : pay) s += v[k];
        values[k] = s / nPath;
    }
    double a = 0;
    for (double v : agg) a += v;
    *aggValue = a / nPath;
    for (size_t j = 0; j < nParam; ++j)
    {
        double s = 0;
        for (auto& v : rk) s += v[j];
        risks[j] = s / nPath;
    }
    return 0;
}

int orc_sobol_ints(int dim, int64_t firstPath, int nPaths, uint32_t* out)
{
    if (dim > CF_SOBOL_MAX_DIM) return -1;
    Sobol s(dim);
    s.skipTo(uint64_t(firstPath));
    for (int i = 0; i < nPaths; ++i)
    {
        s.next();
        std::memcpy(out + size_t(i) * dim, s.state.data(), sizeof(unsigned) * dim);
    }
    return 0;
}

int orc_sobol_gauss(int dim, int64_t firstPath, int nPaths, double* out)
{
    if (dim > CF_SOBOL_MAX_DIM) return -1;
    Sobol s(dim);
    s.skipTo(uint64_t(firstPath));
    for (int i = 0; i < nPaths; ++i) s.nextG(out + size_t(i) * dim);
    return 0;
}

int orc_mrg_gauss(unsigned s1, unsigned s2, int dim, int64_t firstPath, int nPaths, double* out)
{
    Mrg r(s1, s2, dim);
    r.skipTo(uint64_t(firstPath));
    for (int i = 0; i < nPaths; ++i) r.nextG(out + size_t(i) * dim);
    return 0;
}

int orc_mrg_state(unsigned s1, unsigned s2, int dim, int64_t firstPath, double* st)
{
    Mrg r(s1, s2, dim);
    r.skipTo(uint64_t(firstPath) & ~uint64_t(1));
    st[0] = r.x0; st[1] = r.x1; st[2] = r.x2; st[3] = r.y0; st[4] = r.y1; st[5] = r.y2;
    return 0;
}

double orc_inv_normal_cdf(double p) { return invNormalCdf(p); }
double orc_normal_cdf(double x) { return normalCdf(x); }

int orc_calib(const orc_ivs* ivs, const double* inclSpots, int nIS, double maxDs, const double* inclTimes, int nIT,
              double maxDtVol, int* nS, int* nT, double* spots, double* times, double* lvols)
{
    const CalibGrid g = calibGrid(inclSpots, nIS, maxDs, inclTimes, nIT, maxDtVol);
    *nS = int(g.spots.size());
    *nT = int(g.times.size());
    if (!lvols) return 0;
    std::copy(g.spots.begin(), g.spots.end(), spots);
    std::copy(g.times.begin(), g.times.end(), times);
    RiskViewT<double> rv;
    const auto lv = calibrate<double>(*ivs, g, rv);
    std::copy(lv.begin(), lv.end(), lvols);
    return 0;
}

int orc_calib_adjoint(const orc_ivs* ivs, const double* inclSpots, int nIS, double maxDs, const double* inclTimes,
                      int nIT, double maxDtVol, const double* rvK, int nK, const double* rvM, int nM,
                      const double* micro, int refSeedQuirk, double* vega)
{
    return orc_calib_adjoint_given(ivs, inclSpots, nIS, maxDs, inclTimes, nIT, maxDtVol, rvK, nK, rvM, nM, micro,
                                   refSeedQuirk, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, vega, 0);
}

int orc_calib_adjoint_given(const orc_ivs* ivs, const double* inclSpots, int nIS, double maxDs,
                            const double* inclTimes, int nIT, double maxDtVol, const double* rvK, int nK,
                            const double* rvM, int nM, const double* micro, int refSeedQuirk, const double* calls,
                            const double* vegas, double* ownCalls, double* ownVegas, double* pointAdj,
                            double* absTerms, double* vega, int pointwise)
{
    Tape tape;
    gTape = &tape;
    const CalibGrid g = calibGrid(inclSpots, nIS, maxDs, inclTimes, nIT, maxDtVol);
    RiskViewT<Var> rv;
    rv.empty = false;
    rv.strikes.assign(rvK, rvK + nK);
    rv.mats.assign(rvM, rvM + nM);
    for (int i = 0; i < nK * nM; ++i) rv.spreads.push_back(leaf(0.0));
    const size_t n5 = g.spots.size() * g.times.size() * 5;
    if (ownCalls) std::fill(ownCalls, ownCalls + n5, 0.0);
    if (ownVegas) std::fill(ownVegas, ownVegas + n5, 0.0);
    vector<int> volNode(n5, -1);
    const CalibPoints pts{calls, vegas, ownCalls, ownVegas, volNode.data()};
    const auto lv = calibrate<Var>(*ivs, g, rv, pointwise ? &pts : nullptr);
    tape.width = 1;
    tape.sizeAdj();
    // Flat-extrapolated local vols are copies of the edge node (mcMdlDupire.h:320-324), so the
    // exact adjoint adds their microbucket into that node.  The reference seeds by assignment
    // (main.h:541-547): for a shared node the last (spot-major) assignment wins.
    for (size_t i = 0; i < lv.size(); ++i)
        if (lv[i].i >= 0)
        {
            if (refSeedQuirk) tape.adj[size_t(lv[i].i)] = micro[i];
            else tape.adj[size_t(lv[i].i)] += micro[i];
        }
    tape.sweep(tape.nodes.size(), 0);
    for (int i = 0; i < nK * nM; ++i) vega[i] = tape.adj[size_t(rv.spreads[i].i)];
    if (pointwise && (pointAdj || absTerms))
    {
        // the adjoint of each point's implied vol; then, per spread node, the sum over points of
        // |that adjoint| x the point's interpolation weight on the node (the weights are >= 0): a
        // second sweep seeded with the absolute point adjoints only
        vector<double> pa(n5, 0.0);
        for (size_t k = 0; k < n5; ++k)
            if (volNode[k] >= 0) pa[k] = tape.adj[size_t(volNode[k])];
        if (pointAdj) std::copy(pa.begin(), pa.end(), pointAdj);
        if (absTerms)
        {
            std::fill(tape.adj.begin(), tape.adj.end(), 0.0);
            for (size_t k = 0; k < n5; ++k)
                if (volNode[k] >= 0) tape.adj[size_t(volNode[k])] += std::fabs(pa[k]);
            tape.sweep(tape.nodes.size(), 0);
            for (int i = 0; i < nK * nM; ++i) absTerms[i] = tape.adj[size_t(rv.spreads[i].i)];
        }
    }
    gTape = nullptr;
    return 0;
}

int orc_superbucket(const orc_ivs* ivs, double spot, double maxDt, const orc_product* p, const double* notionals,
                    const double* inclSpots, int nIS, double maxDs, const double* inclTimes, int nIT,
                    double maxDtVol, const double* rvK, int nK, const double* rvM, int nM, int sobol, int nPath,
                    unsigned s1, unsigned s2, int refSeedQuirk, double* value, double* delta, double* vega,
                    double* microOut)
{
    // main.h:453-569: calibrate, MC adjoints to local vols, calibration adjoint to the risk view.
    int nS, nT;
    orc_calib(ivs, inclSpots, nIS, maxDs, inclTimes, nIT, maxDtVol, &nS, &nT, nullptr, nullptr, nullptr);
    vector<double> spots(nS), times(nT), lv(size_t(nS) * nT);
    orc_calib(ivs, inclSpots, nIS, maxDs, inclTimes, nIT, maxDtVol, &nS, &nT, spots.data(), times.data(), lv.data());
    orc_model m{};
    m.kind = 1;
    m.spot = spot;
    m.nS = nS;
    m.nT = nT;
    m.spots = spots.data();
    m.times = times.data();
    m.vols = lv.data();
    m.maxdt = maxDt;
    const int nPay = nPayoffs(*p);
    vector<double> vals(nPay), risks(1 + size_t(nS) * nT);
    double agg;
    orc_risk(&m, p, sobol, nPath, s1, s2, notionals, vals.data(), &agg, risks.data());
    *value = agg;
    *delta = risks[0];
    if (microOut) std::copy(risks.begin() + 1, risks.end(), microOut);
    return orc_calib_adjoint(ivs, inclSpots, nIS, maxDs, inclTimes, nIT, maxDtVol, rvK, nK, rvM, nM,
                             risks.data() + 1, refSeedQuirk, vega);
}

int orc_fill(const double* x, int n, double maxDx, double minDx, const double* add, int nAdd, double* out)
{
    const auto f = nAdd ? fillData(vector<double>(x, x + n), maxDx, minDx, add, add + nAdd)
                        : fillData(vector<double>(x, x + n), maxDx, minDx);
    if (out) std::copy(f.begin(), f.end(), out);
    return int(f.size());
}

}  // extern "C"

extern "C" {

int orc_m_shapes(const orc_mmodel* m, const orc_mproduct* p, int* nPay, int* nParam, int* simDim)
{
    if (nPay) *nPay = mPayoffs(*p);
    if (nParam) *nParam = int(mParams(*m));
    MdRun<double> mr;
    mr.allocate(*m, *p);
    if (simDim) *simDim = int(mr.nSteps()) * m->nA;
    return 0;
}

int orc_m_value(const orc_mmodel* m, const orc_mproduct* p, int sobol, int nPath, unsigned s1, unsigned s2,
                double* values, double* stderrs)
{
    const int nPay = mPayoffs(*p);
    vector<double> sum(nPay, 0.0), sq(nPay, 0.0);
    try
    {
        mRun(*m, *p, sobol, s1, s2, uint64_t(nPath), nullptr, 0, sum.data(), sq.data(), nullptr, nullptr);
    }
    catch (const std::exception&)
    {
        return -1;
    }
    for (int k = 0; k < nPay; ++k)
    {
        values[k] = sum[k] / nPath;
        if (stderrs) stderrs[k] = std::sqrt(std::max(0.0, sq[k] / nPath - values[k] * values[k]) / nPath);
    }
    return 0;
}

int orc_m_risk(const orc_mmodel* m, const orc_mproduct* p, int sobol, int nPath, unsigned s1, unsigned s2,
               const double* weights, double* values, double* aggValue, double* risks)
{
    const int nPay = mPayoffs(*p);
    const size_t nParam = mParams(*m);
    vector<double> sum(nPay, 0.0), rk(nParam, 0.0);
    double agg = 0.0;
    try
    {
        mRun(*m, *p, sobol, s1, s2, uint64_t(nPath), weights, 1, sum.data(), nullptr, &agg, rk.data());
    }
    catch (const std::exception&)
    {
        return -1;
    }
    for (int k = 0; k < nPay; ++k) values[k] = sum[k] / nPath;
    *aggValue = agg / nPath;
    for (size_t j = 0; j < nParam; ++j) risks[j] = rk[j] / nPath;
    return 0;
}

int orc_m_risk_multi(const orc_mmodel* m, const orc_mproduct* p, int sobol, int nPath, unsigned s1, unsigned s2,
                     double* values, double* risks)
{
    const int nPay = mPayoffs(*p);
    const size_t nParam = mParams(*m);
    vector<double> sum(nPay, 0.0), rk(nParam * nPay, 0.0);
    try
    {
        mRun(*m, *p, sobol, s1, s2, uint64_t(nPath), nullptr, 2, sum.data(), nullptr, nullptr, rk.data());
    }
    catch (const std::exception&)
    {
        return -1;
    }
    for (int k = 0; k < nPay; ++k) values[k] = sum[k] / nPath;
    for (size_t j = 0; j < rk.size(); ++j) risks[j] = rk[j] / nPath;
    return 0;
}

int orc_m_init(const orc_mmodel* m, const orc_mproduct* p, double* chol, double* stds, double* drifts, double* ffs,
               double* alphas, int* dynamics, double* numeraires)
{
    MdRun<double> mr;
    mr.allocate(*m, *p);
    mr.putParams(false);
    try
    {
        mr.init();
    }
    catch (const std::exception&)
    {
        return -1;
    }
    std::copy(mr.chol.begin(), mr.chol.end(), chol);
    std::copy(mr.stds.begin(), mr.stds.end(), stds);
    std::copy(mr.drifts.begin(), mr.drifts.end(), drifts);
    std::copy(mr.ffs.begin(), mr.ffs.end(), ffs);
    std::copy(mr.alphas.begin(), mr.alphas.end(), alphas);
    std::copy(mr.dyn.begin(), mr.dyn.end(), dynamics);
    std::copy(mr.nums.begin(), mr.nums.end(), numeraires);
    return 0;
}

}  // extern "C"
