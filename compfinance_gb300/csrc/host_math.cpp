// Host-side pieces of the reference's algorithms (see host_math.h).  Compiled with
// -ffp-contract=off so the double arithmetic rounds exactly like the reference's.
#include "host_math.h"

#include <charconv>
#include <cstdio>
#include <system_error>
#include <iterator>

namespace cf {

std::vector<double> fill_data(const std::vector<double>& original, double maxDx, double minDx,
                              const std::vector<double>& add)
{
    std::vector<double> seq;
    if (!add.empty())
        std::set_union(original.begin(), original.end(), add.begin(), add.end(), std::back_inserter(seq),
                       [minDx](double x, double y) { return x < y - minDx; });
    else
        seq = original;
    std::vector<double> out;
    if (seq.empty()) return out;
    out.push_back(seq[0]);
    for (size_t i = 1; i < seq.size(); ++i)
    {
        const double cur = out.back(), nxt = seq[i];
        if (nxt - cur > maxDx)
        {
            const int n = int((nxt - cur) / maxDx - kEps) + 1;
            const double h = (nxt - cur) / n;
            for (double t = cur + h; t < nxt - minDx; t += h) out.push_back(t);
        }
        out.push_back(nxt);
    }
    return out;
}

double interp_lin(const double* x, size_t n, const double* y, double x0)
{
    const double* it = std::upper_bound(x, x + n, x0);
    if (it == x + n) return y[n - 1];
    if (it == x) return y[0];
    const size_t k = size_t(it - x) - 1;
    const double t = (x0 - x[k]) / (x[k + 1] - x[k]);
    return y[k] + (y[k + 1] - y[k]) * t;
}

// "%.2f" (correctly rounded, as printf; to_chars avoids the locale and format parsing)
std::string fmt2(double x)
{
    char b[400];
    const auto r = std::to_chars(b, b + sizeof b, x, std::chars_format::fixed, 2);
    if (r.ec != std::errc())
    {
        std::snprintf(b, sizeof b, "%.2f", x);
        return b;
    }
    return std::string(b, r.ptr);
}

namespace {
struct JKInit
{
    int s, a;
    unsigned m[13];
};
const JKInit kJK[] = {
#include "../data/sobol_joe_kuo.inc"
};
}  // namespace

int sobol_max_dim() { return CF_SOBOL_MAX_DIM; }

std::vector<uint32_t> sobol_dirs(int dims)
{
    std::vector<uint32_t> d(size_t(32) * dims);
    for (int dim = 0; dim < dims; ++dim)
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
        for (int k = 0; k < 32; ++k) d[size_t(k) * dims + dim] = uint32_t(m[k] << (31 - k));
    }
    return d;
}

static void matmul_mod(const uint64_t a[9], const uint64_t b[9], uint64_t m, uint64_t r[9])
{
    uint64_t t[9];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
        {
            unsigned __int128 s = 0;
            for (int l = 0; l < 3; ++l) s += (unsigned __int128)a[3 * i + l] * b[3 * l + j];
            t[3 * i + j] = uint64_t(s % m);
        }
    std::copy(t, t + 9, r);
}

void mrg_jump_tables(uint32_t A[256][12], uint32_t B[256][12])
{
    const uint64_t m1 = 4294967087ULL, m2 = 4294944443ULL;
    const uint64_t a[9] = {0, 1403580, m1 - 810728, 1, 0, 0, 0, 1, 0};
    const uint64_t b[9] = {527612, 0, m2 - 1370589, 1, 0, 0, 0, 1, 0};
    auto fill = [](const uint64_t* g, uint64_t m, uint32_t T[256][12]) {
        uint64_t p[9];  // g^(16^k)
        std::copy(g, g + 9, p);
        for (int k = 0; k < 16; ++k)
        {
            uint64_t q[9];  // g^(d 16^k)
            std::copy(p, p + 9, q);
            std::fill(T[16 * k], T[16 * k] + 12, 0u);
            for (int d = 1; d < 16; ++d)
            {
                for (int i = 0; i < 12; ++i) T[16 * k + d][i] = i < 9 ? uint32_t(q[i]) : 0u;
                matmul_mod(q, p, m, q);
            }
            std::copy(q, q + 9, p);  // g^(16^(k+1))
        }
    };
    fill(a, m1, A);
    fill(b, m2, B);
}

double normal_dens(double x) { return x < -10.0 || 10.0 < x ? 0.0 : std::exp(-0.5 * x * x) / 2.506628274631; }

double normal_cdf(double x)
{
    if (x < -10.0) return 0.0;
    if (x > 10.0) return 1.0;
    if (x < 0.0) return 1.0 - normal_cdf(-x);
    const double t = 1.0 / (1.0 + 0.2316419 * x);
    const double pol =
        t * (0.319381530 + t * (-0.356563782 + t * (1.781477937 + t * (-1.821255978 + t * 1.330274429))));
    return 1.0 - normal_dens(x) * pol;
}

double black_scholes(double spot, double strike, double vol, double mat)
{
    const double sd = vol * std::sqrt(mat);
    if (sd <= kEps) return std::max(0.0, spot - strike);
    const double d2 = std::log(spot / strike) / sd - 0.5 * sd;
    const double d1 = d2 + sd;
    return spot * normal_cdf(d1) - strike * normal_cdf(d2);
}

double black_scholes_ivol(double spot, double strike, double prem, double mat)
{
    if (prem <= std::max(0.0, spot - strike) + kEps) return 0.0;
    double u = 0.5;
    while (black_scholes(spot, strike, u, mat) < prem) u *= 2;
    double l = 0.05;
    while (black_scholes(spot, strike, l, mat) > prem) l /= 2;
    double pu = black_scholes(spot, strike, u, mat), pl = black_scholes(spot, strike, l, mat);
    while (u - l > 1.e-12)
    {
        const double m = 0.5 * (u + l), pm = black_scholes(spot, strike, m, mat);
        if (pm > prem) { u = m; pu = pm; }
        else { l = m; pl = pm; }
    }
    return l + (prem - pl) / (pu - pl) * (u - l);
}

double merton_price(double spot, double strike, double vol, double mat, double intens, double meanJmp,
                    double stdJmp)
{
    const double varJmp = stdJmp * stdJmp, mv2 = meanJmp + 0.5 * varJmp, comp = intens * (std::exp(mv2) - 1),
                 var = vol * vol, intensT = intens * mat;
    unsigned fact = 1;
    double iT = 1.0, res = 0.0;
    for (size_t n = 0; n < 10; ++n)
    {
        const double s = spot * std::exp(n * mv2 - comp * mat), v = std::sqrt(var + n * varJmp / mat);
        res += std::exp(-intensT) * iT / fact * black_scholes(s, strike, v, mat);
        fact *= unsigned(n + 1);
        iT *= intensT;
    }
    return res;
}

double inv_normal_bsm(double p)
{
    const bool sup = p > 0.5;
    const double up = sup ? 1.0 - p : p;
    const double x = up - 0.5;
    if (std::fabs(x) < 0.42)
    {
        const double r = x * x;
        const double v = x * (((-25.44106049637 * r + 41.39119773534) * r + -18.61500062529) * r + 2.50662823884) /
                         ((((3.13082909833 * r + -21.06224101826) * r + 23.08336743743) * r + -8.47351093090) * r + 1.0);
        return sup ? -v : v;
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

void inv_normal_table(double denom, float* out)
{
    const int nSub = 1 << INVN_SUB_BITS;
    const double pi = 3.14159265358979323846;
    for (int b = 0; b < 32; ++b)
        for (int sub = 0; sub < nSub; ++sub)
        {
            // piece: up in 2^b (1 + (sub + z) / nSub), z in [0, 1)
            double z[4], y[4];
            for (int i = 0; i < 4; ++i)
            {
                z[i] = 0.5 - 0.5 * std::cos((2 * i + 1) * pi / 8.0);
                const double up = std::ldexp(1.0 + (sub + z[i]) / nSub, b);
                y[i] = inv_normal_bsm(up / denom);
            }
            // cubic through the four nodes: Vandermonde solve by Gaussian elimination
            double A[4][5];
            for (int i = 0; i < 4; ++i)
            {
                double zk = 1.0;
                for (int k = 0; k < 4; ++k)
                {
                    A[i][k] = zk;
                    zk *= z[i];
                }
                A[i][4] = y[i];
            }
            for (int c = 0; c < 4; ++c)
            {
                int piv = c;
                for (int r = c + 1; r < 4; ++r)
                    if (std::fabs(A[r][c]) > std::fabs(A[piv][c])) piv = r;
                for (int k = 0; k < 5; ++k) std::swap(A[c][k], A[piv][k]);
                for (int r = 0; r < 4; ++r)
                    if (r != c)
                    {
                        const double f = A[r][c] / A[c][c];
                        for (int k = c; k < 5; ++k) A[r][k] -= f * A[c][k];
                    }
            }
            float* o = out + 4 * (b * nSub + sub);
            for (int k = 0; k < 4; ++k) o[k] = float(A[k][4] / A[k][k]);
        }
}

BucketGrid bucket_grid(const std::vector<float>& X)
{
    BucketGrid g;
    const int nS = int(X.size());
    if (nS < 1) return g;
    if (nS == 1)  // local vol flat in spot: unit buckets, the knot in the middle of the first
    {
        g.ok = g.oneCompare = true;
        g.x0 = X[0] - 0.5f;
        g.invW = 1.0f;
        g.first = {0, 1, 1};
        return g;
    }
    double minGap = INFINITY;
    for (int j = 0; j + 1 < nS; ++j) minGap = std::min(minGap, double(X[j + 1]) - double(X[j]));
    const double range = nS > 1 ? double(X[nS - 1]) - double(X[0]) : 0.0;
    int nBf = 8;
    while (nBf < 4096 && range / nBf > minGap / 1.5) nBf *= 2;
    g.ok = nS > 1 && minGap > 0 && range / nBf <= minGap / 1.5;
    // default grid: nBf buckets from the first knot
    const double wDefault = range > 0 ? range / nBf : 1.0;
    g.x0 = X[0];
    g.invW = float(1.0 / wDefault);
    int nB = nBf;
    double w = wDefault;
    if (g.ok)
    {
        // counts 2 (nS - 1) and 3 (nS - 1) put every knot of an evenly spaced grid at the same
        // place in its bucket; then the power of two and a run of counts above the smallest
        std::vector<int> cands = {2 * (nS - 1), 3 * (nS - 1), nBf};
        const int n0 = std::max(8, int(std::ceil(1.5 * range / minGap)));
        for (int k = 0; k < 48; ++k) cands.push_back(n0 + k);
        for (size_t c = 0; c < cands.size() && !g.oneCompare; ++c)
        {
            const int N = cands[c];
            if (N < 8 || N > 4096) continue;
            const float iw = float(1.0 / (range / N));
            const double Wd = 1.0 / double(iw);  // the width the kernel's FP32 index uses
            if (Wd > minGap / 1.5) continue;
            for (double off : {0.5, 0.25, 0.75, 0.125, 0.375, 0.625, 0.875})
            {
                const float b0 = float(double(X[0]) - off * Wd);
                // two buckets past the last knot: a state above it finds no knot to compare
                const int nb = int(std::ceil((double(X[nS - 1]) - double(b0)) / Wd)) + 2;
                const double eps =
                    8.0 * std::ldexp(1.0, -23) * (double(X[nS - 1]) - double(b0) + 2.0 * Wd + std::fabs(double(b0)));
                bool fits = Wd > 10.0 * eps && nb <= 4098;
                for (int j = 0; fits && j < nS; ++j)
                {
                    const double u = (double(X[j]) - double(b0)) / Wd;
                    fits = std::min(u - std::floor(u), std::ceil(u) - u) * Wd >= eps;
                }
                if (fits)
                {
                    g.x0 = b0;
                    g.invW = iw;
                    nB = nb;
                    w = Wd;
                    g.oneCompare = true;
                    break;
                }
            }
        }
    }
    g.first.resize(size_t(nB));
    for (int b = 0; b < nB; ++b)
    {
        const double edge = double(g.x0) + b * w;
        g.first[size_t(b)] =
            int(std::upper_bound(X.begin(), X.end(), edge, [](double e, float x) { return e < double(x); }) - X.begin());
    }
    return g;
}

}  // namespace cf
