// Host-side pieces of the reference's algorithms that run once per model/product:
// grid refinement, interpolation, timelines, Sobol direction numbers, mrg32k3a jump tables.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <string>
#include <vector>

namespace cf {

constexpr double kEps = 1.0e-08;                  // gaussians.h:8
constexpr double kHalfDay = 0.00136986301369863;  // mcMdlDupire.h:26
constexpr double kOneHour = 0.000114469;          // mcPrd.h:26

// fillData, utility.h:11-79: the sorted union of `original` and `add` (points closer than
// minDx merged), then extra points so that no gap exceeds maxDx.
std::vector<double> fill_data(const std::vector<double>& original, double maxDx, double minDx,
                              const std::vector<double>& add = {});

// interp, interp.h:26-63 (linear or smoothstep, flat extrapolation) for double y.
double interp_lin(const double* x, size_t n, const double* y, double x0);

// "%.2f" as std::ostringstream << fixed << setprecision(2) prints it (mcPrd.h labels).
std::string fmt2(double x);

// Sobol direction numbers [32][dims] of the first `dims` dimensions, regenerated from the
// Joe-Kuo initialisation data with the recurrence m_k = 2a_1 m_{k-1} ^ ... ^ 2^s m_{k-s} ^ m_{k-s}.
int sobol_max_dim();
std::vector<uint32_t> sobol_dirs(int dims);

// Jump tables of the two mrg32k3a recurrences (matrices A mod m1 and B mod m2,
// mrg32k3a.h:319-358): record 16k + d holds A^(d 16^k) (B^(d 16^k)) for k = 0..15 and d = 1..15,
// row-major 3x3 in words 0..8, words 9..11 and record 16k + 0 zero.
void mrg_jump_tables(uint32_t A[256][12], uint32_t B[256][12]);

// Beasley-Springer-Moro inverse normal (gaussians.h:47-87), in double.
double inv_normal_bsm(double p);

// Piecewise-cubic table of the inverse normal for the FP32 kernels.  A draw's lower-half
// integer up in [1, 2^31] (the uniform is up / denom) is located by its leading bit (binade b
// = 31 - clz(up), 32 of them) and the next INVN_SUB_BITS bits (sub-interval); within the
// piece, z in [0, 1) is the fraction of the remaining bits.  Entry 4*(b * 2^SUB + sub) + k is
// the coefficient of z^k of the cubic through the inverse normal at four Chebyshev nodes of
// the piece (max error 1.2e-8 against the double-precision function).  The value is the
// lower-half Gaussian (negative); the upper half is its negation.
constexpr int INVN_SUB_BITS = 4;
constexpr int INVN_PIECES = 32 << INVN_SUB_BITS;
void inv_normal_table(double denom, float* out /* [INVN_PIECES][4] */);

// Equal buckets over the log-spot knots of the FP32 Dupire kernels: bucket b is
// [x0 + b / invW, x0 + (b + 1) / invW) and first[b] the index of the first knot above its left
// edge (the upper_bound of the edge).  ok: every bucket holds at most one knot (buckets
// narrower than 2/3 of the smallest knot spacing, at most 4096 of them).  oneCompare: besides,
// no knot lies within eps = 8 x 2^-23 x the span of a bucket edge, so the bucket index of a
// state x computed in FP32, (x - x0) invW, is exact or one off next to an edge with no knot
// near; then upper_bound(x) = first[b] + (knot first[b] <= x), one comparison.  Without
// oneCompare the grid is the default one (from the first knot), searched with two comparisons.
struct BucketGrid
{
    bool ok = false, oneCompare = false;
    float x0 = 0.0f, invW = 1.0f;
    std::vector<int> first;
};
BucketGrid bucket_grid(const std::vector<float>& knots);

// Black-Scholes formula, Zelen-Severo normal CDF, implied vol, Merton (analytics.h:8-91).
double normal_cdf(double x);
double normal_dens(double x);
double black_scholes(double spot, double strike, double vol, double mat);
double black_scholes_ivol(double spot, double strike, double prem, double mat);
double merton_price(double spot, double strike, double vol, double mat, double intens, double meanJmp,
                    double stdJmp);

}  // namespace cf
