// Device building blocks of the Monte Carlo kernels: fixed-point accumulation, the
// mrg32k3a recurrence and its jump-ahead in integer arithmetic, Sobol points, the
// Beasley-Springer-Moro inverse normal, and bounded-wait bulk copies into shared memory.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "cf_params.h"

namespace cf {

// ---------------------------------------------------------------------------------------
// Fixed-point accumulation (see cf_params.h).
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ void fix_split(double v, long long& hi, long long& lo)
{
    hi = __double2ll_rn(v * 1048576.0);               // units of 2^-20
    const double r = v - (double)hi * (1.0 / 1048576.0);  // exact (Sterbenz)
    lo = __double2ll_rn(r * 1152921504606846976.0);    // units of 2^-60
}

// FP32 values are split with integer operations only (float <-> int64 conversions are slow
// on this part): v = m 2^s with a 24-bit mantissa m, hi = trunc(v 2^20), lo = the remaining
// bits in units of 2^-60.  Exact whenever |v| >= 2^-36; below that lo truncates (< 2^-60).
__device__ __forceinline__ void fix_split(float v, long long& hi, long long& lo)
{
    const unsigned b = __float_as_uint(v);
    const int E = int((b >> 23) & 0xffu);
    if (E == 0)
    {
        hi = lo = 0;  // zero and subnormals (< 2^-126)
        return;
    }
    const long long m = (long long)((b & 0x7fffffu) | 0x800000u);
    const int s = E - 150;  // v = +-m 2^s
    long long h, l;
    if (s + 20 >= 0)
    {
        h = m << (s + 20 < 39 ? s + 20 : 39);  // |v| >= 2^42 saturates (outside the hi range)
        l = 0;
    }
    else if (s + 60 >= 0)
    {
        const int r = -(s + 20);  // 1..40 bits below the 2^-20 unit
        h = r < 64 ? (m >> r) : 0;
        l = (m & ((1LL << r) - 1)) << (s + 60);
    }
    else
    {
        h = 0;
        l = -(s + 60) < 64 ? (m >> (-(s + 60))) : 0;
    }
    const bool neg = b >> 31;
    hi = neg ? -h : h;
    lo = neg ? -l : l;
}

template <class Real>
__device__ __forceinline__ void fix_add(long long* slot, Real v)
{
    long long hi, lo;
    fix_split(v, hi, lo);
    if (hi) atomicAdd(reinterpret_cast<unsigned long long*>(slot), (unsigned long long)hi);
    if (lo) atomicAdd(reinterpret_cast<unsigned long long*>(slot + 1), (unsigned long long)lo);
}

// A node slab word in units of 2^-NODE_SHIFT, added exactly into a global hi/lo pair.
__device__ __forceinline__ void node_flush(long long* g, long long n)
{
    if (!n) return;
    const long long hi = n >> (NODE_SHIFT - FIX_HI_SHIFT);
    const long long lo = (n - (hi << (NODE_SHIFT - FIX_HI_SHIFT))) << (FIX_LO_SHIFT - NODE_SHIFT);
    if (hi) atomicAdd(reinterpret_cast<unsigned long long*>(g), (unsigned long long)hi);
    if (lo) atomicAdd(reinterpret_cast<unsigned long long*>(g + 1), (unsigned long long)lo);
}

// Block slab -> global accumulators; lo is normalised into hi first so that the global
// lo word stays far from overflow.
__device__ __forceinline__ void fix_flush(long long* g, const long long* s)
{
    long long hi = s[0], lo = s[1];
    const long long carry = lo >> FIX_CARRY_SHIFT;
    hi += carry;
    lo -= carry << FIX_CARRY_SHIFT;
    if (hi) atomicAdd(reinterpret_cast<unsigned long long*>(g), (unsigned long long)hi);
    if (lo) atomicAdd(reinterpret_cast<unsigned long long*>(g + 1), (unsigned long long)lo);
}

__host__ __device__ __forceinline__ double fix_value(long long hi, long long lo)
{
    return (double)hi * (1.0 / 1048576.0) + (double)lo * (1.0 / 1152921504606846976.0);
}

// ---------------------------------------------------------------------------------------
// mrg32k3a (L'Ecuyer), integer form of mrg32k3a.h:55-81.  The reference computes the
// recurrences in doubles whose products stay below 2^53, so every value is an exact
// integer and this uint64 arithmetic produces the same states bit for bit.
// ---------------------------------------------------------------------------------------
constexpr unsigned long long MRG_M1 = 4294967087ULL;
constexpr unsigned long long MRG_M2 = 4294944443ULL;
constexpr unsigned long long MRG_A12 = 1403580ULL, MRG_A13 = 810728ULL;
constexpr unsigned long long MRG_A21 = 527612ULL, MRG_A23 = 1370589ULL;
constexpr unsigned long long MRG_C1 = 209ULL;    // 2^32 mod m1
constexpr unsigned long long MRG_C2 = 22853ULL;  // 2^32 mod m2

struct MrgState
{
    unsigned x0, x1, x2, y0, y1, y2;  // x0 newest (reference: myXn, myXn1, myXn2)
};

// p mod m1 for p < 2^54 with 32-bit multiply-adds: 2^32 = 209 (mod m1).
__device__ __forceinline__ unsigned mrg_mod1(unsigned long long p)
{
    const unsigned long long t = (unsigned long long)(unsigned)(p >> 32) * 209u + (unsigned)p;  // < 2^32 + 2^30
    unsigned r = (unsigned)t + (unsigned)(t >> 32) * 209u;                                     // < 2^32
    return r >= 4294967087u ? r - 4294967087u : r;
}

// p mod m2 for p < 2^54: 2^32 = 22853 (mod m2).
__device__ __forceinline__ unsigned mrg_mod2(unsigned long long p)
{
    unsigned long long t = (unsigned long long)(unsigned)(p >> 32) * 22853u + (unsigned)p;  // < 2^37 + 2^32
    t = (unsigned long long)(unsigned)(t >> 32) * 22853u + (unsigned)t;                      // < 2^32 + 2^20
    unsigned r = (unsigned)t + (unsigned)(t >> 32) * 22853u;                                 // < 2^32
    return r >= 4294944443u ? r - 4294944443u : r;
}

// Next integer difference d in [1, m1]; the reference's uniform is d / (m1 + 1).
__device__ __forceinline__ unsigned mrg_next(MrgState& s)
{
    const unsigned xn = mrg_mod1((unsigned long long)s.x1 * 1403580u + (unsigned long long)(4294967087u - s.x2) * 810728u);
    const unsigned yn = mrg_mod2((unsigned long long)s.y0 * 527612u + (unsigned long long)(4294944443u - s.y2) * 1370589u);
    s.x2 = s.x1; s.x1 = s.x0; s.x0 = xn;
    s.y2 = s.y1; s.y1 = s.y0; s.y0 = yn;
    return xn > yn ? xn - yn : xn + (unsigned)(MRG_M1 - yn);
}

// Jump tables of one generator: record 16k + d (k the position of a hexadecimal digit of the
// skip, d its value, 1..15) holds M^(d 16^k) mod m, 9 words row-major and 3 words of padding
// (three 16-byte loads).  A skip of up to 64 bits takes one matrix-vector product per nonzero
// hexadecimal digit.
constexpr int MRG_JUMP_RECORD = 12;
constexpr int MRG_JUMP_RECORDS = 256;

// v <- M v mod m, m = 2^32 - C with C < 2^15 (2^32 = C mod m): each 32 x 32-bit product is
// folded once and the three of a row summed below 2^49; two more folds leave s < 2^32 + C < 2m
// and one subtraction the residue.
template <unsigned C, unsigned M>
__device__ __forceinline__ void mrg_matvec(const unsigned* rec, unsigned v[3])
{
    const uint4* r4 = reinterpret_cast<const uint4*>(rec);
    const uint4 a = __ldg(r4), b = __ldg(r4 + 1), c = __ldg(r4 + 2);
    const unsigned e[9] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w, c.x};
    unsigned r[3];
#pragma unroll
    for (int j = 0; j < 3; ++j)
    {
        unsigned long long s = 0;
#pragma unroll
        for (int l = 0; l < 3; ++l)
        {
            const unsigned long long q = (unsigned long long)e[3 * j + l] * v[l];
            s += (unsigned long long)(unsigned)(q >> 32) * C + (unsigned)q;  // < 2^47 + 2^32
        }
        s = (unsigned long long)(unsigned)(s >> 32) * C + (unsigned)s;  // < 2^33
        s = (unsigned long long)(unsigned)(s >> 32) * C + (unsigned)s;  // < 2^32 + C
        r[j] = unsigned(s >= M ? s - M : s);
    }
    v[0] = r[0]; v[1] = r[1]; v[2] = r[2];
}

// State after skipping n numbers from the seed state (mrg32k3a.h:306-394 multiplies binary
// powers of the recurrence matrices; here the powers M^(d 16^k) are precomputed tables).
__device__ __forceinline__ MrgState mrg_jump(unsigned s1, unsigned s2, unsigned long long n, const unsigned* A,
                                             const unsigned* B)
{
    unsigned x[3] = {s1, s1, s1}, y[3] = {s2, s2, s2};
    for (int k = 0; n; ++k, n >>= 4)
    {
        const int d = int(n & 15);
        if (d)
        {
            mrg_matvec<209u, 4294967087u>(A + (16 * k + d) * MRG_JUMP_RECORD, x);
            mrg_matvec<22853u, 4294944443u>(B + (16 * k + d) * MRG_JUMP_RECORD, y);
        }
    }
    return MrgState{x[0], x[1], x[2], y[0], y[1], y[2]};
}

// ---------------------------------------------------------------------------------------
// Inverse normal: Beasley-Springer-Moro, gaussians.h:47-87 (published constants).
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ double inv_normal_cdf(double p)
{
    const bool sup = p > 0.5;
    const double up = sup ? 1.0 - p : p;
    const double x = up - 0.5;
    if (fabs(x) < 0.42)
    {
        const double r = x * x;
        const double v = x * (((-25.44106049637 * r + 41.39119773534) * r + -18.61500062529) * r + 2.50662823884) /
                         ((((3.13082909833 * r + -21.06224101826) * r + 23.08336743743) * r + -8.47351093090) * r + 1.0);
        return sup ? -v : v;
    }
    double r = log(-log(up));
    r = 0.3374754822726147 +
        r * (0.9761690190917186 +
             r * (0.1607979714918209 +
                  r * (0.0276438810333863 +
                       r * (0.0038405729373609 +
                            r * (0.0003951896511919 +
                                 r * (0.0000321767881768 + r * (0.0000002888167364 + r * 0.0000003960315187)))))));
    return sup ? r : -r;
}

// FP32 form: the caller passes up = min(p, 1-p) computed from the integer draw (so the
// tails keep their bits) and which side of 1/2 the draw fell on.
__device__ __forceinline__ float inv_normal_up(float up, bool sup)
{
    const float x = up - 0.5f;
    if (fabsf(x) < 0.42f)
    {
        const float r = x * x;
        const float v = __fdividef(x * (((-25.44106049637f * r + 41.39119773534f) * r + -18.61500062529f) * r + 2.50662823884f),
                                   (((3.13082909833f * r + -21.06224101826f) * r + 23.08336743743f) * r + -8.47351093090f) * r + 1.0f);
        return sup ? -v : v;
    }
    float r = __logf(-__logf(up));
    r = 0.3374754822726147f +
        r * (0.9761690190917186f +
             r * (0.1607979714918209f +
                  r * (0.0276438810333863f +
                       r * (0.0038405729373609f +
                            r * (0.0003951896511919f +
                                 r * (0.0000321767881768f + r * (0.0000002888167364f + r * 0.0000003960315187f)))))));
    return sup ? r : -r;
}

// Gaussian of an mrg32k3a draw d in [1, m1].
__device__ __forceinline__ double mrg_gauss_d(unsigned d)
{
    return inv_normal_cdf((double)d / 4294967088.0);  // same division as the reference
}
__device__ __forceinline__ float mrg_gauss_f(unsigned d)
{
    const unsigned half = 2147483544u;              // (m1 + 1) / 2
    const bool sup = d > half;
    const unsigned up = sup ? 4294967088u - d : d;  // exact integer 1 - p scaled, below 2^31
    return inv_normal_up(__int2float_rn(int(up)) * (1.0f / 4294967088.0f), sup);
}

// Gaussian of a Sobol integer state s (sobol.h:110-116, truncated constant sobol.h:26).
__device__ __forceinline__ double sobol_gauss_d(unsigned s)
{
    return inv_normal_cdf(2.3283064365387E-10 * (double)s);
}
__device__ __forceinline__ float sobol_gauss_f(unsigned s)
{
    const bool sup = s >= 2147483648u;
    // up in [1, 2^31].  2^31 (s = 2^31, the coordinate 1/2 of every dimension at the first
    // point) does not fit a signed int; a plain cast of it was compiled to a signed conversion
    // and turned 1/2 into -1/2 (a NaN Gaussian).  2^31 - 1 rounds to the same float 2^31, so
    // the signed conversion of up - [up == 2^31] is exact for every up.
    const unsigned up = sup ? 0u - s : s;
    return inv_normal_up(__int2float_rn(int(up - (up >> 31))) * 2.3283064365386963e-10f, sup);
}

template <class Real>
__device__ __forceinline__ Real mrg_gauss(unsigned d);
template <>
__device__ __forceinline__ double mrg_gauss<double>(unsigned d) { return mrg_gauss_d(d); }
template <>
__device__ __forceinline__ float mrg_gauss<float>(unsigned d) { return mrg_gauss_f(d); }
template <class Real>
__device__ __forceinline__ Real sobol_gauss(unsigned s);
template <>
__device__ __forceinline__ double sobol_gauss<double>(unsigned s) { return sobol_gauss_d(s); }
template <>
__device__ __forceinline__ float sobol_gauss<float>(unsigned s) { return sobol_gauss_f(s); }

// Sobol point of index n (path n-1): XOR of direction numbers over the set bits of gray(n)
// (sobol.h:119-151).  dir is [32][stride] for the dimensions of the launch.
__device__ __forceinline__ unsigned sobol_state(const unsigned* dir, int stride, int d, unsigned long long n)
{
    unsigned long long g = n ^ (n >> 1);
    unsigned s = 0;
    while (g)
    {
        const int b = __ffsll((long long)g) - 1;
        s ^= __ldg(dir + (size_t)b * stride + d);
        g &= g - 1;
    }
    return s;
}

// ---------------------------------------------------------------------------------------
// Bulk copies global -> shared through the TMA unit (cp.async.bulk, no tensor map), with
// completion tracked by an mbarrier.  Every wait is bounded.  A wait that expires records
// DEVERR_TMA_TIMEOUT; the block then waits once more (bounded) for its copies in flight and
// returns, so the launch fails (CF_E_DEVICE on the host) and no block computes on, or exits
// with, a copy outstanding against its shared memory that it could still wait for.
// Requirements: dst, src 16-byte aligned; bytes a multiple of 16 and < 2^20.
// ---------------------------------------------------------------------------------------
constexpr int MBAR_WAIT_LIMIT = 1 << 20;  // try_wait polls before a wait gives up

__device__ __forceinline__ void mbar_init(unsigned long long* mbar, unsigned count)
{
    const unsigned bar = (unsigned)__cvta_generic_to_shared(mbar);
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// One thread: arrive on mbar expecting `bytes`, and start the copy that completes them.
__device__ __forceinline__ void bulk_load(void* dst, const void* src, unsigned bytes, unsigned long long* mbar)
{
    const unsigned bar = (unsigned)__cvta_generic_to_shared(mbar);
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(d),
                 "l"(src), "r"(bytes), "r"(bar)
                 : "memory");
}

// Waits (bounded) for phase `parity` of mbar to complete; true when it did.
__device__ __forceinline__ bool mbar_wait(unsigned long long* mbar, unsigned parity)
{
    const unsigned bar = (unsigned)__cvta_generic_to_shared(mbar);
    unsigned done = 0;
    for (int it = 0; it < MBAR_WAIT_LIMIT && !done; ++it)
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
    return done != 0;
}

// Whole block: copies `bytes` from src into dst and waits for them.  Returns false (uniformly
// over the block) when the wait expired; the error flag is then set and the caller must return
// at once, without reading dst.
__device__ __forceinline__ bool bulk_copy_to_smem(void* dst, const void* src, unsigned bytes,
                                                  unsigned long long* mbar, int* err)
{
    if (threadIdx.x == 0)
    {
        mbar_init(mbar, 1);
        bulk_load(dst, src, bytes, mbar);
    }
    __syncthreads();
    const bool done = mbar_wait(mbar, 0);
    const int ok = __syncthreads_and((int)done);
    if (!ok)
    {
        if (threadIdx.x == 0) atomicOr(err, DEVERR_TMA_TIMEOUT);
        mbar_wait(mbar, 0);  // let the copy land before the block returns (bounded)
        __syncthreads();
    }
    return ok != 0;
}

}  // namespace cf
