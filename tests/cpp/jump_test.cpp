// Host check of the mrg32k3a jump tables (compfinance_gb300/csrc/host_math.cpp): a skip of n taken
// with the radix-16 records (one matrix-vector product per nonzero hexadecimal digit, as the
// kernels take it) equals n steps of the recurrences, for small n by iteration and for large n
// by binary powers of the recurrence matrices.
#include <cstdint>
#include <cstdio>
#include <vector>

#include "host_math.h"

using u64 = uint64_t;
static const u64 M1 = 4294967087ULL, M2 = 4294944443ULL;

static void matvec(const u64 a[9], u64 v[3], u64 m)
{
    u64 r[3];
    for (int i = 0; i < 3; ++i)
    {
        unsigned __int128 s = 0;
        for (int l = 0; l < 3; ++l) s += (unsigned __int128)a[3 * i + l] * v[l];
        r[i] = u64(s % m);
    }
    for (int i = 0; i < 3; ++i) v[i] = r[i];
}

static void matmul(const u64 a[9], const u64 b[9], u64 m, u64 r[9])
{
    u64 t[9];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
        {
            unsigned __int128 s = 0;
            for (int l = 0; l < 3; ++l) s += (unsigned __int128)a[3 * i + l] * b[3 * l + j];
            t[3 * i + j] = u64(s % m);
        }
    for (int i = 0; i < 9; ++i) r[i] = t[i];
}

// the state (newest first) after n steps, by the tables
static void by_tables(const uint32_t T[256][12], u64 m, u64 v[3], u64 n)
{
    for (int k = 0; n; ++k, n >>= 4)
    {
        const int d = int(n & 15);
        if (!d) continue;
        u64 a[9];
        for (int i = 0; i < 9; ++i) a[i] = T[16 * k + d][i];
        matvec(a, v, m);
    }
}

// n steps by binary powers of the one-step matrix
static void by_powers(const u64 g[9], u64 m, u64 v[3], u64 n)
{
    u64 p[9];
    for (int i = 0; i < 9; ++i) p[i] = g[i];
    for (; n; n >>= 1)
    {
        if (n & 1) matvec(p, v, m);
        matmul(p, p, m, p);
    }
}

// The kernels' reduction (cf_device.cuh, mrg_matvec): each 32 x 32-bit product folded once with
// 2^32 = C (mod m), the three of a row summed, two more folds and one conditional subtraction.
template <u64 C, u64 M>
static u64 folded_row(const u64 e[3], const u64 v[3])
{
    u64 s = 0;
    for (int l = 0; l < 3; ++l)
    {
        const u64 q = e[l] * v[l];
        s += (q >> 32) * C + (q & 0xffffffffULL);
    }
    s = (s >> 32) * C + (s & 0xffffffffULL);
    s = (s >> 32) * C + (s & 0xffffffffULL);
    return s >= M ? s - M : s;
}

static int failures = 0;
static void check(bool c, const char* what, u64 n)
{
    std::printf("%s %s n=%llu\n", c ? "ok" : "FAIL", what, (unsigned long long)n);
    failures += !c;
}

int main()
{
    static uint32_t A[256][12], B[256][12];
    cf::mrg_jump_tables(A, B);
    const u64 a[9] = {0, 1403580, M1 - 810728, 1, 0, 0, 0, 1, 0};
    const u64 b[9] = {527612, 0, M2 - 1370589, 1, 0, 0, 0, 1, 0};
    bool zero = true;
    for (int k = 0; k < 16; ++k)
        for (int i = 0; i < 12; ++i) zero = zero && A[16 * k][i] == 0 && B[16 * k][i] == 0;
    for (int r = 0; r < 256; ++r)
        for (int i = 9; i < 12; ++i) zero = zero && A[r][i] == 0 && B[r][i] == 0;
    check(zero, "unused_records_and_padding_zero", 0);
    // small skips against the recurrences themselves, from the seed state (12345 x 3, 1234 x 3)
    for (u64 n : {u64(1), u64(2), u64(15), u64(16), u64(17), u64(255), u64(256), u64(4097), u64(9999)})
    {
        u64 x[3] = {12345, 12345, 12345}, y[3] = {1234, 1234, 1234};
        for (u64 s = 0; s < n; ++s)
        {
            matvec(a, x, M1);
            matvec(b, y, M2);
        }
        u64 tx[3] = {12345, 12345, 12345}, ty[3] = {1234, 1234, 1234};
        by_tables(A, M1, tx, n);
        by_tables(B, M2, ty, n);
        check(tx[0] == x[0] && tx[1] == x[1] && tx[2] == x[2] && ty[0] == y[0] && ty[1] == y[1] && ty[2] == y[2],
              "tables_vs_iteration", n);
    }
    // large skips (a path's first draw at 2^22 paths x 520 steps and beyond) against binary powers
    for (u64 n : {(u64(1) << 40) + 12345, u64(2097151) * 156, u64(0xFEDCBA9876543ULL), ~u64(0) >> 1})
    {
        u64 x[3] = {12345, 12345, 12345}, y[3] = {1234, 1234, 1234};
        by_powers(a, M1, x, n);
        by_powers(b, M2, y, n);
        u64 tx[3] = {12345, 12345, 12345}, ty[3] = {1234, 1234, 1234};
        by_tables(A, M1, tx, n);
        by_tables(B, M2, ty, n);
        check(tx[0] == x[0] && tx[1] == x[1] && tx[2] == x[2] && ty[0] == y[0] && ty[1] == y[1] && ty[2] == y[2],
              "tables_vs_powers", n);
    }
    // the folded reduction against exact arithmetic, at the extremes (entries and states up to m - 1)
    // and on pseudo-random rows
    {
        bool ok = true;
        u64 r = 88172645463325252ULL;
        auto next = [&]() { r ^= r << 13; r ^= r >> 7; r ^= r << 17; return r; };
        for (int it = 0; it < 200000 && ok; ++it)
        {
            u64 e1[3], v1[3], e2[3], v2[3];
            for (int l = 0; l < 3; ++l)
            {
                const bool edge = it < 64;
                e1[l] = edge ? M1 - 1 - (it >> l & 1) : next() % M1;
                v1[l] = edge ? M1 - 1 - (it >> (l + 3) & 1) : next() % M1;
                e2[l] = edge ? M2 - 1 - (it >> l & 1) : next() % M2;
                v2[l] = edge ? M2 - 1 - (it >> (l + 3) & 1) : next() % M2;
            }
            unsigned __int128 x1 = 0, x2 = 0;
            for (int l = 0; l < 3; ++l)
            {
                x1 += (unsigned __int128)e1[l] * v1[l];
                x2 += (unsigned __int128)e2[l] * v2[l];
            }
            ok = folded_row<209, M1>(e1, v1) == u64(x1 % M1) && folded_row<22853, M2>(e2, v2) == u64(x2 % M2);
        }
        check(ok, "folded_reduction_exact", 200000);
    }
    return failures ? 1 : 0;
}
