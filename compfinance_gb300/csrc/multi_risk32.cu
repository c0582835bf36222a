// FP32 AADriskMulti of a European portfolio on the Dupire model (mcSimulAADMulti,
// mcBase.h:775-989; Europeans, mcPrd.h:305-399; Dupire, mcMdlDupire.h:238-280): the risk of
// every payoff to every local-vol node.
//
// The risk of payoff (e, j) = max(S_e - K_ej, 0) is the path average of dS_e/dtheta over the
// paths whose spot at maturity e is above K_ej.  With the strikes of a maturity sorted, a path
// pays the m_e lowest of them, so its adjoint for maturity e belongs to bucket (e, m_e), and
// per-strike sums are suffix sums over buckets (multi_finish).  Adding each path's node
// contributions (up to four per step and maturity) straight into the [bucket][node] table
// costs a global atomic each.  Here the paths are grouped by bucket first, so that a block
// can sum many paths of one bucket in shared memory:
//  1. multi32_forward simulates the paths with the quantised interpolation of
//     dupire_risk32 and stores per path and step one packed word (interval, weight) and the
//     Gaussian, and per (maturity, path) the bucket and the spot; the spots go to per-bucket
//     fixed-point sums and the entries of each bucket are counted (the values need only
//     these two sums per bucket: the numeraire is 1);
//  2. multi32_scan lays the buckets out back to back and cuts each into chunks of at most
//     M32_CHUNK entries;
//  3. multi32_scatter writes each (path, spot) entry into its bucket's segment (block-level
//     bucket counts, one global cursor add per block and bucket);
//  4. multi32_reverse takes chunks: all entries of a chunk belong to one bucket, so the block
//     sweeps its paths back from maturity e into one int32 slab of the local-vol nodes (native
//     shared-memory adds in units of 2^-nodeShiftF, the unit dupire_risk32 uses for rounds of
//     256 paths) and adds the slab to the bucket's row once per chunk.
// Every contribution is rounded once on its own, so the sums do not depend on the order of
// the entries in a bucket, on the chunking or on the grid: results are deterministic.
#include <cuda_runtime.h>

#include "cf_device.cuh"
#include "multi32.h"

namespace cf {

namespace {

constexpr int MB = 128;  // threads per block (forward and reverse)
constexpr int MW = MB / 32;
constexpr int T_BITS = 22;  // packed step word: interval in bits 23..31, weight t in 22 bits
constexpr unsigned T_MASK = (1u << T_BITS) - 1;
constexpr int LO_SHIFT = T_BITS + 1;
constexpr unsigned TWO_BITS = 0x40000000u;         // bits of 2.0f; t + 2 in [2, 3)
constexpr float T_MAX = 1.0f - 1.0f / 4194304.0f;
constexpr float AV_MAX = 512.0f;  // larger contributions go exactly to the global accumulators

__host__ __device__ inline size_t a16(size_t x) { return (x + 15) & ~size_t(15); }

struct FwdLayout
{
    size_t val, hist, xs, ir, bucket, ks, evOff, base, total;
};

__host__ __device__ inline FwdLayout fwd_layout(int rng, const Multi32Args& A)
{
    const McParams& p = A.p;
    FwdLayout L;
    size_t off = 0;
    L.val = off;  // sum of S per bucket (the counts are the bucket histogram)
    off += a16(size_t(A.nBuckets) * 16);
    L.hist = off;
    off += a16(size_t(A.nBuckets) * 4);
    L.xs = off;
    off += a16(size_t(p.nS + 2) * 4);
    L.ir = off;
    off += a16(size_t(p.nS + 1) * 8);
    L.bucket = off;
    off += a16(size_t(p.nBucketsF) * 4);
    L.ks = off;
    off += a16(size_t(A.nKs) * 4);
    L.evOff = off;
    off += a16(size_t(p.nEv + 1) * 4);
    L.base = off;
    if (rng == RNG_SOBOL) off += a16(size_t(MW) * (size_t(p.nSteps) | 1) * 4);
    L.total = off;
    return L;
}

struct RevLayout
{
    size_t node, ir, stepc, spot, misc, total;
};

__host__ __device__ inline RevLayout rev_layout(const Multi32Args& A)
{
    const McParams& p = A.p;
    RevLayout L;
    size_t off = 0;
    L.node = off;
    off += a16(size_t(p.nS) * p.nT * 4);
    L.ir = off;
    off += a16(size_t(p.nS + 1) * 8);
    L.stepc = off;
    off += a16(size_t(p.nSteps) * 16);
    L.spot = off;
    off += 16;
    L.misc = off;
    off += 16;
    L.total = off;
    return L;
}

// ---------------------------------------------------------------------------------------
// 1. forward
// ---------------------------------------------------------------------------------------
template <int RNGK>
__global__ void __launch_bounds__(MB) multi32_forward(const Multi32Args A)
{
    constexpr int NP = RNGK == RNG_MRG ? 2 : 1;
    const McParams& p = A.p;
    extern __shared__ __align__(128) unsigned char smem[];
    const FwdLayout L = fwd_layout(RNGK, A);
    long long* sVal = reinterpret_cast<long long*>(smem + L.val);
    int* hist = reinterpret_cast<int*>(smem + L.hist);
    float* sXs = reinterpret_cast<float*>(smem + L.xs);
    float2* sIr = reinterpret_cast<float2*>(smem + L.ir);
    int* sBucket = reinterpret_cast<int*>(smem + L.bucket);
    float* sKs = reinterpret_cast<float*>(smem + L.ks);
    int* sEvOff = reinterpret_cast<int*>(smem + L.evOff);
    const int tid = threadIdx.x, lane = tid & 31, wib = tid >> 5;
    const int nS = p.nS, nSteps = p.nSteps, nEv = p.nEv, nB = A.nBuckets;
    for (int i = tid; i < 2 * nB; i += MB) sVal[i] = 0;
    for (int i = tid; i < nB; i += MB) hist[i] = 0;
    for (int i = tid; i < nS + 2; i += MB) sXs[i] = p.xsF[i];
    for (int i = tid; i < nS + 1; i += MB) sIr[i] = make_float2(p.irF[2 * i], p.irF[2 * i + 1]);
    for (int i = tid; i < p.nBucketsF; i += MB) sBucket[i] = p.bucketF[i];
    for (int i = tid; i < A.nKs; i += MB) sKs[i] = A.ksF[i];
    for (int i = tid; i <= nEv; i += MB) sEvOff[i] = A.evOff[i];
    __syncthreads();

    const float2* td = reinterpret_cast<const float2*>(p.tdF);
    const int tPitch = nS + 1;
    const float s0 = p.s0f, bX0 = p.bX0F, bInvW = p.bInvWF;
    const int nBf = p.nBucketsF;
    const float4* gInvn = reinterpret_cast<const float4*>(p.invnF);
    const long long nPath = p.nPath;

    // Gaussian of a lower-half integer draw up in [1, 2^31] (sup: the draw was in the upper
    // half): piecewise cubic in the bits after the leading one (the table of dupire_risk32)
    auto gaussT = [&](unsigned up, bool sup) -> float {
        const int lz = __clz(up);
        const unsigned nrm = up << lz;
        const int piece = ((31 - lz) << 4) | int((nrm >> 27) & 15u);
        const float z = __uint_as_float(0x3F800000u | ((nrm << 5) >> 9)) - 1.0f;
        const float4 c = __ldg(gInvn + piece);
        const float g = fmaf(fmaf(fmaf(c.w, z, c.z), z, c.y), z, c.x);
        return sup ? -g : g;
    };
    // upper_bound of xs among the knots (a fine bucket holds at most one knot)
    auto search = [&](float xs) -> int {
        const float fb = (xs - bX0) * bInvW;
        int b = 0;
        if (fb > 0.0f) b = fb < float(nBf - 1) ? int(fb) : nBf - 1;
        const int l0 = sBucket[b];
        const int lo = l0 + (sXs[l0 + 1] <= xs ? 1 : 0) - (sXs[l0] > xs ? 1 : 0);
        return lo < nS ? lo : nS;
    };
    // maturity e of path: bucket = number of sorted strikes below the spot
    auto event = [&](int e, long long path, float x) {
        const float S = s0 * expf(x);
        const int o = sEvOff[e] - e, n = sEvOff[e + 1] - sEvOff[e] - 1;
        int lo = 0, hi = n;
        while (lo < hi)
        {
            const int mid = (lo + hi) >> 1;
            if (sKs[o + mid] < S) lo = mid + 1;
            else hi = mid;
        }
        const size_t at = size_t(e) * size_t(nPath) + size_t(path);
        A.evB[at] = (unsigned short)lo;
        A.evS[at] = S;
        if (lo > 0)
        {
            const int bk = sEvOff[e] + lo;
            fix_add(sVal + 2 * bk, S);
            atomicAdd(hist + bk, 1);
        }
    };

    // one unit: NP paths from path0 (an antithetic pair, or one Sobol path)
    auto runUnit = [&](int nAct, long long path0, auto&& gen) {
        float x[NP];
        uint2 prev[NP];
#pragma unroll
        for (int a = 0; a < NP; ++a)
        {
            x[a] = 0.0f;
            prev[a] = make_uint2(0u, 0u);
        }
        const int e0 = __ldg(p.evAtStep);
        if (e0 >= 0)
#pragma unroll
            for (int a = 0; a < NP; ++a)
                if (a < nAct) event(e0, path0 + a, 0.0f);
        for (int s = 0; s < nSteps; ++s)
        {
            const float g = gen(s);
            const float2* trow = td + size_t(s) * tPitch;
#pragma unroll
            for (int a = 0; a < NP; ++a)
            {
                if (a >= nAct) break;
                const float ga = a ? -g : g;
                const int lo = search(x[a]);
                const float2 ir = sIr[lo];
                const float t2 = fminf((x[a] - ir.x) * ir.y, T_MAX) + 2.0f;
                const unsigned tq = __float_as_uint(t2) & T_MASK;
                const float2 yd = __ldg(trow + lo);
                const float v = fmaf(yd.y, t2, yd.x);  // table (y - 2 d, d)
                const uint2 r = make_uint2((unsigned(lo) << LO_SHIFT) | tq, __float_as_uint(ga));
                // records are written in pairs of steps (one 16-byte store)
                if (s & 1)
                    *reinterpret_cast<uint4*>(A.rec + 2 * (size_t(path0 + a) * A.pitch + (s - 1))) =
                        make_uint4(prev[a].x, prev[a].y, r.x, r.y);
                else if (s == nSteps - 1)
                    *reinterpret_cast<uint4*>(A.rec + 2 * (size_t(path0 + a) * A.pitch + s)) =
                        make_uint4(r.x, r.y, 0u, 0u);
                else
                    prev[a] = r;
                x[a] += v * (-0.5f * v + ga);
            }
            const int e = __ldg(p.evAtStep + s + 1);
            if (e >= 0)
#pragma unroll
                for (int a = 0; a < NP; ++a)
                    if (a < nAct) event(e, path0 + a, x[a]);
        }
    };

    const long long T = (long long)gridDim.x * MB;
    const long long tg = (long long)blockIdx.x * MB + tid;
    if (RNGK == RNG_MRG)
    {
        const long long nUnits = (nPath + 1) / 2;
        const long long per = (nUnits + T - 1) / T;
        const long long u0 = tg * per;
        const long long u1 = u0 + per < nUnits ? u0 + per : nUnits;
        if (u0 < u1)
        {
            MrgState st = mrg_jump(p.seed1, p.seed2, (unsigned long long)(p.firstPath / 2 + u0) * nSteps, p.mrgJumpA,
                                   p.mrgJumpB);
            for (long long u = u0; u < u1; ++u)
                runUnit((2 * u + 1 < nPath) ? 2 : 1, 2 * u, [&](int) {
                    const unsigned d = mrg_next(st);   // in [1, m1]; uniform d / (m1 + 1)
                    const bool sup = d > 2147483544u;  // (m1 + 1) / 2
                    return gaussT(sup ? 4294967088u - d : d, sup);
                });
        }
    }
    else
    {
        // a warp's batch b: lane l runs Sobol index n = 32 b + l (path n - 1)
        const int pitch = nSteps | 1;
        unsigned* base = reinterpret_cast<unsigned*>(smem + L.base) + wib * pitch;
        const long long nBatches = nPath / 32 + 1;
        for (;;)
        {
            // warps take batches from the launch counter one at a time: the warps of an SM
            // progress at different speeds, and a fixed share each would leave the last ones alone
            unsigned long long bc = 0;
            if (lane == 0) bc = atomicAdd(p.claim, 1ull);
            const long long b = (long long)__shfl_sync(0xffffffffu, bc, 0);
            if (b >= nBatches) break;
            __syncwarp();
            for (int d = lane; d < nSteps; d += 32)
                base[d] = sobol_state(p.sobolDir, nSteps, d, (unsigned long long)(p.firstPath + b * 32));
            __syncwarp();
            const long long n = b * 32 + lane;
            if (n >= 1 && n <= nPath)
                runUnit(1, n - 1, [&](int i) {
                    const unsigned sb = base[i] ^ sobol_state(p.sobolDir, nSteps, i, (unsigned long long)lane);
                    const bool sup = sb >= 2147483648u;
                    return gaussT(sup ? 0u - sb : (sb > 1u ? sb : 1u), sup);
                });
        }
    }
    __syncthreads();
    for (int i = tid; i < nB; i += MB) fix_flush(&A.accVal[2 * (5 * i + 1)], &sVal[2 * i]);
    for (int i = tid; i < nB; i += MB)
        if (hist[i]) atomicAdd(A.cnt + i, hist[i]);
}

// ---------------------------------------------------------------------------------------
// 2. bucket segments and chunks (one warp)
// ---------------------------------------------------------------------------------------
__global__ void multi32_scan(const Multi32Args A)
{
    const int lane = threadIdx.x, nB = A.nBuckets;
    const int per = (nB + 31) / 32, lo = lane * per, hi = lo + per < nB ? lo + per : nB;
    int c = 0, ch = 0;
    for (int i = lo; i < hi; ++i)
    {
        const int n = A.cnt[i];
        c += n;
        ch += (n + M32_CHUNK - 1) / M32_CHUNK;
    }
    int ic = c, ich = ch;  // inclusive warp scans
#pragma unroll
    for (int d = 1; d < 32; d <<= 1)
    {
        const int u = __shfl_up_sync(0xffffffffu, ic, d), v = __shfl_up_sync(0xffffffffu, ich, d);
        if (lane >= d)
        {
            ic += u;
            ich += v;
        }
    }
    int off = ic - c, choff = ich - ch;
    for (int i = lo; i < hi; ++i)
    {
        const int n = A.cnt[i];
        A.accVal[2 * (5 * i)] = (long long)n << FIX_HI_SHIFT;  // sum of numeraire^-1 = 1 per path
        A.start[i] = off;
        A.chunkStart[i] = choff;
        off += n;
        choff += (n + M32_CHUNK - 1) / M32_CHUNK;
    }
    if (lane == 31)
    {
        A.start[nB] = ic;
        A.chunkStart[nB] = ich;
    }
}

// ---------------------------------------------------------------------------------------
// 3. entries into their bucket segments.  A block takes SC_PER consecutive (maturity, path)
// entries, ranks them within its own bucket counts (shared-memory atomics) and reserves its
// range of each bucket with one global add, so that the global cursors see one add per
// block and bucket instead of one per warp.
// ---------------------------------------------------------------------------------------
constexpr int SC_BLOCK = 256, SC_ITEMS = 8, SC_PER = SC_BLOCK * SC_ITEMS;

__global__ void __launch_bounds__(SC_BLOCK) multi32_scatter(const Multi32Args A)
{
    extern __shared__ int sCount[];  // [nBuckets]: block counts, then the block's global offsets
    const int nB = A.nBuckets, tid = threadIdx.x;
    const long long nPath = A.p.nPath;
    const long long total = (long long)A.p.nEv * nPath;
    const long long i0 = (long long)blockIdx.x * SC_PER;
    for (int i = tid; i < nB; i += SC_BLOCK) sCount[i] = 0;
    __syncthreads();
    int bk[SC_ITEMS], rank[SC_ITEMS];
#pragma unroll
    for (int j = 0; j < SC_ITEMS; ++j)
    {
        const long long i = i0 + j * SC_BLOCK + tid;
        bk[j] = -1;
        if (i < total)
        {
            const int m = A.evB[i];
            if (m > 0)
            {
                bk[j] = __ldg(A.evOff + int(i / nPath)) + m;
                rank[j] = atomicAdd(sCount + bk[j], 1);
            }
        }
    }
    __syncthreads();
    for (int i = tid; i < nB; i += SC_BLOCK)
    {
        const int c = sCount[i];
        if (c) sCount[i] = __ldg(A.start + i) + atomicAdd(A.cursor + i, c);
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < SC_ITEMS; ++j)
        if (bk[j] >= 0)
        {
            const long long i = i0 + j * SC_BLOCK + tid;
            const int at = sCount[bk[j]] + rank[j];
            A.list[2 * at] = int(i - (i / nPath) * nPath);
            A.list[2 * at + 1] = __float_as_int(A.evS[i]);
        }
}

// ---------------------------------------------------------------------------------------
// 4. reverse sweeps of bucket chunks
// ---------------------------------------------------------------------------------------
__global__ void __launch_bounds__(MB) multi32_reverse(const Multi32Args A)
{
    const McParams& p = A.p;
    extern __shared__ __align__(128) unsigned char smem[];
    const RevLayout L = rev_layout(A);
    int* node = reinterpret_cast<int*>(smem + L.node);
    float2* sIr = reinterpret_cast<float2*>(smem + L.ir);
    int4* stepc = reinterpret_cast<int4*>(smem + L.stepc);
    long long* spotSlab = reinterpret_cast<long long*>(smem + L.spot);
    int* misc = reinterpret_cast<int*>(smem + L.misc);
    const int tid = threadIdx.x;
    const int nS = p.nS, nT = p.nT, nSteps = p.nSteps, nNodes = nS * nT, nB = A.nBuckets;
    const float wScale = ldexpf(1.0f, p.nodeShiftF);
    for (int i = tid; i < nNodes; i += MB) node[i] = 0;
    for (int i = tid; i < nS + 1; i += MB) sIr[i] = make_float2(p.irF[2 * i], p.irF[2 * i + 1]);
    for (int i = tid; i < nSteps; i += MB)
        stepc[i] = make_int4(p.colA[i], p.colB[i], __float_as_int(p.cAf[i] * wScale), __float_as_int(p.cBf[i] * wScale));
    if (tid < 2) spotSlab[tid] = 0;
    __syncthreads();

    const float2* td = reinterpret_cast<const float2*>(p.tdF);
    const int tPitch = nS + 1;
    const float spot = (float)p.spot;
    const int nChunks = __ldg(A.chunkStart + nB);
    const int hiShift = FIX_HI_SHIFT - p.nodeShiftF;

    for (;;)
    {
        if (tid == 0) misc[0] = atomicAdd(A.work, 1);
        __syncthreads();
        const int c = misc[0];
        if (c >= nChunks) break;
        // bucket of chunk c: the last b with chunkStart[b] <= c (empty buckets share starts)
        int lo = 0, hi = nB;
        while (hi - lo > 1)
        {
            const int mid = (lo + hi) >> 1;
            if (__ldg(A.chunkStart + mid) <= c) lo = mid;
            else hi = mid;
        }
        const int b = lo;
        int e0 = 0, e1 = p.nEv;  // maturity of bucket b: the last e with evOff[e] <= b
        while (e1 - e0 > 1)
        {
            const int mid = (e0 + e1) >> 1;
            if (__ldg(A.evOff + mid) <= b) e0 = mid;
            else e1 = mid;
        }
        const int iE = __ldg(p.evPoint + e0);
        const int first = __ldg(A.start + b) + (c - __ldg(A.chunkStart + b)) * M32_CHUNK;
        const int end = __ldg(A.start + b + 1);
        const int count = end - first < M32_CHUNK ? end - first : M32_CHUNK;
        long long* row = A.accRisk + 2 * size_t(b) * A.nParam;

        for (int idx = tid; idx < count; idx += MB)
        {
            const int path = __ldg(A.list + 2 * (first + idx));
            float ax = __int_as_float(__ldg(A.list + 2 * (first + idx) + 1));  // d payoff / d x_e = S_e
            const uint4* rr = reinterpret_cast<const uint4*>(A.rec + 2 * size_t(path) * A.pitch);
            auto step = [&](int s, unsigned W, unsigned gbits) {
                const float ga = __uint_as_float(gbits);
                const int l = int(W >> LO_SHIFT);
                const float t2 = __uint_as_float(TWO_BITS | (W & T_MASK)), t = t2 - 2.0f;
                const float2 yd = __ldg(td + size_t(s) * tPitch + l);
                const float2 ir = sIr[l];
                const float v = fmaf(yd.y, t2, yd.x);  // the forward's expression
                const float av = ax * (ga - v);  // d x_{s+1} / d v = g - v
                ax += av * (yd.y * ir.y);        // d x_{s+1} / d x_s = 1 + (g - v) dv/dx
                if (av == 0.0f) return;
                const int jl = l - (l > 0 ? 1 : 0);
                const bool inner = l > 0 && l < nS;  // two spot knots; one at the flat ends
                const float cR = av * t, cL = av - cR;
                const int4 sc = stepc[s];
                if (fabsf(av) < AV_MAX)
                {
                    const float wa = __int_as_float(sc.z), wb = __int_as_float(sc.w);
                    int* nl = node + jl * nT;
                    atomicAdd(nl + sc.x, __float2int_rn(cL * wa));
                    if (wb != 0.0f) atomicAdd(nl + sc.y, __float2int_rn(cL * wb));
                    if (inner && cR != 0.0f)
                    {
                        atomicAdd(nl + nT + sc.x, __float2int_rn(cR * wa));
                        if (wb != 0.0f) atomicAdd(nl + nT + sc.y, __float2int_rn(cR * wb));
                    }
                }
                else
                {
                    const float ca = __ldg(p.cAf + s), cb = __ldg(p.cBf + s);
                    fix_add(row + 2 * (1 + jl * nT + sc.x), cL * ca);
                    if (cb != 0.0f) fix_add(row + 2 * (1 + jl * nT + sc.y), cL * cb);
                    if (inner && cR != 0.0f)
                    {
                        fix_add(row + 2 * (1 + (jl + 1) * nT + sc.x), cR * ca);
                        if (cb != 0.0f) fix_add(row + 2 * (1 + (jl + 1) * nT + sc.y), cR * cb);
                    }
                }
            };
            // steps iE-1 .. 0, stored in pairs (2k, 2k+1); the next pair is loaded one ahead
            int s = iE - 1;
            if (s >= 0)
            {
                uint4 cur = __ldg(rr + (s >> 1));
                for (;;)
                {
                    const int k = s >> 1;
                    const uint4 nxt = k > 0 ? __ldg(rr + k - 1) : make_uint4(0u, 0u, 0u, 0u);
                    if (s & 1)
                    {
                        step(s, cur.z, cur.w);
                        --s;
                    }
                    step(s, cur.x, cur.y);
                    --s;
                    if (s < 0) break;
                    cur = nxt;
                }
            }
            fix_add(spotSlab, ax / spot);  // x_0 = log(spot)
        }
        __syncthreads();
        // the chunk's slab -> the bucket's row (node words in units of 2^-nodeShiftF: exact in hi)
        for (int i = tid; i < nNodes; i += MB)
        {
            const int v = node[i];
            if (v)
            {
                node[i] = 0;
                atomicAdd(reinterpret_cast<unsigned long long*>(row + 2 * (1 + i)),
                          (unsigned long long)((long long)v << hiShift));
            }
        }
        if (tid == 0)
        {
            fix_flush(row, spotSlab);
            spotSlab[0] = spotSlab[1] = 0;
        }
        __syncthreads();
    }
}

const void* fwd_ptr(int rng)
{
    return rng == RNG_MRG ? (const void*)&multi32_forward<RNG_MRG> : (const void*)&multi32_forward<RNG_SOBOL>;
}

}  // namespace

size_t m32_forward_smem(int rng, const Multi32Args& a) { return fwd_layout(rng, a).total; }
size_t m32_reverse_smem(const Multi32Args& a) { return rev_layout(a).total; }

int m32_occupancy(int rng, size_t smemFwd, size_t smemRev, int* occFwd, int* occRev)
{
    cudaError_t e = cudaFuncSetAttribute(fwd_ptr(rng), cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smemFwd);
    if (!e) e = cudaFuncSetAttribute((const void*)&multi32_reverse, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smemRev);
    if (!e) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(occFwd, fwd_ptr(rng), MB, smemFwd);
    if (!e) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(occRev, (const void*)&multi32_reverse, MB, smemRev);
    return (int)e;
}

int launch_multi32(int rng, int gridFwd, size_t smemFwd, int gridRev, size_t smemRev, const Multi32Args& a,
                   void* stream)
{
    cudaStream_t st = (cudaStream_t)stream;
    Multi32Args q = a;
    void* args[] = {&q};
    cudaError_t e = cudaLaunchKernel(fwd_ptr(rng), dim3(gridFwd), dim3(MB), args, smemFwd, st);
    if (!e) e = cudaLaunchKernel((const void*)&multi32_scan, dim3(1), dim3(32), args, 0, st);
    const long long total = (long long)a.p.nEv * a.p.nPath;
    if (!e)
        e = cudaLaunchKernel((const void*)&multi32_scatter, dim3(unsigned((total + SC_PER - 1) / SC_PER)),
                             dim3(SC_BLOCK), args, size_t(a.nBuckets) * 4, st);
    if (!e) e = cudaLaunchKernel((const void*)&multi32_reverse, dim3(gridRev), dim3(MB), args, smemRev, st);
    return (int)e;
}

}  // namespace cf
