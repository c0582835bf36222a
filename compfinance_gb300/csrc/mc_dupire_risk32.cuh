// FP32 Dupire risk kernel: value and path-wise adjoint of one aggregate of the European or
// smoothed up-and-out payoffs (mcSimulAAD, mcBase.h:427-532, for Dupire, mcMdlDupire.h:238-280,
// with the products of mcPrd.h:113-288), FP32 path arithmetic, exact fixed-point sums.
//
// A block of 128 threads runs rounds of work units (an antithetic mrg32k3a pair, or one Sobol
// path, per thread), claimed from a launch-wide counter, each in three phases:
//  1. forward: each thread simulates its unit and stores per step one packed word per path
//     (the interval of the log-spot grid, the interpolation weight t to 22 bits, and whether
//     the monitoring date at that point fell in the barrier's smoothing band) plus the
//     unit's Gaussian; band dates also store the survival factor before the date and the
//     spot.  The forward itself uses the quantised weight, so the reverse sweep replays
//     exactly the operations of the forward.
//  2. compaction: paths whose adjoint seed is zero (knocked out, or out of the money at
//     maturity) contribute nothing to any risk; the block appends the others to a
//     first-in-first-out list of pending paths.  The scratch is a ring of R32_RING round
//     slots, so a listed path may wait up to two rounds for its sweep.
//  3. reverse: while 128 paths are pending, the block sweeps a chunk of 128 (one path per
//     thread, every thread busy); a partial chunk runs only when the oldest pending paths'
//     slot is about to be rewritten, and once at the end.  Each listed path is swept back
//     from maturity to today by one thread, with no block barrier inside the sweep.  The
//     adjoint of each local-vol value the step used is split over its two spot knots and,
//     with the step's time weights, over its two time columns.  Each of the (up to) four
//     parts is rounded once to an integer in units of 2^-nodeShiftF and added (native 32-bit
//     shared atomics) to an int32 slab of the local-vol nodes; parts of large adjoints go, in
//     the same unit, to a block-private int64 slab in global memory (64-bit atomics).  The
//     host picks nodeShiftF so that no int32 word can overflow within 256 paths; after each
//     chunk (at most 128 paths) the int32 slab is moved into the int64 slab, whose words are
//     added to the accumulators once, at the end.  Each contribution is rounded once, so
//     every sum is independent of how paths are grouped into warps, blocks, chunks and
//     launches.
//
// The kernel template is instantiated in two translation units: mc_dupire_risk32_l1.cu (the
// forward reads the local-vol rows through L1) and mc_dupire_risk32_tma.cu (rows staged into
// shared memory by bulk copies), so that each kernel holds one form of the forward.
#pragma once
#include <cuda_runtime.h>

#include "cf_device.cuh"

namespace cf {

namespace {

constexpr int RB = 128;                 // threads per block
constexpr int RW = RB / 32;             // warps per block
constexpr int T_BITS = 22;              // interpolation weight bits of the packed step word
constexpr unsigned T_MASK = (1u << T_BITS) - 1;
constexpr unsigned BAND_BIT = 1u << T_BITS;
constexpr int LO_SHIFT = T_BITS + 1;    // interval index in bits 23..31
// t in [0, 1) is quantised through the float t + 2 in [2, 3), whose low 22 mantissa bits
// are round(t 2^22): no conversion instruction either way
constexpr unsigned TWO_BITS = 0x40000000u;         // bits of 2.0f
constexpr float T_MAX = 1.0f - 1.0f / 4194304.0f;  // t + 2 stays below 3
// Contributions with |adjoint| >= AV_MAX go to the block's int64 node slab in global memory
// (native 64-bit adds, same unit) instead of the int32 shared slab (the host's choice of
// nodeShiftF assumes this bound).  After a path passes through the barrier's smoothing band
// its state adjoint is of the order of the spot over the band width, so this is common.
constexpr float AV_MAX = 512.0f;
// pending-path list: a power of two above the most it holds (127 left over + 2 RB new)
constexpr int LIST_CAP = 512;

__host__ __device__ inline size_t a16(size_t x) { return (x + 15) & ~size_t(15); }

struct R32Layout
{
    size_t slab, node, ir, bucket, listIdx, cnt, mbar, stepc, invn, rows, base, total;
};

__host__ __device__ inline R32Layout r32_layout(int rng, const McParams& p)
{
    R32Layout L;
    size_t off = 0;
    L.slab = off;
    off += a16(size_t(4 + 2 * p.nPay + 2) * 16);
    L.node = off;  // int32 local-vol node slab of the current chunk
    off += a16(size_t(p.nS) * p.nT * 4);
    L.ir = off;
    off += a16(size_t(p.nS + 1) * 8);
    L.bucket = off;  // per bucket: its first knot's interval l0 and the knot above (xs[l0 + 1])
    off += a16(size_t(p.nBucketsF) * 8);
    L.listIdx = off;  // (ring slot << 8) | (thread << 1) | path of the pair
    off += a16(size_t(LIST_CAP) * 2);
    L.cnt = off;    // per-warp counts, then the claimed chunk (first round, rounds)
    off += 32;
    L.mbar = off;   // completion barriers of the two row buffers
    off += 16;
    L.stepc = off;  // per-step node columns and weights of the reverse
    off += a16(size_t(p.nSteps) * 16);
    L.invn = off;   // piecewise-cubic inverse normal, 512 pieces (when staged: p.stageY)
    if (p.stageY) off += size_t(512) * 16;
    L.rows = off;   // two buffers of rowChunk local-vol rows (y - 2d, d)[nS + 1]
    if (p.rowChunk) off += a16(size_t(2) * p.rowChunk * (p.nS + 1) * 8);
    L.base = off;
    if (rng == RNG_SOBOL) off += a16(size_t(RW) * (size_t(p.nSteps) | 1) * 4);
    L.total = off;
    return L;
}

// Nine blocks per SM (56 registers) where that costs no spills: the kernel is bound by issue
// and latency, and a ninth block hides more of it (60x30 barrier, mrg32k3a: 3.8% faster).  The
// Sobol barrier variant would spill at 56 registers and keeps eight.
template <int PROD, int RNGK, bool ROWS>
__global__ void __launch_bounds__(RB, (PROD == PROD_UOC && RNGK == RNG_SOBOL) ? 8 : 9)
    dupire_risk32(const McParams p)
{
    constexpr int NP = RNGK == RNG_MRG ? 2 : 1;
    constexpr bool UOC = PROD == PROD_UOC;
    extern __shared__ __align__(128) unsigned char smem[];
    const R32Layout L = r32_layout(RNGK, p);
    long long* slab = reinterpret_cast<long long*>(smem + L.slab);  // [0,2) spot adjoint, payoffs from 8
    long long* paySlab = slab + 8;
    int* node = reinterpret_cast<int*>(smem + L.node);
    float2* sIr = reinterpret_cast<float2*>(smem + L.ir);
    int2* sBucket = reinterpret_cast<int2*>(smem + L.bucket);
    unsigned short* listIdx = reinterpret_cast<unsigned short*>(smem + L.listIdx);
    int* cnt = reinterpret_cast<int*>(smem + L.cnt);
    long long* sClaim = reinterpret_cast<long long*>(smem + L.cnt + 16);
    unsigned long long* mbar = reinterpret_cast<unsigned long long*>(smem + L.mbar);
    int4* sStepc = reinterpret_cast<int4*>(smem + L.stepc);
    float4* sInvn = reinterpret_cast<float4*>(smem + L.invn);
    float2* sRows = reinterpret_cast<float2*>(smem + L.rows);

    const int tid = threadIdx.x, lane = tid & 31, wib = tid >> 5;
    const int nS = p.nS, nT = p.nT, nSteps = p.nSteps, nPay = p.nPay, nNodes = nS * nT;
    // block-private int64 node slab in global memory, after the scratch fields: during a sweep
    // it takes the large contributions (64-bit atomic adds); between sweeps word i is read and
    // written only by thread i mod RB
    long long* gnode = reinterpret_cast<long long*>(static_cast<char*>(p.scratch) + p.nodeSlabOffset) +
                       size_t(blockIdx.x) * nNodes;
    const int K = ROWS ? p.rowChunk : 0;  // the host launches ROWS kernels with an even rowChunk >= 2
    if (ROWS && tid == 0)
    {
        mbar_init(mbar, 1);
        mbar_init(mbar + 1, 1);
    }
    for (int i = tid; i < 2 * (4 + 2 * nPay + 2); i += RB) slab[i] = 0;
    for (int i = tid; i < nNodes; i += RB)
    {
        node[i] = 0;
        gnode[i] = 0;
    }
    for (int i = tid; i < nS + 1; i += RB) sIr[i] = make_float2(p.irF[2 * i], p.irF[2 * i + 1]);
    for (int i = tid; i < p.nBucketsF; i += RB)
    {
        const int l0 = p.bucketF[i];
        sBucket[i] = make_int2(l0, __float_as_int(p.xsF[l0 + 1]));
    }
    const float4* gInvn = reinterpret_cast<const float4*>(p.invnF);
    const bool stageInvn = p.stageY != 0;
    if (stageInvn)
        for (int i = tid; i < 512; i += RB) sInvn[i] = gInvn[i];
    for (int i = tid; i < nSteps; i += RB) sStepc[i] = p.stepcF[i];
    __syncthreads();

    const float2* td = reinterpret_cast<const float2*>(p.tdF);
    const int tPitch = nS + 1;
    const float strike = (float)p.strike, barSmooth = (float)p.barSmooth, minusSmooth = (float)p.minusSmooth,
                twoSmooth = (float)p.twoSmooth;
    const float invTwo = -1.0f / twoSmooth;
    const float logBand = p.logBandF;
    const float s0 = p.s0f;
    const float spot = (float)p.spot;
    const float w0 = nPay > 0 ? p.wf[0] : 0.0f, w1 = nPay > 1 ? p.wf[1] : 0.0f;
    const float bX0 = p.bX0F, bInvW = p.bInvWF;
    const float bMaxF = float(p.nBucketsF - 1);

    // scratch [ring slot][field][point][thread], 32-bit offsets (the host keeps it below 2^31
    // elements).  Point nSteps of a path's step-word field holds its adjoint seed, and point
    // nSteps of its survival-factor field (barrier) the seed of the survival factor.
    const int Ti = int(gridDim.x) * RB;
    const int rowStride = (nSteps + 1) * Ti;
    constexpr int F_G = 0, F_W = 1, F_B = 1 + NP, F_S = 1 + 2 * NP;
    constexpr int NF = UOC ? 1 + 3 * NP : 1 + NP;
    const int slotStride = NF * rowStride;
    float* const scr = reinterpret_cast<float*>(p.scratch);
    float* fs = scr;  // the slot of the current unit round
    const int myCol = int(blockIdx.x) * RB + tid;
    const int seedRow = nSteps * Ti;
    const bool evEvery = p.evEvery != 0;

    // Gaussian of a lower-half integer draw up in [1, 2^31] (uniform up / denom of the
    // generator; sup: the draw was in the upper half): the piece is the leading bit of up and
    // the 4 bits after it, z the fraction of the remaining bits, the value a cubic in z.
    auto gaussT = [&](unsigned up, bool sup) -> float {
        const int lz = __clz(up);
        const unsigned nrm = up << lz;  // leading one at bit 31
        const int piece = ((31 - lz) << 4) | int((nrm >> 27) & 15u);
        const float z = __uint_as_float(0x3F800000u | ((nrm << 5) >> 9)) - 1.0f;
        const float4 c = stageInvn ? sInvn[piece] : __ldg(gInvn + piece);
        const float g = fmaf(fmaf(fmaf(c.w, z, c.z), z, c.y), z, c.x);
        return sup ? -g : g;
    };

    // upper_bound of xs among the knots: a bucket holds at most one knot, and the host placed
    // the buckets so that no knot lies near an edge, where the FP32 bucket index can be one off;
    // so xs lies above the knot below the bucket's first interval, and only the knot above it
    // needs a comparison
    auto search = [&](float xs) -> int {
        const int b = __float2int_rz(fminf(fmaxf((xs - bX0) * bInvW, 0.0f), bMaxF));  // NaN -> 0
        const int2 e = sBucket[b];
        const int lo = e.x + (__int_as_float(e.y) <= xs ? 1 : 0);
        return lo < nS ? lo : nS;  // +inf would pass the last sentinel
    };

    // ---------------------------------------------------------------------------------
    // One unit: forward, payoff sums, adjoint seeds.  The seeds of live paths (nonzero seed)
    // go to point nSteps of their slot's fields; live[] says which paths are live.
    // ---------------------------------------------------------------------------------
    // Local-vol rows of the forward: with K = rowChunk > 0, chunk c (steps [cK, cK + K)) is
    // copied into row buffer c mod 2 by one bulk copy, issued when chunk c - 1 starts, so it
    // has landed by the time chunk c needs it; otherwise rows are read through L1.
    unsigned rowPhase = 0;  // bit b: parity of the next completion of buffer b (uniform)
    auto issueRows = [&](int c) {  // thread 0
        const int s0 = c * K, n = min(K, nSteps - s0);
        // rows start on 16-byte boundaries (K is even, a row is 8 (nS + 1) bytes); the size is
        // rounded up to 16 bytes inside the table's 16-byte padded region
        bulk_load(sRows + (c & 1) * K * tPitch, td + size_t(s0) * tPitch, unsigned(a16(size_t(n) * tPitch * 8)),
                  mbar + (c & 1));
    };

    bool live[NP];
    // Returns false (uniformly) when a row copy did not complete: the block must then return.
    auto forward = [&](int nAct, auto&& gen) -> bool {
        float x[NP], alive[NP], euro[NP], sT[NP], bLast[NP];
        bool dead[NP];
        unsigned flag[NP];
#pragma unroll
        for (int a = 0; a < NP; ++a)
        {
            x[a] = 0.0f;
            alive[a] = 1.0f;
            euro[a] = sT[a] = bLast[a] = 0.0f;
            dead[a] = false;
            flag[a] = 0;
            live[a] = false;
        }

        // product date at point i (i < nSteps: monitoring only; i == nSteps: maturity)
        auto event = [&](int i, int a) {
            const bool last = i == nSteps;
            if (!UOC)
            {
                if (last)
                {
                    const float S = s0 * expf(x[a]);
                    sT[a] = S;
                    euro[a] = S - strike > 0.0f ? S - strike : 0.0f;
                }
                return;
            }
            if (!last && (dead[a] || !(x[a] > logBand))) return;
            const float S = s0 * expf(x[a]);
            if (!dead[a])
            {
                if (S > barSmooth) dead[a] = true;
                else if (S > minusSmooth)
                {
                    if (last) bLast[a] = alive[a];
                    else
                    {
                        fs[(F_B + a) * rowStride + i * Ti + myCol] = alive[a];
                        fs[(F_S + a) * rowStride + i * Ti + myCol] = S;
                    }
                    alive[a] *= (barSmooth - S) / twoSmooth;
                    flag[a] = BAND_BIT;  // the band flag, in its place in the step word
                }
            }
            if (last)
            {
                sT[a] = S;
                const float m = p.callPut ? (strike - S) : (S - strike);
                euro[a] = m > 0.0f ? m : 0.0f;
            }
        };

        if (nAct && p.evAtStep[0] >= 0)
#pragma unroll
            for (int a = 0; a < NP; ++a)
                if (a < nAct) event(0, a);
        // steps [s0, s1), with the local-vol row of step s at rowOf(s) (entry lo at rowOf(s)[lo]);
        // the scratch pointers of the Gaussian and the step words advance by one point per step
        auto steps = [&](int s0, int s1, auto&& rowOf) {
            float* pg = fs + F_G * rowStride + s0 * Ti + myCol;
            unsigned* pw = reinterpret_cast<unsigned*>(fs) + F_W * rowStride + s0 * Ti + myCol;
            for (int s = s0; s < s1; ++s, pg += Ti, pw += Ti)
            {
                const float g = gen(s);
                __stcs(pg, g);  // streamed: read once, in the reverse
                const float2* rs = rowOf(s);
#pragma unroll
                for (int a = 0; a < NP; ++a)
                {
                    if (a >= nAct) break;
                    const float ga = a ? -g : g;
                    const int lo = search(x[a]);
                    const float2 ir = sIr[lo];
                    const float t2 = fminf((x[a] - ir.x) * ir.y, T_MAX) + 2.0f;
                    const unsigned tq = __float_as_uint(t2) & T_MASK;
                    float2 yd;
                    if constexpr (ROWS) yd = rs[lo];  // shared memory
                    else yd = __ldg(rs + lo);
                    const float v = fmaf(yd.y, t2, yd.x);  // table (y - 2 d, d)
                    __stcs(pw + a * rowStride, (unsigned(lo) << LO_SHIFT) | flag[a] | tq);
                    flag[a] = 0;  // the flag of point s + 1 is set by its date, if any
                    x[a] += v * (-0.5f * v + ga);
                }
                // the barrier monitors at dates only (and a date below the band needs nothing
                // before maturity: one test for both paths of the pair); a European's one date
                // is the last point
                if (UOC ? (evEvery || __ldg(p.evAtStep + s + 1) >= 0) &&
                              (s + 1 == nSteps || fmaxf(x[0], x[NP - 1]) > logBand)
                        : s + 1 == nSteps)
#pragma unroll
                    for (int a = 0; a < NP; ++a)
                        if (a < nAct) event(s + 1, a);
            }
        };
        if constexpr (ROWS)
        {
            // every thread of the block takes part in the chunk loop (its barriers), with or
            // without a unit; a buffer is rewritten only after all threads passed the barrier
            // of the chunk that follows the one that read it
            const int nChunks = (nSteps + K - 1) / K;
            if (tid == 0) issueRows(0);  // buffer 0 was last read before the previous round's list barrier
            for (int c = 0; c < nChunks; ++c)
            {
                const int b = c & 1;
                const bool done = mbar_wait(mbar + b, (rowPhase >> b) & 1u);
                rowPhase ^= 1u << b;
                if (!__syncthreads_and(done))
                {
                    if (tid == 0) atomicOr(p.err, DEVERR_TMA_TIMEOUT);
                    mbar_wait(mbar + b, ((rowPhase >> b) & 1u) ^ 1u);  // let the late copy land (bounded)
                    __syncthreads();
                    return false;
                }
                if (tid == 0 && c + 1 < nChunks) issueRows(c + 1);
                const float2* buf = sRows + b * K * tPitch;  // row s at buf + (s - cK) tPitch
                const int s0 = c * K;
                if (nAct) steps(s0, min(s0 + K, nSteps), [&](int s) { return buf + (s - s0) * tPitch; });
            }
        }
        else
        {
            if (nAct) steps(0, nSteps, [&](int s) { return td + size_t(s) * tPitch; });
        }
        if (!nAct) return true;

        // payoffs, sums, adjoint seeds
#pragma unroll
        for (int a = 0; a < NP; ++a)
        {
            if (a >= nAct) break;
            float ax, aAl = 0.0f, agg;
            if (UOC)
            {
                const float p0 = dead[a] ? 0.0f : alive[a] * euro[a];
                fix_add(&paySlab[0], p0);
                fix_add(&paySlab[2 * nPay], p0 * p0);
                fix_add(&paySlab[2], euro[a]);
                fix_add(&paySlab[2 * (nPay + 1)], euro[a] * euro[a]);
                agg = w0 * p0 + w1 * euro[a];
                const float aEuro = dead[a] ? w1 : w0 * alive[a] + w1;
                aAl = dead[a] ? 0.0f : w0 * euro[a];
                const float m = p.callPut ? (strike - sT[a]) : (sT[a] - strike);
                float aF = m > 0.0f ? (p.callPut ? -aEuro : aEuro) : 0.0f;
                if (flag[a])
                {
                    aF += aAl * bLast[a] * invTwo;
                    aAl *= (barSmooth - sT[a]) / twoSmooth;
                }
                ax = aF * sT[a];
            }
            else
            {
                fix_add(&paySlab[0], euro[a]);
                fix_add(&paySlab[2 * nPay], euro[a] * euro[a]);
                agg = w0 * euro[a];
                ax = euro[a] > 0.0f ? w0 * sT[a] : 0.0f;
            }
            fix_add(&paySlab[2 * (2 * nPay)], agg);
            fix_add(&paySlab[2 * (2 * nPay + 1)], agg * agg);
            live[a] = ax != 0.0f || aAl != 0.0f;
            if (live[a])
            {
                fs[(F_W + a) * rowStride + seedRow + myCol] = ax;
                if (UOC) fs[(F_B + a) * rowStride + seedRow + myCol] = aAl;
            }
        }
        return true;
    };

    // contribution c (units of 1) to spot j of a step's vol row (its columns and weights in
    // sc), too large for the shared slab: into the block's int64 slab, rounded once like the
    // shared adds.  gnode is written only by these adds during a sweep and only by its owning
    // thread between sweeps (barriers in between).
    auto bigAdd = [&](const int4 sc, int j, float c) {
        long long* g = gnode + j * nT;
        atomicAdd(reinterpret_cast<unsigned long long*>(g + sc.x),
                  (unsigned long long)__float2ll_rn(c * __int_as_float(sc.z)));
        const float wb = __int_as_float(sc.w);
        if (wb != 0.0f)
            atomicAdd(reinterpret_cast<unsigned long long*>(g + sc.y), (unsigned long long)__float2ll_rn(c * wb));
    };

    // ---------------------------------------------------------------------------------
    // Pending-path list: a first-in-first-out ring of LIST_CAP entries in shared memory.
    // head, q2 and q1 are uniform over the block: q2 entries of round r-2 and then q1 of round
    // r-1 are pending at the start of round r (q2 + q1 < RB).
    // ---------------------------------------------------------------------------------
    int head = 0, q2 = 0, q1 = 0;

    // Appends the round's live paths (slot `slot`) behind the pending ones; returns how many.
    auto collect = [&](int slot) -> int {
        const unsigned b0 = __ballot_sync(0xffffffffu, live[0]);
        const unsigned b1 = NP == 2 ? __ballot_sync(0xffffffffu, live[NP - 1]) : 0u;
        if (lane == 0) cnt[wib] = __popc(b0) + __popc(b1);
        __syncthreads();
        int total = 0, off = head + q2 + q1;
#pragma unroll
        for (int w = 0; w < RW; ++w)
        {
            const int c = cnt[w];
            off += w < wib ? c : 0;
            total += c;
        }
        const unsigned lt = (1u << lane) - 1u;
        if (live[0])
            listIdx[(off + __popc(b0 & lt)) & (LIST_CAP - 1)] = (unsigned short)((slot << 8) | (tid << 1));
        if (NP == 2 && live[NP - 1])
            listIdx[(off + __popc(b0) + __popc(b1 & lt)) & (LIST_CAP - 1)] =
                (unsigned short)((slot << 8) | (tid << 1) | 1);
        __syncthreads();
        return total;
    };

    // Sweeps the first n (uniform, 1..RB) pending paths back, one per thread, then moves the
    // chunk's slab into this thread's words of the block's int64 slab.
    auto sweep = [&](int n) {
        if (tid < n)
        {
            const int e = listIdx[(head + tid) & (LIST_CAP - 1)];
            const int a = e & 1;
            const int col = int(blockIdx.x) * RB + ((e >> 1) & (RB - 1));
            const float* es = scr + (e >> 8) * slotStride;  // the path's ring slot
            float ax = es[(F_W + a) * rowStride + seedRow + col];
            float aAl = UOC ? es[(F_B + a) * rowStride + seedRow + col] : 0.0f;
            const unsigned* sw = reinterpret_cast<const unsigned*>(es) + (F_W + a) * rowStride + col;
            const float* sg = es + F_G * rowStride + col;
            unsigned wNext = 0;  // packed word of the step after s: band flag of point s + 1
            // software pipeline: the step words and Gaussians are loaded three steps ahead
            // (they come from DRAM), the local-vol entry and interval record of a step one
            // step ahead, so that only the adjoint itself is carried from step to step
            unsigned wA = __ldcs(sw + (nSteps - 1) * Ti), wB = 0, wC = 0;
            float gA = __ldcs(sg + (nSteps - 1) * Ti), gB = 0.0f, gC = 0.0f;
            if (nSteps >= 2)
            {
                wB = __ldcs(sw + (nSteps - 2) * Ti);
                gB = __ldcs(sg + (nSteps - 2) * Ti);
            }
            if (nSteps >= 3)
            {
                wC = __ldcs(sw + (nSteps - 3) * Ti);
                gC = __ldcs(sg + (nSteps - 3) * Ti);
            }
            float2 ydA = __ldg(td + size_t(nSteps - 1) * tPitch + int(wA >> LO_SHIFT));
            float2 irA = sIr[wA >> LO_SHIFT];
            for (int s = nSteps - 1; s >= 0; --s)
            {
                if (UOC && (wNext & BAND_BIT))
                {
                    const int i = s + 1;
                    const float before = es[(F_B + a) * rowStride + i * Ti + col];
                    const float S = es[(F_S + a) * rowStride + i * Ti + col];
                    const float aF = aAl * before * invTwo;
                    aAl *= (barSmooth - S) / twoSmooth;
                    ax += aF * S;
                }
                const unsigned W = wA;
                const float g1 = gA;
                const float2 yd = ydA, ir = irA;
                wA = wB;
                gA = gB;
                wB = wC;
                gB = gC;
                if (s >= 3)
                {
                    wC = __ldcs(sw + (s - 3) * Ti);
                    gC = __ldcs(sg + (s - 3) * Ti);
                }
                if (s >= 1)
                {
                    const int loN = int(wA >> LO_SHIFT);
                    ydA = __ldg(td + size_t(s - 1) * tPitch + loN);
                    irA = sIr[loN];
                }
                const float ga = a ? -g1 : g1;
                const int lo = int(W >> LO_SHIFT);
                const float t2 = __uint_as_float(TWO_BITS | (W & T_MASK)), t = t2 - 2.0f;
                const float v = fmaf(yd.y, t2, yd.x);  // the forward's expression
                const float av = ax * (ga - v);      // d x_{s+1} / d v = g - v
                ax += av * (yd.y * ir.y);            // d x_{s+1} / d x_s = 1 + (g - v) dv/dx
                if (av != 0.0f)
                {
                    const int jl = lo - (lo > 0 ? 1 : 0);
                    const bool inner = lo > 0 && lo < nS;  // two spot knots; one at the flat ends
                    const float cR = av * t, cL = av - cR;
                    const int4 sc = sStepc[s];
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
                        bigAdd(sc, jl, cL);
                        if (inner && cR != 0.0f) bigAdd(sc, jl + 1, cR);
                    }
                }
                wNext = W;
            }
            if (UOC && (wNext & BAND_BIT))  // band at today's date
            {
                const float before = es[(F_B + a) * rowStride + col];
                const float S = es[(F_S + a) * rowStride + col];
                ax += aAl * before * invTwo * S;
            }
            fix_add(&slab[0], ax / spot);  // x_0 = log(spot)
        }
        head += n;
        __syncthreads();
        // the chunk's slab -> this thread's words of the block's int64 slab
        for (int i = tid; i < nNodes; i += RB)
        {
            const int v = node[i];
            if (v)
            {
                node[i] = 0;
                gnode[i] = __ldcg(gnode + i) + v;  // L2: the sweep's 64-bit adds land there
            }
        }
        __syncthreads();  // the next chunk adds into the cleared slab
    };

    // End of round r (its paths in ring slot `slot`; slot < 0: after the last round): list its
    // live paths, sweep full chunks, and sweep the rest if paths of round r-2 are still pending
    // (round r+1 rewrites their slot) or no round follows.  The trip counts depend only on
    // uniform values, so every barrier is reached by the whole block.
    auto endRound = [&](int slot) {
        const int count = q2 + q1 + (slot >= 0 ? collect(slot) : 0);
        int done = 0;
        for (;;)
        {
            const int left = count - done;
            const int n = left >= RB ? RB : (done < q2 || slot < 0) ? left : 0;
            if (n == 0) break;
            sweep(n);
            done += n;
        }
        const int old = q2 + q1 - done;  // round r-1's paths still pending
        q2 = old > 0 ? old : 0;
        q1 = count - done - q2;
    };
    auto slotOf = [&](long long it) {
        const int k = int(it % R32_RING);
        fs = scr + k * slotStride;
        return k;
    };

    // Unit rounds (RB units of the generator, or RW Sobol batches of 32 paths) are claimed from
    // the launch's counter in chunks of G consecutive rounds, G shrinking with the rounds left
    // (guided self-scheduling): the blocks resident on one SM progress at different speeds, and
    // with a fixed share each an SM would run its last rounds with few of them left.  A thread
    // runs the G units of its chunk that follow each other in its generator, with one skip-ahead.
    // With fewer ring slots than R32_RING a block runs at most p.roundCap rounds (the host's
    // cap times the grid covers every round).
    long long it = 0;  // rounds this block has run: round it uses ring slot it mod R32_RING
    const long long cap = p.roundCap > 0 ? p.roundCap : LLONG_MAX;
    auto claim = [&](long long nRounds) {  // chunk [sClaim[0], sClaim[0] + sClaim[1]) (uniform)
        __syncthreads();  // every thread has read the previous chunk
        if (tid == 0)
        {
            const long long seen = (long long)*reinterpret_cast<volatile unsigned long long*>(p.claim);
            long long g = (nRounds - seen) / (2LL * gridDim.x);
            g = g > 1 ? g : 1;
            g = g < cap - it ? g : cap - it;
            sClaim[1] = g;
            sClaim[0] = g > 0 ? (long long)atomicAdd(p.claim, (unsigned long long)g) : LLONG_MAX;
        }
        __syncthreads();
    };
    if (RNGK == RNG_MRG)
    {
        const long long nUnits = (p.nPath + 1) / 2;
        const long long nRounds = (nUnits + RB - 1) / RB;
        for (;;)
        {
            claim(nRounds);
            const long long r0 = sClaim[0], G = sClaim[1];
            if (r0 >= nRounds) break;
            const long long u0 = r0 * RB + tid * G;  // this thread's units u0 .. u0 + G - 1
            MrgState st{};
            if (u0 < nUnits) st = mrg_jump(p.seed1, p.seed2, (unsigned long long)(p.firstPath / 2 + u0) * nSteps, p.mrgJumpA, p.mrgJumpB);
            for (long long j = 0; j < G; ++j, ++it)
            {
                const long long u = u0 + j;
                const int nAct = u < nUnits ? ((2 * u + 1 < p.nPath) ? 2 : 1) : 0;
                const int slot = slotOf(it);
                if (!forward(nAct, [&](int) {
                        const unsigned d = mrg_next(st);   // in [1, m1]; uniform d / (m1 + 1)
                        const bool sup = d > 2147483544u;  // (m1 + 1) / 2
                        return gaussT(sup ? 4294967088u - d : d, sup);
                    }))
                    return;  // a row copy failed (error flag set): the launch fails
                endRound(slot);
            }
        }
    }
    else
    {
        // Sobol: in round r warp w takes batch b = r RW + w; lane l runs index n = 32b + l
        // (path n-1); state(n) = state(32b) ^ state(l).
        const int pitch = nSteps | 1;
        unsigned* base = reinterpret_cast<unsigned*>(smem + L.base) + wib * pitch;
        const long long nBatches = p.nPath / 32 + 1;
        const long long nRounds = (nBatches + RW - 1) / RW;
        for (;;)
        {
            claim(nRounds);
            const long long r0 = sClaim[0], G = sClaim[1];
            if (r0 >= nRounds) break;
            for (long long j = 0; j < G; ++j, ++it)
            {
                const long long b = (r0 + j) * RW + wib;
                int nAct = 0;
                if (b < nBatches)
                {
                    __syncwarp();
                    for (int d = lane; d < nSteps; d += 32)
                        base[d] = sobol_state(p.sobolDir, nSteps, d, (unsigned long long)(p.firstPath + b * 32));
                    __syncwarp();
                    const long long n = b * 32 + lane;
                    nAct = (n >= 1 && n <= p.nPath) ? 1 : 0;
                }
                const int slot = slotOf(it);
                if (!forward(nAct, [&](int i) {
                        const unsigned sb = base[i] ^ sobol_state(p.sobolDir, nSteps, i, (unsigned long long)lane);
                        const bool sup = sb >= 2147483648u;
                        return gaussT(sup ? 0u - sb : (sb > 1u ? sb : 1u), sup);  // state 0 occurs only at index 0
                    }))
                    return;  // a row copy failed (error flag set): the launch fails
                endRound(slot);
            }
        }
    }
    endRound(-1);  // the paths still pending after the last round

    __syncthreads();
    if (tid == 0) fix_flush(&p.acc[0], &slab[0]);
    // node words in units of 2^-nodeShiftF (nodeShiftF <= FIX_HI_SHIFT): exact in the hi word
    for (int i = tid; i < nNodes; i += RB)
    {
        const long long v = __ldcg(gnode + i);
        if (v) atomicAdd(reinterpret_cast<unsigned long long*>(&p.acc[2 * (1 + i)]),
                         (unsigned long long)(v << (FIX_HI_SHIFT - p.nodeShiftF)));
    }
    for (int i = tid; i < 2 * nPay + 2; i += RB) fix_flush(&p.acc[2 * (p.nRisk + i)], &paySlab[2 * i]);
}

}  // namespace

template <bool ROWS>
const void* dupire_risk32_ptr_t(int prod, int rng)
{
    if (prod == PROD_UOC && rng == RNG_MRG) return (const void*)&dupire_risk32<PROD_UOC, RNG_MRG, ROWS>;
    if (prod == PROD_UOC && rng == RNG_SOBOL) return (const void*)&dupire_risk32<PROD_UOC, RNG_SOBOL, ROWS>;
    if (prod == PROD_EUROPEAN && rng == RNG_MRG) return (const void*)&dupire_risk32<PROD_EUROPEAN, RNG_MRG, ROWS>;
    if (prod == PROD_EUROPEAN && rng == RNG_SOBOL) return (const void*)&dupire_risk32<PROD_EUROPEAN, RNG_SOBOL, ROWS>;
    return nullptr;
}

}  // namespace cf
