// Launch descriptors shared by the host planner (engine.cpp) and the CUDA kernels.
//
// A (model, product) pair is lowered once into flat device tables: the simulation timeline,
// per-step model coefficients, the event map from simulation steps to product dates, and
// the product's constants.  Kernels never see strings, virtual calls or host pointers.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace cf {

enum ModelKind : int { MODEL_BS = 0, MODEL_DUPIRE = 1, MODEL_MULTI = 2 };
enum ProductKind : int
{
    PROD_EUROPEAN = 0,
    PROD_UOC = 1,
    PROD_EUROPEANS = 2,
    PROD_CONTINGENT = 3,
    PROD_BASKETS = 4,
    PROD_AUTOCALL = 5
};
// Dynamics of one asset of the multi-asset displaced model (mcMdlMultiDisplaced.h:31-37).
enum MdDynamics : int { MD_LOGNORMAL = 0, MD_NORMAL = 1, MD_SURNORMAL = 2, MD_SUBNORMAL = 3 };

// Derived quantities of the multi-asset model, one array (the kernels' inputs, and the
// quantities whose path adjoints the risk kernel sums): initial spots [nA], Cholesky factor
// [nA][nA] (lower triangle used), per step stds, drifts and dividend-adjusted forward factors
// [nSteps][nA] each, displacements [nA], numeraires of the product dates [nEv].
struct MdLayout
{
    int s0, chol, std_, drift, ff, alpha, num, total;
};
__host__ __device__ inline MdLayout md_layout(int nA, int nSteps, int nEv)
{
    MdLayout L;
    L.s0 = 0;
    L.chol = nA;
    L.std_ = L.chol + nA * nA;
    L.drift = L.std_ + nSteps * nA;
    L.ff = L.drift + nSteps * nA;
    L.alpha = L.ff + nSteps * nA;
    L.num = L.alpha + nA;
    L.total = L.num + nEv;
    return L;
}
enum RngKind : int { RNG_MRG = 0, RNG_SOBOL = 1 };

// Error bits written by kernels into McParams::err (host turns them into CF_E_DEVICE).
enum DeviceError : int { DEVERR_TMA_TIMEOUT = 1, DEVERR_FIXED_RANGE = 2 };

// Fixed-point accumulation: every sum is held as two int64 words, hi in units of 2^-20 and
// lo in units of 2^-60.  Integer addition is associative, so sums are bit-identical for any
// order of the atomic adds (deterministic across launches, grids and streams).
constexpr int FIX_HI_SHIFT = 20;
constexpr int FIX_LO_SHIFT = 60;
constexpr int FIX_CARRY_SHIFT = FIX_LO_SHIFT - FIX_HI_SHIFT;

// FP32 local-vol adjoints (risk launches of the Dupire model) are gathered in two stages.
// Each warp adds, per simulation step, the adjoints of the step's vol row Y[i][.] into a
// per-warp row of int32 words in units of 2^-ROW_SHIFT (one native shared-memory add per
// contribution; |contribution| < ROW_MAX, so a word that receives at most 64 of them per
// step cannot overflow; larger ones go straight to the global accumulators).  After the
// step the warp multiplies each row word by the step's integer time weights
// W = round(w 2^WEIGHT_SHIFT) and adds the exact int64 product to the block's node slab, in
// units of 2^-NODE_SHIFT.  Every operation is an exact integer operation on per-contribution
// roundings, so the sums do not depend on how paths are grouped into warps or blocks.
constexpr int ROW_SHIFT = 16;
constexpr float ROW_MAX = 256.0f;
constexpr int WEIGHT_SHIFT = 23;
constexpr int NODE_SHIFT = ROW_SHIFT + WEIGHT_SHIFT;

// Accumulator layout (one hi/lo pair each):
//   [0, nRisk)                   parameter adjoints (risk mode; 0 in value mode)
//   [nRisk, nRisk+nPay)          sum of payoff k
//   [nRisk+nPay, nRisk+2nPay)    sum of payoff k squared
//   nRisk+2nPay, +1              sum / sum of squares of the aggregate sum_k w_k payoff_k
struct McParams
{
    // sizes: the launch simulates paths [firstPath, firstPath + nPath) of the run's sequence
    // (a shard; firstPath a multiple of 64, so antithetic pairs and Sobol warp batches stay whole)
    long long nPath;
    long long firstPath;
    int nSteps;      // Gaussians per path (simDim)
    int nEv;         // product event dates
    int nPay;
    int nRisk;       // parameters carried in the accumulators (0 for value runs)
    int nAcc;

    // random numbers
    unsigned seed1, seed2;
    const unsigned* sobolDir;              // [32][nSteps]
    const unsigned* mrgJumpA;  // jump tables of the first component (mrg_jump)
    const unsigned* mrgJumpB;  // and of the second

    // model: Black-Scholes
    int spotMeasure;
    double spot, vol;
    const double* bsD;    // [5][nSteps]: drift, std, dt, sqrt(dt), d drift / d vol
    const float* bsF;
    // model: Dupire
    int nS, nT;
    double x0d;           // starting state of the FP64 form: log(spot)
    float s0f;            // FP32 form works in y = x - log(spot), spot = s0f * exp(y)
    const double* Xd;     // [nS] log spots (FP32 form: shifted by -log(spot))
    const float* Xf;
    const double* invdXd; // [nS] 1 / (X[k+1] - X[k])
    const float* invdXf;
    const double* Yd;     // [nSteps][nS] local vols pre-interpolated in time, times sqrt(dt)
    const float* Yf;
    const int* colA;      // [nSteps] time node of the lower time weight
    const int* colB;
    const double* cAd;    // [nSteps] d Y[i][j] / d vol[j][colA] (= sqrt(dt) * (1 - tw))
    const float* cAf;
    const double* cBd;    // [nSteps] d Y[i][j] / d vol[j][colB] (0 when flat)
    const float* cBf;
    const int* wAi;       // [nSteps] round(cA 2^WEIGHT_SHIFT), FP32 form's node weights
    const int* wBi;
    int nodeFlushUnits;   // FP32 risk: units per thread between node slab flushes (>= 1)
    int nodeDirect;       // FP32 risk: 1 = add row products straight to the global accumulators
    int stageY;           // 1: stage Y into shared memory (cp.async.bulk); in dupire_risk32,
                          // stage the inverse-normal table instead
    // Bucket index of the log-spot grid: bucket b of nBuckets equal slices of [X0, X_last]
    // holds the upper_bound of its left edge, a starting guess for the interpolation search.
    int nBuckets;
    const int* bucket;
    double bX0d, bInvWd;
    float bX0f, bInvWf;

    // events
    const int* evAtStep;  // [nSteps+1] product date index reached at timeline point i, or -1
    int evEvery;          // 1 when every point after today is a product date
    const int* evPoint;   // [nEv] timeline point of product date e
    const double* evD;    // [10][nEv]: ff, tauF, disc, tauD, numeraire (factor), t, needNum,
                          // libor(t_e, t_e+1), its derivative to the rate, coverage t_e+1 - t_e
    const float* evF;

    // product
    int callPut;
    double strike, barSmooth, minusSmooth, twoSmooth;
    double coupon, cbSmooth;  // contingent bond: coupon, smoothing width (first spot x smooth)
    double logBandD;      // band test threshold in the state variable (FP64 form)
    float logBandF;       // (FP32 form)
    const double* kD;     // Europeans strikes, flattened by event
    const float* kF;
    const int* evPayOff;  // [nEv+1] payoff offsets per event (Europeans)

    // risk
    const double* w;      // [nPay] aggregation weights
    const float* wf;

    // outputs
    long long* acc;       // [nAcc][2]
    int* err;
    double* pathOut;      // value launches of mc_kernel: every path's payoffs [path][nPay] (path
                          // index within the launch), or null

    // per-thread scratch of the reverse sweep, layout [field][step][thread]
    void* scratch;
    long long scratchThreads;
    int scratchFields;

    // FP32 Dupire risk kernel (dupire_risk32): interval tables of the log-spot grid.
    // Interval lo in [0, nS] is the upper_bound of the state among the knots; for each step
    // and interval the local vol is y + d t with t = (x - xr) ir in [0, 1), flat (d = ir = 0)
    // outside the grid.
    int fast32;           // 1 when the plan carries these tables (the launch may use the kernel)
    const float* xsF;     // [nS + 2] knots with -inf / +inf sentinels at both ends
    const float* irF;     // [nS + 1][2] (xr, ir) per interval
    const float* tdF;     // [nSteps][nS + 1][2] (y - 2 d, d) per step and interval
    const int* bucketF;   // [nBucketsF] upper_bound of each bucket's left edge; buckets are
                          // narrower than 2/3 of the smallest knot spacing (at most one knot each)
                          // and, for dupire_risk32, no knot lies near an edge
    int nBucketsF;
    float bX0F, bInvWF;
    // Node adjoints are rounded to units of 2^-nodeShiftF (<= FIX_HI_SHIFT), chosen per plan so
    // that an int32 shared slab word cannot overflow within one unit round; each block also
    // keeps an int64 node slab in the scratch buffer at byte offset nodeSlabOffset.
    int nodeShiftF;
    long long nodeSlabOffset;
    const float* invnF;   // [512][4] piecewise-cubic inverse normal of the launch's generator
    // dupire_risk32: per step (colA, colB, time weights A and B in units of 2^-nodeShiftF as
    // float bits), the node columns and weights of the reverse sweep's local-vol adjoints
    const int4* stepcF;
    // dupire_risk32: local-vol rows staged into shared memory by bulk copies, rowChunk steps per
    // copy, double-buffered (0: rows are read through L1)
    int rowChunk;
    // dupire_risk32: the launch's round counter (zero at launch), from which blocks claim their
    // unit rounds, and the most rounds one block may run (0: no limit), set when the scratch
    // holds fewer than R32_RING round slots
    unsigned long long* claim;
    long long roundCap;

    // multi-asset displaced model (mcMdlMultiDisplaced.h) with Baskets / Autocall
    // (mcPrdMulti.h); nSteps is the number of time steps, the Gaussians per path nSteps * nA
    int nA;
    int prodKind;         // PROD_BASKETS or PROD_AUTOCALL
    const int* mdDyn;     // [nA] MdDynamics
    const double* mdD;    // derived quantities (md_layout), FP64 and FP32 copies
    const float* mdF;
    const double* mdAssetD;  // [nA] basket weights, or autocall reference levels
    const float* mdAssetF;
    double acKo, acStrike, acCpn, acDt, acSmooth;  // autocall: KO level, put strike, coupon, period, smoothing

    // Dupire raw inputs for bumped revaluation (bumpRisk): vols [nS][nT] spot-major, and per
    // step sqrt(dt) and the time weight t of interp_lin, so that a bumped node's sqrt(dt) sigma
    // is recomputed exactly like the host computes Y
    const double* volsD;
    const double* stepSqD;
    const double* stepTwD;
};

// Kernel configuration chosen by the host.
struct McLaunch
{
    int model, prod, rng, fp32, risk;
    int grid, block;
    size_t smem;
    int fast;             // FP32 Dupire risk through dupire_risk32: 1 (rows read through L1) or 2
                          // (rows staged by bulk copies, p.rowChunk > 0)
};

int launch_mc(const McLaunch& l, const McParams& p, void* stream);   // returns cudaError_t
int mc_smem_bytes(const McLaunch& l, const McParams& p, int stageY, size_t* bytes);
int mc_occupancy(const McLaunch& l, size_t smem, int* blocksPerSM);
// dupire_risk32 staging (p.stageY: inverse-normal table in shared memory; p.rowChunk: local-vol
// rows staged by bulk copies) that keeps occ0 blocks per SM; sets *smem, returns the occupancy.
int r32_staging(McLaunch& l, McParams& p, int occ0, size_t* smem);
// dupire_risk32 keeps the reverse-sweep scratch of its last R32_RING unit rounds (a live path
// may wait up to two rounds before its sweep); a block's round r uses slot r mod R32_RING, so a
// launch of fewer rounds per block (p.roundCap) needs only as many slots.
constexpr int R32_RING = 3;
// Unit rounds of a launch of `threads` threads over nPath paths (the generic kernel's threads
// all run that many; dupire_risk32's blocks claim rounds as they go, that many on average).
long long mc_rounds(const McLaunch& l, long long nPath, long long threads);
// Reverse-sweep scratch fields of a risk launch of `rounds` unit rounds.
int mc_scratch_fields(const McLaunch& l, long long rounds);
// Bytes of a risk launch's scratch buffer: p.scratchFields fields [field][point][thread] for
// grid*128 threads, then (dupire_risk32) one int64 node slab per block.  Sets p.nodeSlabOffset.
size_t mc_scratch_bytes(const McLaunch& l, McParams& p, long long grid);
// Whether a (model, product, precision, mode) launch of this plan runs dupire_risk32
// (CF_FAST32=0 in the environment selects the generic kernel instead).
int mc_use_fast32(const McParams& plan, int prod, int fp32, int risk);
int launch_finalize(const McParams& p, double invN, double* out, void* stream);

}  // namespace cf
