/* cfgpu.h -- C ABI of the GB300 Monte Carlo valuation and AAD-risk engine.
 *
 * Drop-in boundary for CompFinance's simulation path (main.h / store.h / mcBase.h):
 * plain C types, caller-allocated outputs, an int status on every call, no exceptions.
 * Every entry point names the reference interface it replaces.  The C++17 wrapper in
 * cfgpu.hpp rebuilds the reference's own signatures (value, AADriskOne, AADriskMulti,
 * dupireSuperbucket, put*) on top of these.
 *
 * Threading: one context per process is the normal use; calls on one context are
 * serialised by an internal lock.  All device memory is owned by the context.
 */
#ifndef CFGPU_H
#define CFGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------------------- */
#define CF_OK 0
#define CF_E_ARG (-1)        /* invalid argument (null pointer, bad size) */
#define CF_E_NOTFOUND (-2)   /* unknown model / product id or payoff label */
#define CF_E_SHAPE (-3)      /* output buffer too small / incompatible model and product */
#define CF_E_CUDA (-4)       /* CUDA runtime error (message in cf_last_error) */
#define CF_E_NOMEM (-5)      /* device allocation failed */
#define CF_E_DEVICE (-6)     /* a kernel reported an error flag (bounded wait expired, range) */
#define CF_E_UNSUPPORTED (-7)

/* Precision of the path arithmetic: CF_FP64 is the parity form (matches the reference to
 * ~1e-12); CF_FP32 keeps the path in FP32 and every sum in exact fixed point. */
#define CF_FP64 0
#define CF_FP32 1

/* NumericalParam, main.h:33-40 (parallel is accepted and ignored: the GPU is always
 * parallel), plus the precision of the path arithmetic. */
typedef struct {
    int parallel;
    int useSobol;
    int numPath;
    int seed1;     /* default 12345 */
    int seed2;     /* default 1234  */
    int precision; /* CF_FP64 or CF_FP32 */
} cf_num_param;

typedef struct cf_context cf_context;

/* ---- context --------------------------------------------------------------------- */
/* Creates a context on CUDA device `device` (replaces the process-wide store and thread
 * pool of store.h:33-36 / threadPool.h:72). */
int cf_create(int device, cf_context** ctx);
int cf_destroy(cf_context* ctx);
/* Copies the last error message of this thread into buf (always NUL-terminated). */
int cf_last_error(char* buf, size_t size);
/* Sets the CUDA stream (cudaStream_t) of subsequent launches; NULL = the context's own. */
int cf_set_stream(cf_context* ctx, void* stream);
int cf_synchronize(cf_context* ctx);
/* Cumulative bytes this context copied host->device and device->host (model tables,
 * weights, results); for end-to-end accounting. */
int cf_transfer_stats(cf_context* ctx, uint64_t* h2dBytes, uint64_t* d2hBytes);

/* ---- store (store.h) -------------------------------------------------------------- */
/* putBlackScholes, store.h:38-54 */
int cf_put_black_scholes(cf_context* ctx, double spot, double vol, int qSpot, double rate, double div,
                         const char* id);
/* putDupire, store.h:56-73; vols spot-major [nSpots][nTimes] */
int cf_put_dupire(cf_context* ctx, double spot, const double* spots, int nSpots, const double* times,
                  int nTimes, const double* vols, double maxDt, const char* id);
/* putEuropean, store.h:128-142 */
int cf_put_european(cf_context* ctx, double strike, double exerciseDate, double settlementDate,
                    const char* id);
/* putBarrier, store.h:144-163 (smooth <= 0 is replaced by 1e-8 as in the reference) */
int cf_put_barrier(cf_context* ctx, double strike, double barrier, double maturity, double monitorFreq,
                   double smooth, int callPut, const char* id);
/* putContingent, store.h:165-180 (ContingentBond, mcPrd.h:404-574): pays (libor(Ti, Ti+1) +
 * coupon) x (Ti+1 - Ti) at Ti+1 when the spot rose over the period (a digital smoothed over
 * +-smooth x the first spot; smooth <= 0: a sharp digital), plus the redemption at maturity. */
int cf_put_contingent(cf_context* ctx, double coupon, double maturity, double payFreq, double smooth, const char* id);
/* putEuropeans, store.h:184-205 (maturities in increasing order) */
int cf_put_europeans(cf_context* ctx, const double* maturities, const double* strikes, int n,
                     const char* id);
/* putDisplaced, store.h:75-94 (MultiDisplaced, mcMdlMultiDisplaced.h:28-717): nA correlated
 * assets (1 to 16, names without blanks) with spots, ATM vols and skews (the displacement rule
 * of mcMdlMultiDisplaced.h:418-444), a discount rate, repo spreads, proportional dividends
 * divs[nDiv][nA] on divDates (increasing), a correlation [nA][nA] whose lower triangle is the
 * model's, and lambda (used correlation = lambda (1 - correl) + correl).  The checks of
 * xPutDisplaced (xlExport.cpp:158-176). */
int cf_put_displaced(cf_context* ctx, int nA, const char* const* assets, const double* spots, const double* atms,
                     const double* skews, double discRate, const double* repoSpreads, int nDiv,
                     const double* divDates, const double* divs, const double* correl, double lambda,
                     const char* id);
/* putBaskets, store.h:224-237 (Baskets, mcPrdMulti.h:181-277): max(sum_a w_a S_a(T) - K, 0)
 * per strike. */
int cf_put_baskets(cf_context* ctx, int nA, const char* const* assets, const double* weights, double maturity,
                   int nK, const double* strikes, const char* id);
/* putAutocall, store.h:239-255 (Autocall, mcPrdMulti.h:279-439): periods equal periods to
 * maturity on the worst performance S_a / ref_a; coupon cpn per year while alive, smoothed
 * knock-out at ko (smoothing max(smooth, 1e-8)), redemption less a put struck at strike. */
int cf_put_autocall(cf_context* ctx, int nA, const char* const* assets, const double* refs, double maturity,
                    int periods, double ko, double strike, double cpn, double smooth, const char* id);
/* The initialised multi-asset model of a (model, product) pair (init, mcMdlMultiDisplaced.h:
 * 407-566), in this order: initial spots [nA], Cholesky factor [nA][nA], stds, drifts and
 * dividend-adjusted forward factors [nSteps][nA] each, displacements [nA], numeraires
 * [nDates]; *count their number (derived == NULL: the count only); dynamics[nA] (when not
 * NULL): 0 lognormal, 1 normal, 2 surnormal, 3 subnormal. */
int cf_md_state(cf_context* ctx, const char* modelId, const char* productId, double* derived, int capacity,
                int* count, int* dynamics);

/* Product::payoffLabels (mcBase.h:137) and Model::parameterLabels (mcBase.h:194): labels
 * written '\n'-separated into buf (NUL-terminated); *count receives their number.  With
 * buf == NULL, *needed receives the buffer size. */
int cf_payoff_labels(cf_context* ctx, const char* productId, char* buf, size_t size, int* count,
                     size_t* needed);
int cf_parameter_labels(cf_context* ctx, const char* modelId, char* buf, size_t size, int* count,
                        size_t* needed);
/* Sizes: number of payoffs, of model parameters, Gaussians per path (Model::simDim). */
int cf_shapes(cf_context* ctx, const char* modelId, const char* productId, int* nPay, int* nParam,
              int* simDim);
/* The local-vol grid of a Dupire model (Dupire::spots / times, mcMdlDupire.h:148-160): sizes,
 * and the knots when spots / times are not NULL.  CF_E_NOTFOUND when the model is not in the
 * store, CF_E_ARG when it is not a Dupire model (the checks of dupireAADRisk, main.h:371-383). */
int cf_model_grid(cf_context* ctx, const char* modelId, int* nSpots, int* nTimes, double* spots, double* times);

/* ---- entry points (main.h) --------------------------------------------------------- */
/* value, main.h:43-96: path averages of every payoff; stderrs (optional) are the Monte
 * Carlo standard errors. */
int cf_value(cf_context* ctx, const char* modelId, const char* productId, const cf_num_param* num,
             double* values, double* stderrs);

/* mcSimul, mcBase.h:267-308: the payoffs of every path, payoffs[numPath * nPay] path-major
 * (path i of the run's random sequence, payoff k in label order), simulated on the device in the
 * precision of num.  Black-Scholes and Dupire models (CF_E_UNSUPPORTED for the multi-asset one). */
int cf_simulate_paths(cf_context* ctx, const char* modelId, const char* productId, const cf_num_param* num,
                      double* payoffs);

/* AADriskOne, main.h:99-173: risks[nParam] of the payoff labelled riskPayoff (NULL or ""
 * = first payoff); payoffValues[nPay]; *riskPayoffValue its value. */
int cf_aad_risk_one(cf_context* ctx, const char* modelId, const char* productId, const cf_num_param* num,
                    const char* riskPayoff, double* payoffValues, double* riskPayoffValue, double* risks);

/* AADriskAggregate, main.h:176-254: risks of sum_k notionals[k] * payoff_k; notionals[nPay]
 * indexed like the payoff labels. */
int cf_aad_risk_aggregate(cf_context* ctx, const char* modelId, const char* productId,
                          const double* notionals, const cf_num_param* num, double* payoffValues,
                          double* aggregateValue, double* risks);

/* AADriskMulti, main.h:269-312: values[nPay], risks[nParam * nPay] parameter-major. */
int cf_aad_risk_multi(cf_context* ctx, const char* modelId, const char* productId, const cf_num_param* num,
                      double* values, double* risks);

/* bumpRisk, main.h:316-359: values[nPay] and risks[nParam * nPay] (parameter-major, like
 * AADriskMulti) by one-sided 1e-8 bumps of every model parameter, repriced on the same random
 * numbers, always in FP64.  method: CF_BUMP_REPRICE revalues a bumped copy of the model per
 * parameter (the reference's procedure); CF_BUMP_PATHWISE (Dupire) re-simulates, for each
 * local-vol node, only the paths that touch it (the same numbers, far less work); CF_BUMP_AUTO
 * picks pathwise where it applies. */
enum { CF_BUMP_AUTO = 0, CF_BUMP_REPRICE = 1, CF_BUMP_PATHWISE = 2 };
int cf_bump_risk(cf_context* ctx, const char* modelId, const char* productId, const cf_num_param* num, int method,
                 double* values, double* risks);

/* Implied-vol surfaces for the Dupire calibration (ivs.h): kind 0 =
 * iv(K,T) = p0 + p1 ln^2(K/p3)/sqrt(T) + p2 ln(K/p3); kind 1 = MertonIVS (ivs.h:147-179)
 * with p = {vol, jump intensity, mean jump, jump std}. */
typedef struct {
    int kind;
    double spot;
    double p[4];
} cf_ivs;

/* dupireCalib, mcMdlDupire.h:337-388 / main.h:414-438.  First call with lvols == NULL to
 * get the grid sizes; lvols spot-major [nS][nT]. */
int cf_dupire_calib(cf_context* ctx, const cf_ivs* ivs, const double* inclSpots, int nInclSpots,
                    double maxDs, const double* inclTimes, int nInclTimes, double maxDtVol, int* nS, int* nT,
                    double* spots, double* times, double* lvols);

/* dupireCalib with a risk view (ivs.h:27-81, the calibration of dupireSuperbucketBump,
 * main.h:575-696): the implied vols are shifted by the view's spreads[nStrikes*nMats],
 * smoothstep-interpolated in strike and maturity. */
int cf_dupire_calib_view(cf_context* ctx, const cf_ivs* ivs, const double* inclSpots, int nInclSpots,
                         double maxDs, const double* inclTimes, int nInclTimes, double maxDtVol,
                         const double* rvStrikes, int nStrikes, const double* rvMats, int nMats,
                         const double* spreads, int* nS, int* nT, double* spots, double* times, double* lvols);

/* dupireSuperbucket, main.h:453-569: calibrate, Monte Carlo adjoints to the local vols
 * (microbucket), then the adjoint of the calibration to the risk view's implied-vol
 * spreads.  vega[nStrikes * nMats]; microbucket[nS * nT] optional.  refSeeding = 1
 * reproduces the reference's seeding of the calibration tape by assignment (main.h:541-547),
 * under which flat-extrapolated local vols overwrite instead of add; 0 is the exact adjoint. */
int cf_dupire_superbucket(cf_context* ctx, const cf_ivs* ivs, double spot, double maxDt, const char* productId,
                          const double* notionals, const double* inclSpots, int nInclSpots, double maxDs,
                          const double* inclTimes, int nInclTimes, double maxDtVol, const double* strikes,
                          int nStrikes, const double* mats, int nMats, const cf_num_param* num, int refSeeding,
                          double* value, double* delta, double* vega, double* microbucket);
/* dupireSuperbucketBump, main.h:575-696: the same outputs by bumping: delta by the spot +1e-8
 * on the same local vols, vega[nStrikes][nMats] by each risk-view implied vol +vegaBump (0: the
 * reference's 1e-5), recalibrated and repriced (FP64 valuations on the same random numbers).
 * The reference takes Merton parameters; any cf_ivs is accepted here. */
int cf_dupire_superbucket_bump(cf_context* ctx, const cf_ivs* ivs, double spot, double maxDt, const char* productId,
                               const double* notionals, const double* inclSpots, int nInclSpots, double maxDs,
                               const double* inclTimes, int nInclTimes, double maxDtVol, const double* strikes,
                               int nStrikes, const double* mats, int nMats, const cf_num_param* num, double vegaBump,
                               double* value, double* delta, double* vega);

/* Test hook, no counterpart in the reference: the Dupire calibration's adjoint alone (the
 * second half of dupireSuperbucket, main.h:519-562), seeded with local-vol adjoints
 * micro[nS*nT] (spot-major, refSeeding as in cf_dupire_superbucket) instead of Monte Carlo
 * ones: vega[nStrikes*nMats].  Per node and point, (K,T), (K,T-h), (K,T+h), (K-h,T), (K+h,T)
 * with h = 1e-4, [nT*nS*5] each and optional: calls and callVegas receive the forward's
 * Black-Scholes prices and their derivatives to the implied vol (the values Dupire's formula
 * and its adjoint were taken at), pointAdj the adjoint of each point's implied vol before the
 * risk view's interpolation spreads it; 0 outside each maturity's +-2.5 std window. */
int cf_calib_adjoint(cf_context* ctx, const cf_ivs* ivs, const double* inclSpots, int nInclSpots, double maxDs,
                     const double* inclTimes, int nInclTimes, double maxDtVol, const double* strikes, int nStrikes,
                     const double* mats, int nMats, const double* micro, int refSeeding, double* vega,
                     double* calls, double* callVegas, double* pointAdj);

/* AADriskAggregate without any device allocation.  No counterpart in the reference.
 * For callers that cannot let a library allocate device memory during a call (memory
 * already reserved by another allocator, or a cudaMalloc / cudaFree stall is unacceptable):
 * the same risk kernel as cf_aad_risk_aggregate, with all its device storage in one 64 MiB
 * static device array held by every GPU that loads the library until process exit.  The
 * (model, product) pair must already be lowered (e.g. by cf_shapes); the first call on a
 * device looks up the array's address and should come before any stream capture; calls
 * that overlap on the GPU share the array and race; requests whose scratch does not fit
 * are rejected with CF_E_SHAPE.  Results: payoffValues[nPay], *aggregateValue, risks[nParam]. */
int cf_aad_risk_aggregate_noalloc(cf_context* ctx, const char* modelId, const char* productId,
                                  const double* notionals, const cf_num_param* num, double* payoffValues,
                                  double* aggregateValue, double* risks);

/* ---- RNG access (sobol.h, mrg32k3a.h), for bit-exactness checks -------------------- */
/* Sobol integer points of paths [firstPath, firstPath+nPaths), dimension dim: out[nPaths*dim]. */
int cf_sobol_points(cf_context* ctx, int dim, int64_t firstPath, int nPaths, uint32_t* out);
/* mrg32k3a state (x0,x1,x2,y0,y1,y2) before path firstPath (even) for dimension dim. */
int cf_mrg_state(cf_context* ctx, unsigned seed1, unsigned seed2, int dim, int64_t firstPath, uint32_t* state6);
/* Gaussians of paths [firstPath, firstPath+nPaths): out[nPaths*dim] (FP64 form). */
int cf_gaussians(cf_context* ctx, int useSobol, unsigned seed1, unsigned seed2, int dim, int64_t firstPath,
                 int nPaths, double* out);

/* Uniforms of paths [firstPath, firstPath+nPaths): out[nPaths*dim], what RNG::nextU returns for
 * them (sobol.h:102-108; mrg32k3a.h:117-148, whose odd paths take 1 - u of the pair's first). */
int cf_uniforms(cf_context* ctx, int useSobol, unsigned seed1, unsigned seed2, int dim, int64_t firstPath, int nPaths,
                double* out);

/* ---- model and product shapes (mcBase.h:122-223) ------------------------------------ */
/* Model::allocate + Model::simDim (mcMdlBS.h:149-195, 280-283; mcMdlDupire.h:165-193, 220-223):
 * the Gaussians per path of a Black-Scholes or Dupire model of the store simulated on a product
 * timeline productTimeline[n]. */
int cf_model_sim_dim(cf_context* ctx, const char* modelId, const double* productTimeline, int n, int* simDim);
/* Product::timeline / Product::defline (mcBase.h:131-132) of a product of the store: per event
 * date its time, whether it needs the numeraire, and the maturities of its forward, discount and
 * libor (which starts at the date); NaN where the date has none.  times == NULL: *count only. */
int cf_product_events(cf_context* ctx, const char* productId, double* times, int* needNumeraire, double* forwardMats,
                      double* discountMats, double* liborEnds, int capacity, int* count);

/* ---- device-resident launches (benchmarks and the serving loop) --------------------- */
/* Enqueues the risk (risk=1, weights[nPay]) or value (risk=0) kernel of (model, product)
 * on the context's stream without synchronising; results stay on the device until
 * cf_fetch_result.  Returns the number of kernel launches enqueued in *launches. */
int cf_enqueue(cf_context* ctx, const char* modelId, const char* productId, const cf_num_param* num, int risk,
               const double* weights, int* launches);
/* Synchronises and converts the last enqueued run: values[nPay], stderrs[nPay] (optional),
 * aggregate (optional), risks[nParam] (risk runs, optional). */
int cf_fetch_result(cf_context* ctx, double* values, double* stderrs, double* aggregate, double* risks);

/* ---- shards of one run (one per GPU, or per call) ------------------------------------ */
/* The paths of a Monte Carlo run are independent, and every sum of a run is kept exactly in
 * integer fixed point (pairs of int64: units of 2^-20 and 2^-60).  A run of N paths can
 * therefore be cut into shards of contiguous path ranges, simulated anywhere, and summed
 * exactly (the sharding of mcParallelSimul's path loop, mcBase.h:331-400, across devices):
 *   cf_enqueue_shard   like cf_enqueue, for paths [firstPath, firstPath + num->numPath) of
 *                      the run's random sequence (firstPath a multiple of 64);
 *   cf_fetch_raw       the raw accumulators of the last enqueue (2 * (nParam + 2 nPay + 2)
 *                      int64 words for a risk run, 2 * (2 nPay + 2) for a value run;
 *                      *nWords receives the count);
 *   cf_results_from_raw  values, stderrs, aggregate, risks of accumulators summed over the
 *                      shards (word-wise int64 sums), for the run's total path count: bit-
 *                      identical to one call over all the paths.  Needs no context. */
int cf_enqueue_shard(cf_context* ctx, const char* modelId, const char* productId, const cf_num_param* num,
                     int64_t firstPath, int risk, const double* weights, int* launches);
int cf_fetch_raw(cf_context* ctx, int64_t* acc, int capacity, int* nWords);
int cf_results_from_raw(const int64_t* acc, int nRisk, int nPay, int64_t nPath, double* values, double* stderrs,
                        double* aggregate, double* risks);

/* ---- serving loop (no counterpart in the reference: main.h runs one call at a time on the
 * ThreadPool, threadPool.h:30-172) -------------------------------------------------------- */
typedef struct cf_server cf_server;

/* kind 0 = value, 1 = risk of sum_k weights[k] payoff_k (weights NULL: payoff 0),
 * 2 = AADriskMulti of a European portfolio.  queueTimeoutMs > 0 expires a request that has
 * not started within that time. */
typedef struct {
    int kind;
    const char* modelId;
    const char* productId;
    cf_num_param num;
    const double* weights;
    int nWeights;
    double queueTimeoutMs;
} cf_request;

typedef struct {
    uint64_t submitted, completed, failed, rejected, cancelled, timedOut;
    double p50Ms, p99Ms, meanMs;  /* submit-to-done latency of completed requests */
    uint64_t pathStepsDone;
    int maxInFlight;
    uint64_t peakFootprint;       /* bytes of admitted requests in flight at once, at most */
    double maxStartMs;            /* longest host-side start of a request (launch set-up) */
    double maxStepMs;             /* longest scheduling round of the server thread */
    uint64_t bufferGrowths;       /* device buffers of the slots grown since the stats were reset */
} cf_serving_stats;

/* Request status values of cf_server_wait. */
#define CF_REQ_QUEUED 0
#define CF_REQ_RUNNING 1
#define CF_REQ_DONE 2
#define CF_REQ_FAILED 3
#define CF_REQ_REJECTED 4
#define CF_REQ_CANCELLED 5
#define CF_REQ_TIMEOUT 6

/* A server with `slots` concurrent execution slots (CUDA streams) admitting requests while
 * their device footprint fits hbmBudgetBytes. */
int cf_server_create(cf_context* ctx, int slots, uint64_t hbmBudgetBytes, cf_server** server);
/* Serving policy (before the first request): shortSlots of the server's slots, on streams of the
 * device's highest priority, take only short requests (values, portfolio risks, and risks of at
 * most longThreshold path-steps); the other slots, at the lowest priority, take only the long
 * risks, each launched as consecutive path ranges of at most chunkPathSteps path-steps (0: one
 * launch) with at most longBlocksPerSM resident blocks per SM (0: the kernel's occupancy).  A
 * risk kernel's blocks stay resident until it ends, so a short request waits for SM room: at
 * most the running chunk, or none when long kernels leave room.  Arrival order holds within each
 * class.  Every sum is exact: a request's results do not depend on any of these choices. */
int cf_server_configure(cf_server* server, int shortSlots, double longThreshold, double chunkPathSteps,
                        int longBlocksPerSM);
/* Admission order of a lane (0: the short requests, or all of them without cf_server_configure;
 * 1: the long risks): order 0 is arrival order, order 1 the least work (path-steps) first, where a
 * request that has waited more than agingMs goes first (oldest first), so that small requests do
 * not wait behind large ones and none waits indefinitely. */
int cf_server_order(cf_server* server, int lane, int order, double agingMs);
int cf_server_destroy(cf_server* server);
int cf_server_submit(cf_server* server, const cf_request* request, uint64_t* id);
int cf_server_cancel(cf_server* server, uint64_t id);
/* Blocks until the request leaves the queue / its slot (timeoutMs < 0: no limit). */
int cf_server_wait(cf_server* server, uint64_t id, int timeoutMs, int* status);
/* Results of a finished request: values[nPay], stderrs[nPay] (kind 0/1), *aggregate, risks
 * (kind 1: [nParam], kind 2: [nParam*nPay]), latency from submission to completion. */
int cf_server_result(cf_server* server, uint64_t id, double* values, double* stderrs, double* aggregate,
                     double* risks, double* latencyMs);
/* Forgets a finished request (frees its result storage). */
int cf_server_release(cf_server* server, uint64_t id);
int cf_server_stats(cf_server* server, cf_serving_stats* stats);
/* Starts the statistics afresh (counters, latencies, peaks) on a server that keeps its slots
   and their device buffers, e.g. between a warm-up stream and a measured one. */
int cf_server_reset_stats(cf_server* server);
/* Test hook: the next n request starts fail as if a device allocation had failed. */
int cf_server_inject_failures(cf_server* server, int startFailures);

/* Test hook, no device call: the equal-width buckets over a Dupire model's log-spot knots
 * (ascending floats) that the FP32 kernels search, no counterpart in the reference.  Bucket b
 * is [x0 + b / invW, x0 + (b + 1) / invW); first[b] is the index of the first knot above its
 * left edge.  ok = 1: every bucket holds at most one knot.  oneCompare = 1: besides, no knot
 * lies near a bucket edge, so the FP32 risk kernel finds a state's interval with one
 * comparison (it runs only on such grids).  first == NULL queries *nBuckets only. */
int cf_bucket_grid(const float* knots, int nKnots, int capacity, float* x0, float* invW, int* nBuckets, int* ok,
                   int* oneCompare, int* first);

#ifdef __cplusplus
}
#endif
#endif /* CFGPU_H */
