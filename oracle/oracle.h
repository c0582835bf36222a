/* CPU restatement of the reference's Monte Carlo valuation / AAD-risk path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker of the CUDA engine: only the
 * tests, the smoke check and the benchmark's CPU-baseline leg load it.  The engine
 * (compfinance_gb300/libcfgpu.so) never calls it and has no CPU fallback.
 *
 * Parity of this restatement is pinned against golden fixtures written by the reference
 * itself (tests/golden/, produced by oracle/_ref/ref_driver through main.h's entry points).
 */
#ifndef CF_ORACLE_H
#define CF_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Model description: Black-Scholes (mcMdlBS.h) or Dupire local vol (mcMdlDupire.h). */
typedef struct {
    int kind;               /* 0 = Black-Scholes, 1 = Dupire */
    double spot;
    /* Black-Scholes */
    double vol, rate, div;
    int spot_measure;
    /* Dupire: vols spot-major [nS][nT] */
    int nS, nT;
    const double* spots;
    const double* times;
    const double* vols;
    double maxdt;
} orc_model;

/* Product description (mcPrd.h): European, up-and-out call/put, portfolio of Europeans,
 * contingent bond. */
typedef struct {
    int kind;               /* 0 = European, 1 = UOC, 2 = Europeans, 3 = ContingentBond */
    double strike, exercise, settlement;             /* European */
    double barrier, maturity, freq, smooth;          /* UOC (strike shared); smooth as given to putBarrier;
                                                        ContingentBond: maturity, payment frequency, smooth */
    int callput;
    int n;                  /* Europeans: n (maturity, strike) pairs */
    const double* mats;
    const double* strikes;
    double coupon;          /* ContingentBond */
} orc_product;

/* Shapes: number of payoffs, parameters, Gaussians per path (simDim). */
int orc_shapes(const orc_model* m, const orc_product* p, int* nPay, int* nParam, int* simDim);

/* Per-path payoffs of mcSimul (serial), out[nPath * nPay]. */
int orc_paths(const orc_model* m, const orc_product* p, int sobol, int nPath, unsigned seed1,
              unsigned seed2, double* out);

/* value(): averages over paths; optional standard errors. nThreads > 1 runs path
 * ranges in parallel (same RNG stream, positioned by skip-ahead). */
int orc_value(const orc_model* m, const orc_product* p, int sobol, int nPath, unsigned seed1,
              unsigned seed2, int nThreads, double* values, double* stderrs);

/* AADriskOne / AADriskAggregate through a restated tape: aggregate = sum_k w[k] payoff_k.
 * values[nPay], aggValue, risks[nParam]. */
int orc_risk(const orc_model* m, const orc_product* p, int sobol, int nPath, unsigned seed1,
             unsigned seed2, const double* weights, double* values, double* aggValue, double* risks);

/* AADriskMulti: risks[nParam * nPay] (parameter-major), values[nPay].
 * refMarkQuirk != 0 reproduces the reference's serial multi-adjoint loop exactly, including
 * its second propagation of the first post-mark tape node of the last path; 0 gives the
 * exact path average (what the engine computes). */
int orc_risk_multi(const orc_model* m, const orc_product* p, int sobol, int nPath, unsigned seed1,
                   unsigned seed2, int refMarkQuirk, double* values, double* risks);

/* Hand-written adjoint (no tape) of the Dupire path for any product, multi-threaded: the
 * timed CPU baseline.  Same outputs as orc_risk. */
int orc_risk_fast(const orc_model* m, const orc_product* p, int sobol, int nPath, unsigned seed1,
                  unsigned seed2, const double* weights, int nThreads, double* values,
                  double* aggValue, double* risks);

/* RNG access for bit-exactness tests. */
int orc_sobol_ints(int dim, int64_t firstPath, int nPaths, uint32_t* out);       /* out[nPaths*dim] */
int orc_sobol_gauss(int dim, int64_t firstPath, int nPaths, double* out);
int orc_mrg_gauss(unsigned s1, unsigned s2, int dim, int64_t firstPath, int nPaths, double* out);
int orc_mrg_state(unsigned s1, unsigned s2, int dim, int64_t firstPath, double* state6);
double orc_inv_normal_cdf(double p);
double orc_normal_cdf(double x);

/* Implied-vol surfaces for the calibration: kind 0 = iv(K,T) = a + b ln^2(K/s)/sqrt(T) + c ln(K/s)
 * with params {a,b,c,s}; kind 1 = Merton jump-diffusion {vol, intensity, meanJmp, stdJmp}. */
typedef struct {
    int kind;
    double spot;
    double p[4];
} orc_ivs;

/* dupireCalib: grid sizes first (lvols == NULL), then the grid. lvols spot-major. */
int orc_calib(const orc_ivs* ivs, const double* inclSpots, int nIS, double maxDs,
              const double* inclTimes, int nIT, double maxDtVol, int* nS, int* nT, double* spots,
              double* times, double* lvols);

/* Calibration adjoint: d/d spread[r][c] of sum_ij microbucket[i][j] * lvol[i][j].
 * refSeedQuirk != 0 reproduces the reference's seeding by assignment (main.h:541-547), under
 * which a flat-extrapolated local vol (a copy of its edge node) overwrites instead of adds. */
int orc_calib_adjoint(const orc_ivs* ivs, const double* inclSpots, int nIS, double maxDs,
                      const double* inclTimes, int nIT, double maxDtVol, const double* rvStrikes,
                      int nK, const double* rvMats, int nM, const double* microbucket,
                      int refSeedQuirk, double* vega);

/* The same adjoint, restated pointwise (pointwise != 0): each of a node's five calls, (K,T),
 * (K,T-h), (K,T+h), (K-h,T), (K+h,T) with h = 1e-4, enters the tape as one node of its implied
 * vol with value c and partial d c / d vol.  calls / vegas ([nT][nS][5], NULL: the oracle's own)
 * give them, so that Dupire's formula, its partials, the risk view's interpolation weights and
 * the seeding are restated at those values.  Optional outputs, [nT][nS][5] (0 outside the
 * +-2.5 std window): ownCalls / ownVegas the oracle's own values, pointAdj the adjoint of each
 * point's implied vol; absTerms[nK*nM]: per spread node, the sum over points of |pointAdj| x the
 * point's interpolation weight on the node (the scale of the terms summed into vega).
 * pointwise == 0: the full tape of orc_calib_adjoint. */
int orc_calib_adjoint_given(const orc_ivs* ivs, const double* inclSpots, int nIS, double maxDs,
                            const double* inclTimes, int nIT, double maxDtVol, const double* rvStrikes,
                            int nK, const double* rvMats, int nM, const double* microbucket,
                            int refSeedQuirk, const double* calls, const double* vegas, double* ownCalls,
                            double* ownVegas, double* pointAdj, double* absTerms, double* vega, int pointwise);

/* dupireSuperbucket: value, delta, vega[nK*nM]; microbucket[nS*nT] optional. */
int orc_superbucket(const orc_ivs* ivs, double spot, double maxDt, const orc_product* p,
                    const double* notionals, const double* inclSpots, int nIS, double maxDs,
                    const double* inclTimes, int nIT, double maxDtVol, const double* rvStrikes,
                    int nK, const double* rvMats, int nM, int sobol, int nPath, unsigned seed1,
                    unsigned seed2, int refSeedQuirk, double* value, double* delta, double* vega,
                    double* microbucket);

/* Multiple correlated assets under displaced Black-Scholes dynamics with proportional
 * dividends (mcMdlMultiDisplaced.h), and the multi-asset products (mcPrdMulti.h). */
typedef struct {
    int nA;                 /* assets */
    double disc;            /* discount rate */
    const double* spots;    /* [nA] */
    const double* spreads;  /* [nA] repo spreads */
    int nDiv;
    const double* divDates; /* [nDiv] */
    const double* divs;     /* [nDiv][nA] proportional dividends */
    const double* atms;     /* [nA] */
    const double* skews;    /* [nA] */
    const double* correl;   /* [nA][nA]; the lower triangle is used */
    double lambda;          /* used correl = lambda (1 - correl) + correl */
} orc_mmodel;

typedef struct {
    int kind;               /* 0 = Baskets, 1 = Autocall */
    int nA;
    const double* weights;  /* Baskets [nA] */
    double maturity;
    int nK;
    const double* strikes;  /* Baskets [nK] */
    const double* refs;     /* Autocall [nA] */
    int periods;
    double ko, strike, cpn, smooth;
} orc_mproduct;

int orc_m_shapes(const orc_mmodel* m, const orc_mproduct* p, int* nPay, int* nParam, int* simDim);
int orc_m_value(const orc_mmodel* m, const orc_mproduct* p, int sobol, int nPath, unsigned seed1,
                unsigned seed2, double* values, double* stderrs);
/* AADriskOne / AADriskAggregate (weights[nPay]) and AADriskMulti (risks[nParam * nPay]) */
int orc_m_risk(const orc_mmodel* m, const orc_mproduct* p, int sobol, int nPath, unsigned seed1,
               unsigned seed2, const double* weights, double* values, double* aggValue, double* risks);
int orc_m_risk_multi(const orc_mmodel* m, const orc_mproduct* p, int sobol, int nPath, unsigned seed1,
                     unsigned seed2, double* values, double* risks);
/* Model quantities after init: chol[nA*nA], stds/drifts/ffs[nSteps*nA], alphas[nA],
 * dynamics[nA] (0 lognormal, 1 normal, 2 surnormal, 3 subnormal), numeraires[nEv]. */
int orc_m_init(const orc_mmodel* m, const orc_mproduct* p, double* chol, double* stds, double* drifts,
               double* ffs, double* alphas, int* dynamics, double* numeraires);

/* fillData(utility.h) for host-logic tests; returns count, fills out when non-NULL. */
int orc_fill(const double* x, int n, double maxDx, double minDx, const double* add, int nAdd,
             double* out);

#ifdef __cplusplus
}
#endif
#endif
