// dupireCalib and dupireSuperbucket (main.h:414-569) on the GPU.
//
// The superbucket is differentiated by checkpointing, as in the reference: the Monte Carlo
// adjoint kernel gives the risk to every local vol (the microbucket), then a separate FP64
// adjoint of the calibration maps it to the risk view's implied-vol spreads.
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "calib_params.h"
#include "engine.h"
#include "host_math.h"

namespace cf {



namespace {

double host_implied(const cf_ivs& s, double K, double T)
{
    if (s.kind == 0)
    {
        const double l = std::log(K / s.p[3]);
        return s.p[0] + s.p[1] * l * l / std::sqrt(T) + s.p[2] * l;
    }
    return black_scholes_ivol(s.spot, K, merton_price(s.spot, K, s.p[0], T, s.p[1], s.p[2], s.p[3]), T);
}

struct CalibRun
{
    std::vector<double> spots, times;
    std::vector<int> il, ih;
    DevBuf buf;
    CalibParams P;
    double* pointAdjBuf = nullptr;  // room for the per-point adjoints of the test hook
};

// Grid (fillData) and the +-2.5 std window of each maturity (mcMdlDupire.h:299-312) on the
// host, exactly as the reference decides them; the 5 calls per node and Dupire's formula on
// the GPU.
int calibrate(Context& c, const cf_ivs& ivs, const double* inclSpots, int nIS, double maxDs, const double* inclTimes,
              int nIT, double maxDtVol, const double* rvK, int nK, const double* rvM, int nM, CalibRun& r,
              const double* spreads = nullptr)
{
    if (!inclSpots || !inclTimes || nIS < 1 || nIT < 1) return fail(CF_E_ARG, "dupireCalib: empty grid");
    if (ivs.kind != 0 && ivs.kind != 1) return fail(CF_E_ARG, "dupireCalib: unknown IVS kind");
    r.spots = fill_data(std::vector<double>(inclSpots, inclSpots + nIS), maxDs, 0.01);
    r.times = fill_data(std::vector<double>(inclTimes, inclTimes + nIT), maxDtVol, kOneHour, {maxDtVol});
    const int nS = int(r.spots.size()), nT = int(r.times.size());
    r.il.resize(nT);
    r.ih.resize(nT);
    for (int j = 0; j < nT; ++j)
    {
        const double T = r.times[j];
        const double atm = black_scholes(ivs.spot, ivs.spot, host_implied(ivs, ivs.spot, T), T);
        const double sd = atm * 2.506628274631;
        int il = 0;
        while (il < nS && r.spots[il] < ivs.spot - 2.5 * sd) ++il;
        int ih = nS - 1;
        while (ih >= 0 && r.spots[ih] > ivs.spot + 2.5 * sd) --ih;
        if (il > ih) return fail(CF_E_SHAPE, "dupireCalib: no spot inside 2.5 std at maturity " + std::to_string(T));
        r.il[j] = il;
        r.ih[j] = ih;
    }
    const size_t n5 = size_t(nS) * nT * 5;
    const size_t bytes = (nS + nT + nK + nM) * 8 + 2 * nT * 4 + 3 * n5 * 8 + size_t(nS) * nT * 16 +
                         size_t(nK) * nM * 24 + 4096;
    int rc = r.buf.ensure(bytes);
    if (rc) return rc;
    char* d = static_cast<char*>(r.buf.ptr);
    size_t off = 0;
    auto take = [&](size_t n) {
        char* p = d + off;
        off += (n + 255) & ~size_t(255);
        return p;
    };
    CalibParams& P = r.P;
    std::memset(&P, 0, sizeof(P));
    P.ivsKind = ivs.kind;
    P.spot = ivs.spot;
    for (int k = 0; k < 4; ++k) P.ivp[k] = ivs.p[k];
    P.nS = nS;
    P.nT = nT;
    P.nK = nK;
    P.nM = nM;
    double* dS = (double*)take(nS * 8);
    double* dT = (double*)take(nT * 8);
    int* dil = (int*)take(nT * 4);
    int* dih = (int*)take(nT * 4);
    P.c = (double*)take(n5 * 8);
    P.vega = (double*)take(n5 * 8);
    r.pointAdjBuf = (double*)take(n5 * 8);  // the test hook's per-point adjoints (P.pointAdj set there)
    P.lvT = (double*)take(size_t(nS) * nT * 8);
    double* dSeed = (double*)take(size_t(nS) * nT * 8);
    P.seed = dSeed;
    double* dK = (double*)take(size_t(nK) * 8 + 8);
    double* dM = (double*)take(size_t(nM) * 8 + 8);
    P.acc = (long long*)take(size_t(nK) * nM * 16 + 16);
    double* dSp = (double*)take(size_t(nK) * nM * 8 + 8);
    P.spreads = spreads ? dSp : nullptr;
    P.spots = dS;
    P.times = dT;
    P.il = dil;
    P.ih = dih;
    P.rvK = dK;
    P.rvM = dM;
    cudaStream_t s = c.stream;
    if (cudaMemcpyAsync(dS, r.spots.data(), nS * 8, cudaMemcpyHostToDevice, s) ||
        cudaMemcpyAsync(dT, r.times.data(), nT * 8, cudaMemcpyHostToDevice, s) ||
        cudaMemcpyAsync(dil, r.il.data(), nT * 4, cudaMemcpyHostToDevice, s) ||
        cudaMemcpyAsync(dih, r.ih.data(), nT * 4, cudaMemcpyHostToDevice, s) ||
        (nK && cudaMemcpyAsync(dK, rvK, nK * 8, cudaMemcpyHostToDevice, s)) ||
        (nM && cudaMemcpyAsync(dM, rvM, nM * 8, cudaMemcpyHostToDevice, s)) ||
        (spreads && cudaMemcpyAsync(dSp, spreads, size_t(nK) * nM * 8, cudaMemcpyHostToDevice, s)))
        return cuda_fail(cudaGetLastError(), "calibration upload");
    // points outside each maturity's window are never priced: zero, for the readers of the calls
    if (cudaMemsetAsync(P.c, 0, n5 * 8, s) != cudaSuccess || cudaMemsetAsync(P.vega, 0, n5 * 8, s) != cudaSuccess)
        return cuda_fail(cudaGetLastError(), "calibration reset");
    rc = launch_calib(P, 0, s);
    if (rc) return cuda_fail(cudaError_t(rc), "calibration kernels");
    return CF_OK;
}

// The calibration adjoint (the second half of main.h:519-562): local-vol adjoints micro[nS][nT]
// -> d / d risk-view spread, vega[nK][nM].  A flat-extrapolated local vol is a copy of the edge
// node of its maturity, so its adjoint belongs to that node: added (exact adjoint) or, with
// refSeeding, assigned as the reference's seeding by assignment does (main.h:541-547).
int calib_adjoint(Context& c, CalibRun& r, const double* micro, int refSeeding, double* vega)
{
    const int nS = r.P.nS, nT = r.P.nT, nK = r.P.nK, nM = r.P.nM;
    std::vector<double> seed(size_t(nS) * nT, 0.0);
    for (int i = 0; i < nS; ++i)
        for (int j = 0; j < nT; ++j)
        {
            const int src = i < r.il[j] ? r.il[j] : i > r.ih[j] ? r.ih[j] : i;
            double& sd = seed[size_t(src) * nT + j];
            if (refSeeding) sd = micro[size_t(i) * nT + j];
            else sd += micro[size_t(i) * nT + j];
        }
    cudaError_t e = cudaMemcpyAsync((void*)r.P.seed, seed.data(), seed.size() * 8, cudaMemcpyHostToDevice, c.stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(r.P.acc, 0, size_t(nK) * nM * 16, c.stream);
    if (e != cudaSuccess) return cuda_fail(e, "calibration adjoint upload");
    const int rc = launch_calib(r.P, 1, c.stream);
    if (rc) return cuda_fail(cudaError_t(rc), "calibration adjoint");
    std::vector<long long> acc(size_t(nK) * nM * 2);
    e = cudaMemcpyAsync(acc.data(), r.P.acc, acc.size() * 8, cudaMemcpyDeviceToHost, c.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
    if (e != cudaSuccess) return cuda_fail(e, "calibration adjoint fetch");
    for (int k = 0; k < nK * nM; ++k) vega[k] = fix_value_host(acc[2 * k], acc[2 * k + 1]);
    return CF_OK;
}

int fetch_lvols(Context& c, CalibRun& r, std::vector<double>& lvols)
{
    const int nS = r.P.nS, nT = r.P.nT;
    std::vector<double> lvT(size_t(nS) * nT);
    cudaError_t e = cudaMemcpyAsync(lvT.data(), r.P.lvT, lvT.size() * 8, cudaMemcpyDeviceToHost, c.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
    if (e != cudaSuccess) return cuda_fail(e, "calibration fetch");
    lvols.resize(lvT.size());
    for (int i = 0; i < nS; ++i)
        for (int j = 0; j < nT; ++j) lvols[size_t(i) * nT + j] = lvT[size_t(j) * nS + i];  // transpose
    return CF_OK;
}

}  // namespace
}  // namespace cf

using namespace cf;

extern "C" {

int cf_dupire_calib(cf_context* ctx, const cf_ivs* ivs, const double* inclSpots, int nInclSpots, double maxDs,
                    const double* inclTimes, int nInclTimes, double maxDtVol, int* nS, int* nT, double* spots,
                    double* times, double* lvols)
{
    return cf_dupire_calib_view(ctx, ivs, inclSpots, nInclSpots, maxDs, inclTimes, nInclTimes, maxDtVol, nullptr, 0,
                                nullptr, 0, nullptr, nS, nT, spots, times, lvols);
}

int cf_dupire_calib_view(cf_context* ctx, const cf_ivs* ivs, const double* inclSpots, int nInclSpots, double maxDs,
                         const double* inclTimes, int nInclTimes, double maxDtVol, const double* rvStrikes,
                         int nStrikes, const double* rvMats, int nMats, const double* spreads, int* nS, int* nT,
                         double* spots, double* times, double* lvols)
{
    if (spreads && (!rvStrikes || !rvMats || nStrikes < 1 || nMats < 1))
        return fail(CF_E_ARG, "dupireCalib: spreads need a risk view");
    if (!ctx || !ivs || !nS || !nT) return fail(CF_E_ARG, "null argument");
    std::lock_guard<std::mutex> lock(ctx->mu);
    cudaSetDevice(ctx->c.device);
    if (!lvols)
    {
        const auto s = fill_data(std::vector<double>(inclSpots, inclSpots + nInclSpots), maxDs, 0.01);
        const auto t = fill_data(std::vector<double>(inclTimes, inclTimes + nInclTimes), maxDtVol, kOneHour, {maxDtVol});
        *nS = int(s.size());
        *nT = int(t.size());
        return CF_OK;
    }
    CalibRun r;
    int rc = calibrate(ctx->c, *ivs, inclSpots, nInclSpots, maxDs, inclTimes, nInclTimes, maxDtVol, rvStrikes,
                       spreads ? nStrikes : 0, rvMats, spreads ? nMats : 0, r, spreads);
    if (rc) return rc;
    std::vector<double> lv;
    if ((rc = fetch_lvols(ctx->c, r, lv))) return rc;
    *nS = int(r.spots.size());
    *nT = int(r.times.size());
    if (spots) std::memcpy(spots, r.spots.data(), r.spots.size() * 8);
    if (times) std::memcpy(times, r.times.data(), r.times.size() * 8);
    std::memcpy(lvols, lv.data(), lv.size() * 8);
    return CF_OK;
}

int cf_dupire_superbucket(cf_context* ctx, const cf_ivs* ivs, double spot, double maxDt, const char* productId,
                          const double* notionals, const double* inclSpots, int nInclSpots, double maxDs,
                          const double* inclTimes, int nInclTimes, double maxDtVol, const double* strikes, int nStrikes,
                          const double* mats, int nMats, const cf_num_param* num, int refSeeding, double* value,
                          double* delta, double* vega, double* microbucket)
{
    if (!ctx || !ivs || !productId || !notionals || !num || !value || !delta || !vega)
        return fail(CF_E_ARG, "null argument");
    if (nStrikes < 1 || nMats < 1 || !strikes || !mats) return fail(CF_E_ARG, "superbucket: empty risk view");
    std::lock_guard<std::mutex> lock(ctx->mu);
    Context& c = ctx->c;
    cudaSetDevice(c.device);
    if (!c.products.count(productId)) return fail(CF_E_NOTFOUND, "superbucket: product not found");
    // 1. calibrate (value), 2. store the model, 3. Monte Carlo adjoints (microbucket)
    CalibRun r;
    int rc = calibrate(c, *ivs, inclSpots, nInclSpots, maxDs, inclTimes, nInclTimes, maxDtVol, strikes, nStrikes,
                       mats, nMats, r);
    if (rc) return rc;
    std::vector<double> lv;
    if ((rc = fetch_lvols(c, r, lv))) return rc;
    const int nS = r.P.nS, nT = r.P.nT;
    ModelDesc m;
    m.kind = MODEL_DUPIRE;
    m.spot = spot;
    m.spots = r.spots;
    m.times = r.times;
    m.vols = lv;
    m.maxDt = maxDt;
    m.version = ++c.versionCounter;
    m.build();
    const std::string mid = "\x01superbucket";
    c.models[mid] = std::move(m);
    Plan* plan;
    if ((rc = c.getPlan(mid, productId, plan))) return rc;
    std::vector<double> risks(plan->nParam);
    if ((rc = c.aggregateRisk(*plan, *num, notionals, nullptr, value, risks.data()))) return rc;
    *delta = risks[0];
    const double* micro = risks.data() + 1;
    if (microbucket) std::memcpy(microbucket, micro, size_t(nS) * nT * 8);
    // 4. the calibration adjoint, seeded with the microbucket
    if ((rc = calib_adjoint(c, r, micro, refSeeding, vega))) return rc;
    c.main.launches = 4;
    return CF_OK;
}

int cf_calib_adjoint(cf_context* ctx, const cf_ivs* ivs, const double* inclSpots, int nInclSpots, double maxDs,
                     const double* inclTimes, int nInclTimes, double maxDtVol, const double* strikes, int nStrikes,
                     const double* mats, int nMats, const double* micro, int refSeeding, double* vega, double* calls,
                     double* callVegas, double* pointAdj)
{
    if (!ctx || !ivs || !micro || !vega) return fail(CF_E_ARG, "null argument");
    if (nStrikes < 1 || nMats < 1 || !strikes || !mats) return fail(CF_E_ARG, "calibration adjoint: empty risk view");
    std::lock_guard<std::mutex> lock(ctx->mu);
    Context& c = ctx->c;
    cudaSetDevice(c.device);
    CalibRun r;
    int rc = calibrate(c, *ivs, inclSpots, nInclSpots, maxDs, inclTimes, nInclTimes, maxDtVol, strikes, nStrikes,
                       mats, nMats, r);
    if (rc) return rc;
    const size_t n5 = size_t(r.P.nS) * r.P.nT * 5;
    r.P.pointAdj = pointAdj ? r.pointAdjBuf : nullptr;
    cudaError_t e = cudaSuccess;
    if (r.P.pointAdj) e = cudaMemsetAsync(r.P.pointAdj, 0, n5 * 8, c.stream);
    if (e == cudaSuccess && calls) e = cudaMemcpyAsync(calls, r.P.c, n5 * 8, cudaMemcpyDeviceToHost, c.stream);
    if (e == cudaSuccess && callVegas) e = cudaMemcpyAsync(callVegas, r.P.vega, n5 * 8, cudaMemcpyDeviceToHost, c.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
    if (e != cudaSuccess) return cuda_fail(e, "calibration prices fetch");
    int rc2 = calib_adjoint(c, r, micro, refSeeding, vega);
    if (rc2 || !pointAdj) return rc2;
    e = cudaMemcpyAsync(pointAdj, r.P.pointAdj, n5 * 8, cudaMemcpyDeviceToHost, c.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
    if (e != cudaSuccess) return cuda_fail(e, "calibration point adjoints fetch");
    return CF_OK;
}

// dupireSuperbucketBump, main.h:575-696: the superbucket by bumping.  The base book value
// of the calibrated model; delta by the spot bumped by 1e-8 on the same local vols; vega[i][j]
// by each risk-view implied vol bumped by vegaBump (the reference's 1e-5 by default),
// recalibrated and repriced.  All valuations
// in FP64 on the same random numbers.
int cf_dupire_superbucket_bump(cf_context* ctx, const cf_ivs* ivs, double spot, double maxDt, const char* productId,
                               const double* notionals, const double* inclSpots, int nInclSpots, double maxDs,
                               const double* inclTimes, int nInclTimes, double maxDtVol, const double* strikes,
                               int nStrikes, const double* mats, int nMats, const cf_num_param* num, double vegaBump,
                               double* value, double* delta, double* vega)
{
    const double h = vegaBump > 0.0 ? vegaBump : 1.0e-05;  // main.h:674
    if (!ctx || !ivs || !productId || !notionals || !num || !value || !delta || !vega)
        return fail(CF_E_ARG, "null argument");
    if (nStrikes < 1 || nMats < 1 || !strikes || !mats) return fail(CF_E_ARG, "superbucket: empty risk view");
    std::lock_guard<std::mutex> lock(ctx->mu);
    Context& c = ctx->c;
    cudaSetDevice(c.device);
    if (!c.products.count(productId)) return fail(CF_E_NOTFOUND, "dupireSuperbucketBump() : product not found");
    cf_num_param n64 = *num;
    n64.precision = CF_FP64;
    const std::string mid = "\x01superbucketBump";
    int rc = CF_OK;
    // the book value sum_k notionals[k] value_k of a Dupire model on the given local vols
    auto book = [&](const CalibRun& r, const std::vector<double>& lv, double s0, double& out) -> int {
        ModelDesc m;
        m.kind = MODEL_DUPIRE;
        m.spot = s0;
        m.spots = r.spots;
        m.times = r.times;
        m.vols = lv;
        m.maxDt = maxDt;
        m.version = ++c.versionCounter;
        m.build();
        c.models[mid] = std::move(m);
        Plan* plan;
        int e = c.getPlan(mid, productId, plan);
        if (e) return e;
        std::vector<double> v(plan->nPay);
        if ((e = c.enqueue(*plan, n64, false, nullptr)) || (e = c.fetch(v.data(), nullptr, nullptr, nullptr))) return e;
        out = 0.0;
        for (int k = 0; k < plan->nPay; ++k) out += notionals[k] * v[k];  // inner_product in payoff order
        return CF_OK;
    };
    CalibRun base;
    std::vector<double> lv;
    if ((rc = calibrate(c, *ivs, inclSpots, nInclSpots, maxDs, inclTimes, nInclTimes, maxDtVol, strikes, nStrikes,
                        mats, nMats, base)) ||
        (rc = fetch_lvols(c, base, lv)) || (rc = book(base, lv, spot, *value)))
        return rc;
    double up = 0.0;
    if ((rc = book(base, lv, spot + 1.0e-08, up))) return rc;
    *delta = (up - *value) * 1.0e+08;
    std::vector<double> spreads(size_t(nStrikes) * nMats, 0.0);
    for (int i = 0; i < nStrikes; ++i)
        for (int j = 0; j < nMats; ++j)
        {
            spreads[size_t(i) * nMats + j] = h;
            CalibRun r;
            std::vector<double> lvb;
            double b = 0.0;
            if ((rc = calibrate(c, *ivs, inclSpots, nInclSpots, maxDs, inclTimes, nInclTimes, maxDtVol, strikes,
                                nStrikes, mats, nMats, r, spreads.data())) ||
                (rc = fetch_lvols(c, r, lvb)) || (rc = book(r, lvb, spot, b)))
                return rc;
            vega[size_t(i) * nMats + j] = (b - *value) / h;
            spreads[size_t(i) * nMats + j] = 0.0;
        }
    c.models.erase(mid);
    return CF_OK;
}

}  // extern "C"
