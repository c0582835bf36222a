// Host engine types behind the C ABI: store entries, lowered plans, the context.
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <utility>
#include <vector>

#include "../../include/cfgpu.h"
#include "cf_params.h"

namespace cf {

int fail(int code, const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);
// return the failure of a CUDA call as a status (CF_E_CUDA / CF_E_NOMEM with the message)
#define CF_CUDA(call)                                       \
    do                                                      \
    {                                                       \
        cudaError_t e_ = (call);                            \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
    } while (0)
double fix_value_host(long long hi, long long lo);
void results_from_acc(const long long* acc, int nRisk, int nPay, long long nPath, double* values, double* stderrs,
                      double* aggregate, double* risks);

struct DevBuf
{
    static std::atomic<unsigned long long> growths;  // allocations made by ensure(), process-wide
    void* ptr = nullptr;
    size_t bytes = 0;
    // grows (never shrinks) the allocation; with a stream, through the stream-ordered allocator
    // on that stream (no device-wide wait: the buffers of serving slots grow while other slots
    // run)
    int ensure(size_t n, cudaStream_t stream = nullptr);
    void release();
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { release(); }
    void swap(DevBuf& o)
    {
        std::swap(ptr, o.ptr);
        std::swap(bytes, o.bytes);
    }
};

// A model of the store (store.h:38-94): Black-Scholes, Dupire, or multiple correlated
// displaced assets.
struct ModelDesc
{
    int kind = MODEL_BS;
    double spot = 0, vol = 0, rate = 0, div = 0;
    bool qSpot = false;
    std::vector<double> spots, times, vols;  // Dupire, vols spot-major
    double maxDt = 0.25;
    // multi-asset displaced (mcMdlMultiDisplaced.h): names, discount rate, per asset spot,
    // repo spread, ATM vol and skew, dividends [nDiv][nA] on divDates, correl [nA][nA] (its
    // lower triangle is the model's), and the correl shift lambda
    std::vector<std::string> assets;
    double disc = 0, lambda = 0;
    std::vector<double> aSpots, spreads, divDates, divs, atms, skews, correl;
    unsigned long long version = 0;
    void build();
    // parameter labels, formatted on first request (a 60x30 grid has 1801: formatting them on
    // every putDupire would cost more than lowering the plan)
    const std::vector<std::string>& labels() const;
    int numParams() const;
    double& param(int i);  // parameter i in label order (bumpRisk)
    const std::vector<std::string>& assetNames() const;

private:
    mutable std::vector<std::string> labels_;
    mutable bool labelsReady_ = false;
};

// A product of the store (store.h:128-255): European, up-and-out, Europeans, contingent
// bond, Baskets, Autocall.
struct ProductDesc
{
    int kind = PROD_EUROPEAN;
    double strike = 0, exercise = 0, settlement = 0, barrier = 0, maturity = 0, freq = 0, smooth = 0;
    double coupon = 0;  // contingent bond
    int callPut = 0;
    std::vector<double> mats, strikes;  // Europeans input pairs; Baskets strikes
    // multi-asset: asset names, basket weights or autocall references, autocall periods, KO, coupon
    std::vector<std::string> assets;
    std::vector<double> weights, refs;
    int periods = 0;
    double ko = 0, cpn = 0;
    // derived
    std::vector<double> timeline, fwdMat, discMat, kflat, libEnd;  // libEnd: libor end per date, NaN if none
    std::vector<int> needNum, payOff;
    std::vector<std::string> labels;
    unsigned long long version = 0;
    void build();
    const std::vector<std::string>& assetNames() const;
};


// The device tables of one (model, product) pair.
struct Plan : std::enable_shared_from_this<Plan>
{
    int model = 0, prod = 0, nSteps = 0, nEv = 0, nPay = 0, nParam = 0;
    bool sobolOk = false;
    bool multi32 = false;  // European portfolio on Dupire with the FP32 tables: multi_risk32.cu
    size_t yBytesD = 0, yBytesF = 0;
    unsigned long long mver = 0, pver = 0;
    std::vector<double> timeline;
    std::vector<int> evAtStep;
    DevBuf tables;
    McParams base;
    // multi-asset model: derived quantities (md_layout) and their Jacobian to the model
    // parameters, [total][nParam], from the host-side adjoint of the model's initialisation
    std::vector<double> mdDerived, mdJac;
    int mdTotal = 0;
};

// Pinned host memory (results are copied into it asynchronously).
struct PinnedBuf
{
    void* ptr = nullptr;
    size_t bytes = 0;
    int ensure(size_t n);
    void release();
    PinnedBuf() = default;
    PinnedBuf(const PinnedBuf&) = delete;
    PinnedBuf& operator=(const PinnedBuf&) = delete;
    ~PinnedBuf() { release(); }
};

// Everything one in-flight run needs: its stream, device buffers, pinned result staging and
// a completion event.  The synchronous API uses the context's main slot; the serving loop
// owns several so that admitted requests overlap on the device.
struct Slot
{
    cudaStream_t stream = nullptr;
    bool ownsStream = false;
    DevBuf work, scratch, multiBuf, paths;
    PinnedBuf hostAcc, hostW;
    cudaEvent_t done = nullptr;
    McParams last;
    Plan* plan = nullptr;
    // keeps the plan of the last run alive (its host data is read when the results are
    // fetched) even if the store replaces it meanwhile; empty for plans the store does not own
    std::shared_ptr<Plan> planRef;
    bool risk = false, multi = false;
    int launches = 0;
    // multi-risk bookkeeping (strike buckets, see multi.cpp)
    std::vector<int> evOff, orig;
    std::vector<double> ks;
    int multiParams = 0;
    long long multiPaths = 0;
    std::vector<double> aggW;  // a multi run's aggregation weights (empty: per-payoff risks)
    size_t accRBytes = 0, accVBytes = 0;
    ~Slot();
};

struct Context
{
    int device = 0;
    cudaStream_t ownStream = nullptr;
    cudaStream_t stream = nullptr;
    int numSMs = 0;
    unsigned long long versionCounter = 0;
    std::map<std::string, ModelDesc> models;
    std::map<std::string, ProductDesc> products;
    std::map<std::pair<std::string, std::string>, std::shared_ptr<Plan>> plans;
    DevBuf jump;
    std::map<int, std::vector<uint32_t>> sobolDirs;  // Sobol direction numbers per dimension count
    const unsigned* jumpA = nullptr;
    const unsigned* jumpB = nullptr;
    DevBuf invn;  // piecewise-cubic inverse normal tables of the FP32 kernels: mrg32k3a, Sobol
    const float* invnMrg = nullptr;
    const float* invnSobol = nullptr;
    Slot main;
    unsigned long long h2d = 0, d2h = 0;  // cumulative transfer bytes

    int init(int dev);
    ~Context();
    int getPlan(const std::string& mid, const std::string& pid, Plan*& out);
    int buildPlan(const ModelDesc& m, const ProductDesc& pd, Plan& plan);
    int buildPlanMd(const ModelDesc& m, const ProductDesc& pd, Plan& plan);  // multi_asset.cpp
    int enqueueMd(Slot& slot, Plan& plan, const cf_num_param& num, bool risk, const double* weights,
                  long long firstPath);
    const ProductDesc* productOf(const Plan& plan) const;
    // pathOut (value runs of the single-asset kernels): device array receiving every path's
    // payoffs [path][nPay].  chunkPaths > 0 (a multiple of 64): the run is launched as
    // consecutive path ranges of at most that many paths, each adding into the same exact
    // accumulators (bit-identical results), so that kernels of other streams get the device
    // between them.  maxBlocksPerSM > 0 caps the launch's resident blocks per SM below the
    // kernel's occupancy, leaving room on every SM for kernels of other streams.
    int enqueue(Slot& slot, Plan& plan, const cf_num_param& num, bool risk, const double* weights,
                long long firstPath = 0, double* pathOut = nullptr, long long chunkPaths = 0,
                int maxBlocksPerSM = 0);
    int fetch(Slot& slot, double* values, double* stderrs, double* aggregate, double* risks);
    bool ready(Slot& slot) const;
    size_t footprint(const Plan& plan, const cf_num_param& num, bool risk) const;
    // AADriskMulti: the multi kernel (European portfolios) is asynchronous like enqueue
    bool multiFast(const Plan& plan) const;
    bool multi32Use(const Plan& plan, const cf_num_param& num) const;  // FP32 Dupire: multi_risk32.cu
    // directRisks: the caller's nParam x nPay array, written before the call returns; aggWeights
    // (nPay): the run's risks are those of the weighted sum of the payoffs (nParam values)
    int enqueueMulti(Slot& slot, Plan& plan, const cf_num_param& num, double* directRisks = nullptr,
                     const double* aggWeights = nullptr);
    int finishMulti(Slot& slot, double* values, double* risks, double* aggregate = nullptr);
    // AADriskOne / AADriskAggregate on the main slot: values, aggregate and risks of sum_k w_k payoff_k
    int aggregateRisk(Plan& plan, const cf_num_param& num, const double* weights, double* values, double* aggregate,
                      double* risks);
    int riskMulti(Plan& plan, const cf_num_param& num, double* values, double* risks);
    // main-slot conveniences of the synchronous API
    int enqueue(Plan& plan, const cf_num_param& num, bool risk, const double* weights, double* pathOut = nullptr)
    {
        main.stream = stream;
        return enqueue(main, plan, num, risk, weights, 0, pathOut);
    }
    int fetch(double* values, double* stderrs, double* aggregate, double* risks)
    {
        return fetch(main, values, stderrs, aggregate, risks);
    }
};

}  // namespace cf

// The opaque handle of the C ABI.
struct cf_context
{
    cf::Context c;
    std::mutex mu;
};
