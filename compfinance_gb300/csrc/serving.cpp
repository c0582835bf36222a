// Serving loop: continuous batching of pricing / risk requests on one GPU.
//
// Optional policy (cf_server_configure): short requests (values, portfolio risks, small risks)
// take their own slots, whose streams have the device's highest priority, and long risks the
// other slots, at the lowest priority, launched in chunks of bounded work and with at most a
// given number of resident blocks per SM.  A risk kernel's blocks stay resident for its whole
// launch, so a short request that starts meanwhile waits for SM room: at most the running chunk,
// or none when the long kernels leave room; arrival order holds within each class.
// A server owns N execution slots (a CUDA stream each, with its own device buffers and
// pinned result staging) and a scheduler thread.  Requests are submitted from any thread;
// the scheduler admits them in arrival order as slots and device memory free up (the memory
// currency is each request's footprint: reverse-sweep scratch plus accumulators), so work that
// arrives while other requests run overlaps with them on the device.  Models, products and
// their lowered tables stay resident in the context between requests.  Results are
// bit-identical whether a request runs alone or in the mix: every sum is exact fixed point
// and every path's random numbers are fixed by its index.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "engine.h"
#include "serving_core.h"

namespace cf {

extern thread_local std::string g_lastError;

struct Request
{
    int kind = 0;  // 0 value, 1 risk (weights), 2 multi
    std::string mid, pid;
    cf_num_param num{};
    std::vector<double> w;
    int nPay = 0, nParam = 0;
    std::vector<double> values, stderrs;
    std::vector<double> risks;  // the first nRisks entries hold the result (a buffer from the pool)
    size_t nRisks = 0;
    double agg = 0;
};

class GpuExec
{
public:
    Context& c;
    std::vector<std::unique_ptr<Slot>> slots;
    std::map<uint64_t, Request>& reqs;
    std::string err;
    int injectStartFailures = 0;
    double chunkPathSteps = 0;  // long requests: most path-steps per launch (0: one launch)
    int longBlocksPerSM = 0;    // long requests: most resident blocks per SM (0: the kernel's occupancy)

    GpuExec(Context& ctx, int n, std::map<uint64_t, Request>& r) : c(ctx), reqs(r)
    {
        for (int i = 0; i < n; ++i)
        {
            auto s = std::make_unique<Slot>();
            cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
            s->ownsStream = true;
            slots.push_back(std::move(s));
        }
    }

    double maxStart = 0;  // seconds, longest start() since the stats were reset

    int start(serve::Job& j, int s)
    {
        const auto t0 = std::chrono::steady_clock::now();
        const int rc = startImpl(j, s);
        maxStart = std::max(maxStart, std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count());
        return rc;
    }

    int startImpl(serve::Job& j, int s)
    {
        if (injectStartFailures > 0)
        {
            --injectStartFailures;
            err = "injected allocation failure";
            return CF_E_NOMEM;
        }
        Request& r = reqs[j.id];
        Plan* plan = nullptr;
        int rc = c.getPlan(r.mid, r.pid, plan);
        if (!rc)
        {
            r.nPay = plan->nPay;
            r.nParam = plan->nParam;
            if (r.kind == 2) rc = c.enqueueMulti(*slots[s], *plan, r.num);
            else
            {
                if (r.kind == 1 && r.w.empty())
                {
                    r.w.assign(plan->nPay, 0.0);
                    r.w[0] = 1.0;
                }
                long long chunk = 0;
                if (j.lane == 1 && chunkPathSteps > 0)
                    chunk = std::max(64LL, (long long)(chunkPathSteps / std::max(1, plan->nSteps)) & ~63LL);
                rc = c.enqueue(*slots[s], *plan, r.num, r.kind == 1, r.w.empty() ? nullptr : r.w.data(), 0, nullptr,
                               chunk, j.lane == 1 ? longBlocksPerSM : 0);
            }
        }
        if (rc) err = g_lastError;
        return rc;
    }

    bool poll(int s) { return c.ready(*slots[s]); }

    // Result buffers of released requests, reused: a portfolio's risks (up to nParam x nPay
    // doubles, 11.5 MB at 7201 x 200) are copied out of the slot in the scheduler thread, and a
    // fresh allocation of that size would first fault its pages in
    std::vector<std::vector<double>> spare;

    int finish(serve::Job& j, int s)
    {
        Request& r = reqs[j.id];
        r.values.assign(r.nPay, 0.0);
        r.stderrs.assign(r.nPay, 0.0);
        r.nRisks = r.kind == 0 ? 0 : (r.kind == 2 ? size_t(r.nParam) * r.nPay : size_t(r.nParam));
        if (r.nRisks && r.risks.size() < r.nRisks)
        {
            if (!spare.empty())
            {
                r.risks.swap(spare.back());
                spare.pop_back();
            }
            if (r.risks.size() < r.nRisks) r.risks.resize(r.nRisks);
        }
        const int rc = c.fetch(*slots[s], r.values.data(), r.kind == 2 ? nullptr : r.stderrs.data(), &r.agg,
                               r.nRisks ? r.risks.data() : nullptr);
        if (rc) err = g_lastError;
        return rc;
    }

    // a released request's result buffer goes back to the pool (at most 64 kept)
    void recycle(Request& r)
    {
        if (r.risks.size() >= 4096 && spare.size() < 64) spare.push_back(std::move(r.risks));
    }

    std::string error() const { return err; }
};

}  // namespace cf

using namespace cf;

struct cf_server
{
    cf_context* ctx;
    std::map<uint64_t, Request> reqs;
    GpuExec ex;
    serve::Scheduler<GpuExec> sched;
    std::mutex mu;
    std::condition_variable wake, done;
    std::thread th;
    bool stop = false;
    std::chrono::steady_clock::time_point t0;
    double longThreshold = -1;  // risks above this many path-steps are long (lane 1); < 0: one lane
    double maxStep = 0;         // seconds, longest scheduling round since the stats were reset
    unsigned long long growths0 = 0;

    cf_server(cf_context* c, int slots, size_t budget)
        : ctx(c), ex(c->c, slots, reqs), sched(ex, slots, budget), t0(std::chrono::steady_clock::now())
    {
    }
    double now() const
    {
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
    void loop()
    {
        cudaSetDevice(ctx->c.device);
        while (true)
        {
            int changes;
            bool idle;
            {
                std::lock_guard<std::mutex> a(ctx->mu);
                std::lock_guard<std::mutex> b(mu);
                if (stop) return;
                const double tStep = now();
                changes = sched.step(tStep);
                maxStep = std::max(maxStep, now() - tStep);
                idle = sched.idle();
            }
            if (changes) done.notify_all();
            if (idle)
            {
                std::unique_lock<std::mutex> l(mu);
                wake.wait_for(l, std::chrono::milliseconds(2));
            }
            else if (!changes)
                std::this_thread::sleep_for(std::chrono::microseconds(20));
        }
    }
};

extern "C" {

int cf_server_create(cf_context* ctx, int slots, uint64_t hbmBudgetBytes, cf_server** out)
{
    if (!ctx || !out || slots < 1 || slots > 64) return fail(CF_E_ARG, "server: 1..64 slots");
    std::lock_guard<std::mutex> lock(ctx->mu);
    cudaSetDevice(ctx->c.device);
    auto s = std::make_unique<cf_server>(ctx, slots, size_t(hbmBudgetBytes));
    s->th = std::thread([p = s.get()] { p->loop(); });
    *out = s.release();
    return CF_OK;
}

int cf_server_configure(cf_server* s, int shortSlots, double longThreshold, double chunkPathSteps,
                        int longBlocksPerSM)
{
    if (!s) return fail(CF_E_ARG, "null server");
    const int n = int(s->ex.slots.size());
    if (shortSlots < 1 || shortSlots >= n) return fail(CF_E_ARG, "server: 1 <= shortSlots < slots");
    if (longThreshold < 0 || chunkPathSteps < 0 || longBlocksPerSM < 0)
        return fail(CF_E_ARG, "server: negative threshold, chunk or block cap");
    std::lock_guard<std::mutex> a(s->ctx->mu);
    std::lock_guard<std::mutex> b(s->mu);
    if (!s->sched.idle() || s->sched.submitted_) return fail(CF_E_ARG, "server: configure before the first request");
    int least = 0, greatest = 0;
    cudaSetDevice(s->ctx->c.device);
    if (cudaDeviceGetStreamPriorityRange(&least, &greatest) != cudaSuccess)
        return cuda_fail(cudaGetLastError(), "stream priorities");
    std::vector<int> lanes(n);
    for (int i = 0; i < n; ++i)
    {
        lanes[i] = i < shortSlots ? 0 : 1;
        Slot& sl = *s->ex.slots[i];
        cudaStream_t st = nullptr;
        if (cudaStreamCreateWithPriority(&st, cudaStreamNonBlocking, lanes[i] ? least : greatest) != cudaSuccess)
            return cuda_fail(cudaGetLastError(), "stream with priority");
        if (sl.stream) cudaStreamDestroy(sl.stream);
        sl.stream = st;
        sl.ownsStream = true;
    }
    s->sched.setLanes(lanes);
    s->longThreshold = longThreshold;
    s->ex.chunkPathSteps = chunkPathSteps;
    s->ex.longBlocksPerSM = longBlocksPerSM;
    return CF_OK;
}

int cf_server_order(cf_server* s, int lane, int order, double agingMs)
{
    if (!s) return fail(CF_E_ARG, "null server");
    if (lane < 0 || lane > 1 || order < 0 || order > 1 || agingMs < 0)
        return fail(CF_E_ARG, "server: lane 0 or 1, order 0 or 1, aging >= 0");
    std::lock_guard<std::mutex> b(s->mu);
    s->sched.setLaneOrder(lane, order, agingMs * 1e-3);
    return CF_OK;
}

int cf_server_destroy(cf_server* s)
{
    if (!s) return CF_OK;
    {
        std::lock_guard<std::mutex> l(s->mu);
        s->stop = true;
    }
    s->wake.notify_all();
    s->th.join();
    // drain in-flight work before the slots (streams, buffers) go away
    for (auto& sl : s->ex.slots)
        if (sl->stream) cudaStreamSynchronize(sl->stream);
    delete s;
    return CF_OK;
}

int cf_server_submit(cf_server* s, const cf_request* r, uint64_t* id)
{
    if (!s || !r || !id || !r->modelId || !r->productId) return fail(CF_E_ARG, "server: malformed request");
    if (r->kind < 0 || r->kind > 2) return fail(CF_E_ARG, "server: unknown request kind");
    if (r->num.numPath <= 0) return fail(CF_E_ARG, "server: numPath must be positive");
    std::lock_guard<std::mutex> a(s->ctx->mu);
    Plan* plan = nullptr;
    int rc = s->ctx->c.getPlan(r->modelId, r->productId, plan);  // also validates the ids
    if (rc) return rc;
    if (r->kind == 2 && !s->ctx->c.multiFast(*plan))
        return fail(CF_E_UNSUPPORTED, "server: multi-risk requests need a European portfolio");
    if (r->weights && r->nWeights != plan->nPay) return fail(CF_E_SHAPE, "server: weights size != payoffs");
    Request q;
    q.kind = r->kind;
    q.mid = r->modelId;
    q.pid = r->productId;
    q.num = r->num;
    if (r->weights) q.w.assign(r->weights, r->weights + r->nWeights);
    const size_t fp = s->ctx->c.footprint(*plan, r->num, r->kind != 0);
    const long long work = (long long)r->num.numPath * plan->nSteps;
    {
        std::lock_guard<std::mutex> b(s->mu);
        const int lane = s->longThreshold >= 0 && r->kind == 1 && double(work) > s->longThreshold ? 1 : 0;
        *id = s->sched.submit(fp, r->queueTimeoutMs / 1000.0, s->now(), work, lane);
        s->reqs[*id] = std::move(q);
    }
    s->wake.notify_all();
    return CF_OK;
}

int cf_server_cancel(cf_server* s, uint64_t id)
{
    if (!s) return fail(CF_E_ARG, "null server");
    std::lock_guard<std::mutex> b(s->mu);
    if (!s->sched.cancel(id, s->now())) return fail(CF_E_ARG, "server: request not queued");
    s->done.notify_all();
    return CF_OK;
}

int cf_server_wait(cf_server* s, uint64_t id, int timeoutMs, int* status)
{
    if (!s || !status) return fail(CF_E_ARG, "null argument");
    std::unique_lock<std::mutex> l(s->mu);
    auto finished = [&] {
        const serve::Job* j = s->sched.get(id);
        return !j || (j->status != serve::QUEUED && j->status != serve::RUNNING);
    };
    if (timeoutMs < 0) s->done.wait(l, finished);
    else s->done.wait_for(l, std::chrono::milliseconds(timeoutMs), finished);
    const serve::Job* j = s->sched.get(id);
    if (!j) return fail(CF_E_NOTFOUND, "server: unknown request");
    *status = j->status;
    if (j->status == serve::FAILED || j->status == serve::REJECTED || j->status == serve::TIMEOUT)
        g_lastError = j->error;
    return CF_OK;
}

int cf_server_result(cf_server* s, uint64_t id, double* values, double* stderrs, double* aggregate, double* risks,
                     double* latencyMs)
{
    if (!s) return fail(CF_E_ARG, "null server");
    std::lock_guard<std::mutex> l(s->mu);
    const serve::Job* j = s->sched.get(id);
    if (!j) return fail(CF_E_NOTFOUND, "server: unknown request");
    if (j->status != serve::DONE) return fail(CF_E_ARG, "server: request not done (" + j->error + ")");
    const Request& r = s->reqs[id];
    if (values) std::memcpy(values, r.values.data(), r.values.size() * 8);
    if (stderrs) std::memcpy(stderrs, r.stderrs.data(), r.stderrs.size() * 8);
    if (aggregate) *aggregate = r.agg;
    if (risks) std::memcpy(risks, r.risks.data(), r.nRisks * 8);
    if (latencyMs) *latencyMs = 1000.0 * (j->tDone - j->tSubmit);
    return CF_OK;
}

int cf_server_release(cf_server* s, uint64_t id)
{
    if (!s) return fail(CF_E_ARG, "null server");
    std::lock_guard<std::mutex> l(s->mu);
    const serve::Job* j = s->sched.get(id);
    if (j && (j->status == serve::QUEUED || j->status == serve::RUNNING))
        return fail(CF_E_ARG, "server: request still in flight");
    s->sched.forget(id);
    auto it = s->reqs.find(id);
    if (it != s->reqs.end())
    {
        s->ex.recycle(it->second);
        s->reqs.erase(it);
    }
    return CF_OK;
}

int cf_server_stats(cf_server* s, cf_serving_stats* out)
{
    if (!s || !out) return fail(CF_E_ARG, "null argument");
    std::lock_guard<std::mutex> l(s->mu);
    auto& q = s->sched;
    out->submitted = q.submitted_;
    out->completed = q.completed_;
    out->failed = q.failed_;
    out->rejected = q.rejected_;
    out->cancelled = q.cancelled_;
    out->timedOut = q.timedOut_;
    out->p50Ms = 1000.0 * q.percentile(q.latencies_, 0.50);
    out->p99Ms = 1000.0 * q.percentile(q.latencies_, 0.99);
    double m = 0;
    for (double x : q.latencies_) m += x;
    out->meanMs = q.latencies_.empty() ? 0.0 : 1000.0 * m / q.latencies_.size();
    out->pathStepsDone = uint64_t(q.workDone_);
    out->maxInFlight = q.maxInFlight_;
    out->peakFootprint = q.peak_;
    out->maxStartMs = 1000.0 * s->ex.maxStart;
    out->maxStepMs = 1000.0 * s->maxStep;
    out->bufferGrowths = DevBuf::growths.load() - s->growths0;
    return CF_OK;
}

int cf_server_reset_stats(cf_server* s)
{
    if (!s) return fail(CF_E_ARG, "null server");
    std::lock_guard<std::mutex> l(s->mu);
    s->sched.resetStats();
    s->ex.maxStart = 0;
    s->maxStep = 0;
    s->growths0 = DevBuf::growths.load();
    return CF_OK;
}

int cf_server_inject_failures(cf_server* s, int startFailures)
{
    if (!s) return fail(CF_E_ARG, "null server");
    std::lock_guard<std::mutex> l(s->mu);
    s->ex.injectStartFailures = startFailures;
    return CF_OK;
}

}  // extern "C"
