// Host-side tests of the serving scheduler (serving_core.h) with a fake executor: admission
// under the memory budget, arrival order, rejection, cancellation, queue time-outs, injected
// start / finish failures, and submitters on several threads.  Prints one line per check:
// "ok <name>" or "FAIL <name> <detail>"; exit status 0 when all pass.
#include <cstdio>
#include <mutex>
#include <random>
#include <set>
#include <thread>
#include <vector>

#include "../../compfinance_gb300/csrc/serving_core.h"

using namespace cf::serve;

struct FakeExec
{
    double now = 0;
    std::vector<double> doneAt = std::vector<double>(64, -1);
    std::map<uint64_t, double> duration;
    int failStarts = 0, failFinishes = 0;
    std::vector<uint64_t> startOrder;
    std::string err;
    int start(Job& j, int s)
    {
        if (failStarts > 0)
        {
            --failStarts;
            err = "injected allocation failure";
            return -5;
        }
        startOrder.push_back(j.id);
        doneAt[s] = now + (duration.count(j.id) ? duration[j.id] : 1.0);
        return 0;
    }
    bool poll(int s) { return doneAt[s] >= 0 && now >= doneAt[s]; }
    int finish(Job&, int s)
    {
        doneAt[s] = -1;
        if (failFinishes > 0)
        {
            --failFinishes;
            err = "injected result failure";
            return -4;
        }
        return 0;
    }
    std::string error() const { return err; }
};

static int failures = 0;
static void check(bool c, const char* name, const std::string& detail = "")
{
    std::printf("%s %s %s\n", c ? "ok" : "FAIL", name, detail.c_str());
    if (!c) ++failures;
}

int main()
{
    {  // budget-limited admission in arrival order, slots reused
        FakeExec ex;
        Scheduler<FakeExec> s(ex, 4, 100);
        std::vector<uint64_t> ids;
        for (int i = 0; i < 10; ++i) ids.push_back(s.submit(40, 0, 0));
        s.step(0);
        check(ex.startOrder.size() == 2, "budget_admits_two", std::to_string(ex.startOrder.size()));
        check(s.inUse_ <= 100, "budget_respected");
        for (double t = 1; t <= 10; t += 1)
        {
            ex.now = t;
            s.step(t);
        }
        check(s.completed_ == 10, "all_complete", std::to_string(s.completed_));
        check(ex.startOrder == ids, "arrival_order");
        check(s.peak_ <= 100 && s.maxInFlight_ == 2, "peak_footprint");
    }
    {  // statistics reset between streams: counters restart, the memory in use stays accounted
        FakeExec ex;
        Scheduler<FakeExec> s(ex, 2, 100);
        for (int i = 0; i < 3; ++i) s.submit(40, 0, 0);
        s.step(0);
        ex.now = 1;
        s.step(1);  // two finish, the third starts
        s.resetStats();
        check(s.completed_ == 0 && s.latencies_.empty() && s.workDone_ == 0, "reset_clears_counters");
        check(s.peak_ == s.inUse_ && s.inUse_ == 40, "reset_keeps_in_use", std::to_string(s.inUse_));
        ex.now = 2;
        s.step(2);
        check(s.completed_ == 1 && s.latencies_.size() == 1 && s.inUse_ == 0, "reset_then_complete");
    }
    {  // lanes: a short request starts on a short slot while long ones wait for the long slots;
       // arrival order holds within each lane; a lane with no slot rejects
        FakeExec ex;
        Scheduler<FakeExec> s(ex, 3, 1000);
        s.setLanes({0, 0, 1});  // two short slots, one long slot
        const uint64_t l1 = s.submit(10, 0, 0, 100, 1), l2 = s.submit(10, 0, 0, 100, 1);
        const uint64_t s1 = s.submit(1, 0, 0, 1, 0), s2 = s.submit(1, 0, 0, 1, 0), s3 = s.submit(1, 0, 0, 1, 0);
        ex.duration[l1] = 5.0;
        s.step(0);
        check(s.get(l1)->status == RUNNING && s.get(l2)->status == QUEUED, "lane_long_one_slot");
        check(s.get(s1)->status == RUNNING && s.get(s2)->status == RUNNING && s.get(s3)->status == QUEUED,
              "lane_short_bypasses_long");
        check(s.slotLane(s.get(l1)->slot) == 1 && s.slotLane(s.get(s1)->slot) == 0, "lane_slots");
        ex.now = 1;
        s.step(1);
        check(s.get(s3)->status == RUNNING && s.get(l2)->status == QUEUED, "lane_order_within");
        for (double t = 2; t <= 12; t += 1)
        {
            ex.now = t;
            s.step(t);
        }
        check(s.completed_ == 5 && s.get(l2)->tStart >= 5.0, "lane_long_fifo");
        const uint64_t bad = s.submit(1, 0, 12, 1, 2);
        check(s.get(bad)->status == REJECTED && !s.get(bad)->error.empty(), "lane_without_slot_rejected");
    }
    {  // least-work-first lane: the smallest queued long request starts first; one that has waited
       // past the aging time goes ahead of smaller ones
        FakeExec ex;
        Scheduler<FakeExec> s(ex, 2, 1000);
        s.setLanes({0, 1});
        s.setLaneOrder(1, 1, 2.5);
        const uint64_t first = s.submit(1, 0, 0, 50, 1);
        const uint64_t big = s.submit(1, 0, 0, 400, 1), small = s.submit(1, 0, 0, 100, 1);
        s.step(0);
        check(s.get(first)->status == RUNNING && s.get(big)->status == QUEUED, "sjf_first_runs");
        ex.now = 1;
        s.step(1);
        check(s.get(small)->status == RUNNING && s.get(big)->status == QUEUED, "sjf_least_work_next");
        const uint64_t mid = s.submit(1, 0, 1, 200, 1);
        ex.now = 3;  // big has waited 3 > 2.5 (aged), mid 2: big goes ahead of the smaller mid
        s.step(3);
        check(s.get(big)->status == RUNNING && s.get(mid)->status == QUEUED, "sjf_aged_first");
        const uint64_t tiny = s.submit(1, 0, 3, 10, 1);
        s.step(3);
        check(s.get(tiny)->status == QUEUED, "sjf_slot_busy");
        s.setLaneOrder(1, 0, 0.0);  // back to arrival order: mid (older) before tiny
        ex.now = 20;
        s.step(20);
        check(s.get(mid)->status == RUNNING && s.get(tiny)->status == QUEUED, "order_back_to_fifo");
    }
    {  // slot-limited admission; small requests overlap
        FakeExec ex;
        Scheduler<FakeExec> s(ex, 3, 1000);
        for (int i = 0; i < 7; ++i) s.submit(1, 0, 0);
        s.step(0);
        check(s.maxInFlight_ == 3, "slots_limit");
    }
    {  // rejection of a request larger than the whole budget; the queue keeps flowing
        FakeExec ex;
        Scheduler<FakeExec> s(ex, 2, 100);
        const uint64_t big = s.submit(101, 0, 0);
        const uint64_t ok = s.submit(10, 0, 0);
        s.step(0);
        check(s.get(big)->status == REJECTED && !s.get(big)->error.empty(), "reject_oversize");
        check(s.get(ok)->status == RUNNING, "after_reject_runs");
    }
    {  // cancellation of queued requests only
        FakeExec ex;
        Scheduler<FakeExec> s(ex, 1, 100);
        const uint64_t a = s.submit(10, 0, 0), b = s.submit(10, 0, 0), c = s.submit(10, 0, 0);
        s.step(0);
        check(!s.cancel(a, 0), "cannot_cancel_running");
        check(s.cancel(b, 0) && s.get(b)->status == CANCELLED, "cancel_queued");
        ex.now = 1;
        s.step(1);
        check(s.get(c)->status == RUNNING, "next_after_cancel");
    }
    {  // queue time-out
        FakeExec ex;
        Scheduler<FakeExec> s(ex, 1, 100);
        ex.duration[1] = 5.0;
        s.submit(10, 0, 0);
        const uint64_t b = s.submit(10, 2.0, 0);
        s.step(0);
        ex.now = 3;
        s.step(3);
        check(s.get(b)->status == TIMEOUT, "queue_timeout");
    }
    {  // injected start and finish failures release slots and memory
        FakeExec ex;
        ex.failStarts = 2;
        ex.failFinishes = 1;
        Scheduler<FakeExec> s(ex, 2, 100);
        for (int i = 0; i < 6; ++i) s.submit(30, 0, 0);
        for (double t = 0; t < 10; t += 1)
        {
            ex.now = t;
            s.step(t);
        }
        check(s.failed_ == 3 && s.completed_ == 3, "injected_failures",
              std::to_string(s.failed_) + " " + std::to_string(s.completed_));
        check(s.inUse_ == 0 && s.idle(), "released_after_failures");
        check(s.get(1)->error == "injected allocation failure", "failure_message");
    }
    {  // random stream, several submitter threads, a scheduler thread
        FakeExec ex;
        Scheduler<FakeExec> s(ex, 8, 1000);
        std::mutex mu;
        std::set<uint64_t> all;
        bool stop = false;
        std::thread sched([&] {
            double t = 0;
            while (true)
            {
                std::lock_guard<std::mutex> l(mu);
                ex.now = t;
                s.step(t);
                t += 0.25;
                if (stop && s.idle()) break;
            }
        });
        std::vector<std::thread> subs;
        for (int k = 0; k < 4; ++k)
            subs.emplace_back([&, k] {
                std::mt19937 rng(k);
                for (int i = 0; i < 500; ++i)
                {
                    std::lock_guard<std::mutex> l(mu);
                    const uint64_t id = s.submit(1 + rng() % 300, 0, ex.now);
                    ex.duration[id] = 0.25 * (1 + rng() % 8);
                    all.insert(id);
                }
            });
        for (auto& t : subs) t.join();
        {
            std::lock_guard<std::mutex> l(mu);
            stop = true;
        }
        sched.join();
        check(all.size() == 2000 && s.completed_ == 2000, "threaded_all_complete", std::to_string(s.completed_));
        check(s.peak_ <= 1000 && s.maxInFlight_ <= 8, "threaded_limits");
        const double p50 = Scheduler<FakeExec>::percentile(s.latencies_, 0.5),
                     p99 = Scheduler<FakeExec>::percentile(s.latencies_, 0.99);
        check(p50 > 0 && p99 >= p50, "percentiles");
    }
    return failures ? 1 : 0;
}
