// Slot scheduler of the serving loop (continuous batching).
//
// Requests are admitted in arrival order into a fixed set of execution slots, each with its
// own CUDA stream, under a device-memory budget: a request starts as soon as a slot is free
// and its footprint fits the memory left, so work that arrives while other requests are on
// the GPU overlaps with them.  Slots and requests may be split into lanes (short and long
// requests, say): a request takes only slots of its own lane, and arrival order holds within
// each lane, so a request never waits behind one of another lane; a lane may instead admit its
// least work first (a request that has waited longer than the lane's aging time goes ahead of
// those, oldest first), so that small requests do not queue behind large ones.  Finished slots are reaped
// by polling; queued requests can be cancelled or expire after their queue timeout; a request
// whose footprint exceeds the whole budget, or whose lane has no slot, is rejected at
// submission.  The executor does the work; it is a template parameter
// so that the admission logic is tested on the CPU with a fake executor.
//
// Executor interface:
//   int  start(Job& job, int slot)    0, or an error code (the job fails, the slot is freed)
//   bool poll(int slot)               true once the slot's work has completed
//   int  finish(Job& job, int slot)   0, or an error code (the job fails)
//   std::string error()               message of the last failure
#pragma once

#include <algorithm>
#include <cstdint>
#include <deque>
#include <map>
#include <string>
#include <tuple>
#include <vector>

namespace cf {
namespace serve {

enum Status : int { QUEUED = 0, RUNNING = 1, DONE = 2, FAILED = 3, REJECTED = 4, CANCELLED = 5, TIMEOUT = 6 };

struct Job
{
    uint64_t id = 0;
    int status = QUEUED;
    int slot = -1;
    size_t footprint = 0;
    double tSubmit = 0, tStart = 0, tDone = 0;
    double queueTimeout = 0;  // seconds a request may wait for a slot (0 = no limit)
    std::string error;
    long long work = 0;       // path-steps, for throughput accounting
    int lane = 0;             // the slots it may take: those of its lane
};

template <class Exec>
class Scheduler
{
public:
    Scheduler(Exec& ex, int nSlots, size_t budget) : ex_(ex), slots_(nSlots, 0), lane_(nSlots, 0), budget_(budget) {}

    // Lane of every slot (one entry per slot; lanes 0..nLanes-1).  Set before the first request.
    void setLanes(const std::vector<int>& slotLane)
    {
        if (slotLane.size() == slots_.size()) lane_ = slotLane;
    }
    int slotLane(int s) const { return lane_[s]; }

    // Admission order of a lane: 0 arrival order (the default), 1 least work first, except that
    // requests older than agingSec go first, in arrival order.
    void setLaneOrder(int lane, int order, double agingSec)
    {
        if (lane < 0) return;
        if (lane >= int(order_.size()))
        {
            order_.resize(lane + 1, 0);
            aging_.resize(lane + 1, 0.0);
        }
        order_[lane] = order;
        aging_[lane] = agingSec;
    }
    int laneOrder(int lane) const { return lane < int(order_.size()) ? order_[lane] : 0; }

    // Registers a request; a request larger than the whole budget is rejected at once.
    uint64_t submit(size_t footprint, double queueTimeout, double now, long long work = 0, int lane = 0)
    {
        Job j;
        j.id = ++nextId_;
        j.footprint = footprint;
        j.tSubmit = now;
        j.queueTimeout = queueTimeout;
        j.work = work;
        j.lane = lane;
        if (footprint > budget_ || std::find(lane_.begin(), lane_.end(), lane) == lane_.end())
        {
            j.status = REJECTED;
            j.error = footprint > budget_ ? "request footprint " + std::to_string(footprint) +
                                                " B exceeds the device budget " + std::to_string(budget_) + " B"
                                          : "no slot serves lane " + std::to_string(lane);
            j.tDone = now;
            ++rejected_;
        }
        else
            queue_.push_back(j.id);
        jobs_[j.id] = j;
        ++submitted_;
        return j.id;
    }

    // Cancels a request that has not started yet.
    bool cancel(uint64_t id, double now)
    {
        auto it = jobs_.find(id);
        if (it == jobs_.end() || it->second.status != QUEUED) return false;
        it->second.status = CANCELLED;
        it->second.tDone = now;
        queue_.erase(std::remove(queue_.begin(), queue_.end(), id), queue_.end());
        ++cancelled_;
        return true;
    }

    // One scheduling round: reap finished slots, expire queue time-outs, then admit, lane by
    // lane in each lane's order, while a slot of the lane is free and the lane's next request fits
    // the memory left.  Returns the number of state changes (0 = nothing happened).
    int step(double now)
    {
        int changes = 0;
        for (int s = 0; s < int(slots_.size()); ++s)
        {
            const uint64_t id = slots_[s];
            if (!id || !ex_.poll(s)) continue;
            Job& j = jobs_[id];
            const int rc = ex_.finish(j, s);
            j.tDone = now;
            if (rc)
            {
                j.status = FAILED;
                j.error = ex_.error();
                ++failed_;
            }
            else
            {
                j.status = DONE;
                ++completed_;
                latencies_.push_back(j.tDone - j.tSubmit);
                workDone_ += j.work;
                busy_ += j.tDone - j.tStart;
            }
            inUse_ -= j.footprint;
            slots_[s] = 0;
            ++changes;
        }
        for (auto it = queue_.begin(); it != queue_.end();)
        {
            Job& j = jobs_[*it];
            if (j.queueTimeout > 0 && now - j.tSubmit > j.queueTimeout)
            {
                j.status = TIMEOUT;
                j.tDone = now;
                j.error = "queue time-out";
                ++timedOut_;
                it = queue_.erase(it);
                ++changes;
            }
            else
                ++it;
        }
        // arrival-order lanes, in one pass over the queue
        std::vector<char> blocked;  // lanes whose next request waits
        for (auto it = queue_.begin(); it != queue_.end();)
        {
            Job& j = jobs_[*it];
            if (j.lane >= int(blocked.size())) blocked.resize(j.lane + 1, 0);
            if (blocked[j.lane] || laneOrder(j.lane) != 0)
            {
                ++it;
                continue;
            }
            if (!admit(j, now, changes))  // head of its lane waits
            {
                blocked[j.lane] = 1;
                ++it;
                continue;
            }
            it = queue_.erase(it);
        }
        // least-work lanes: aged requests (oldest first), then the least work (then the oldest)
        for (int lane = 0; lane < int(order_.size()); ++lane)
        {
            if (order_[lane] == 0) continue;
            std::vector<uint64_t> cand;
            for (uint64_t id : queue_)
                if (jobs_[id].lane == lane) cand.push_back(id);
            if (cand.empty()) continue;
            auto key = [&](uint64_t id) {
                const Job& j = jobs_[id];
                const bool aged = aging_[lane] > 0 && now - j.tSubmit > aging_[lane];
                return std::make_tuple(aged ? 0 : 1, aged ? 0LL : j.work, j.id);  // ids grow with arrival
            };
            std::stable_sort(cand.begin(), cand.end(), [&](uint64_t a, uint64_t b) { return key(a) < key(b); });
            for (uint64_t id : cand)
            {
                if (!admit(jobs_[id], now, changes)) break;  // the lane's first choice waits
                queue_.erase(std::find(queue_.begin(), queue_.end(), id));
            }
        }
        return changes;
    }

    bool idle() const
    {
        if (!queue_.empty()) return false;
        for (uint64_t x : slots_)
            if (x) return false;
        return true;
    }

    const Job* get(uint64_t id) const
    {
        auto it = jobs_.find(id);
        return it == jobs_.end() ? nullptr : &it->second;
    }
    void forget(uint64_t id) { jobs_.erase(id); }

    static double percentile(std::vector<double> v, double q)
    {
        if (v.empty()) return 0.0;
        std::sort(v.begin(), v.end());
        const double pos = q * (v.size() - 1);
        const size_t i = size_t(pos);
        const double f = pos - i;
        return i + 1 < v.size() ? v[i] * (1 - f) + v[i + 1] * f : v[i];
    }

    // Clears the counters and latencies (not the queue, nor the memory in use); peak restarts
    // from what is in use now.
    void resetStats()
    {
        submitted_ = completed_ = failed_ = rejected_ = cancelled_ = timedOut_ = 0;
        peak_ = inUse_;
        maxInFlight_ = 0;
        busy_ = 0;
        workDone_ = 0;
        latencies_.clear();
    }

    uint64_t submitted_ = 0, completed_ = 0, failed_ = 0, rejected_ = 0, cancelled_ = 0, timedOut_ = 0;
    size_t inUse_ = 0, peak_ = 0;
    int maxInFlight_ = 0;
    double busy_ = 0;
    long long workDone_ = 0;
    std::vector<double> latencies_;

private:
    // Starts j on a free slot of its lane if one is free and its footprint fits; false if it
    // must wait.  A start that fails ends the job (FAILED) and counts as admitted.
    bool admit(Job& j, double now, int& changes)
    {
        int s = 0;
        while (s < int(slots_.size()) && (slots_[s] || lane_[s] != j.lane)) ++s;
        if (s == int(slots_.size()) || inUse_ + j.footprint > budget_) return false;
        j.tStart = now;
        const int rc = ex_.start(j, s);
        if (rc)
        {
            j.status = FAILED;
            j.error = ex_.error();
            j.tDone = now;
            ++failed_;
        }
        else
        {
            j.status = RUNNING;
            j.slot = s;
            slots_[s] = j.id;
            inUse_ += j.footprint;
            peak_ = std::max(peak_, inUse_);
            int running = 0;
            for (uint64_t x : slots_) running += x != 0;
            maxInFlight_ = std::max(maxInFlight_, running);
        }
        ++changes;
        return true;
    }

    Exec& ex_;
    std::vector<uint64_t> slots_;
    std::vector<int> lane_;
    std::vector<int> order_;      // per lane: 0 arrival order, 1 least work first
    std::vector<double> aging_;   // per lane: seconds after which a request goes first
    size_t budget_;
    uint64_t nextId_ = 0;
    std::deque<uint64_t> queue_;
    std::map<uint64_t, Job> jobs_;
};

}  // namespace serve
}  // namespace cf
