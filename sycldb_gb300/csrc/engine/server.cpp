// Request server: continuous batching of arriving plans over device-resident
// base tables.  No counterpart in the reference, whose application runs one
// plan at a time (app/application.cpp:37-48; executor/ddor_executor.cpp:22-245);
// every result equals what the plain path (sdb_engine_execute) gives for the
// plan alone.
//
// One dispatcher thread owns the device work.  It keeps up to `slots` batches
// in flight, each on its own streams.  Whenever a slot is free and requests
// wait, it takes the longest first-come prefix of the waiting requests that
// fits the free part of the device budget (at most max_batch plans), carves
// the batch's arena, zeroed region and chain-batch tables out of the device
// pool and its result staging out of the pinned pool, records the plans
// against that memory and enqueues them (executor/batch_api.hpp).  Requests
// that arrive while batches run are admitted into the next free slot, so their
// work overlaps on the device with the batches still running.  A finished
// batch (its completion event) hands its results to the caller and returns its
// memory to the pools.  The device budget descends from the reference's
// memory_manager budget (operations/memory_manager.hpp:7-59): admitted plans'
// hash tables and intermediates never exceed it.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <string>
#include <mutex>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "batch_api.hpp"
#include "sycldb_gpu.h"

int sdb_set_error(int status, const char *fmt, ...);

namespace {

using Clock = std::chrono::steady_clock;

// First-fit allocator over [0, size): offsets only, 256-byte granules.
class RegionPool {
public:
    void init(uint64_t size)
    {
        size_ = size;
        free_.clear();
        if (size) free_[0] = size;
        used_ = peak_ = 0;
    }
    static uint64_t round(uint64_t n) { return (std::max<uint64_t>(n, 1) + 255) & ~uint64_t(255); }
    bool alloc(uint64_t n, uint64_t &off)
    {
        n = round(n);
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second < n) continue;
            off = it->first;
            const uint64_t rest = it->second - n;
            free_.erase(it);
            if (rest) free_[off + n] = rest;
            used_ += n;
            peak_ = std::max(peak_, used_);
            return true;
        }
        return false;
    }
    void release(uint64_t off, uint64_t n)
    {
        n = round(n);
        used_ -= n;
        auto it = free_.emplace(off, n).first;
        auto nx = std::next(it);
        if (nx != free_.end() && it->first + it->second == nx->first) {
            it->second += nx->second;
            free_.erase(nx);
        }
        if (it != free_.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) {
                pv->second += it->second;
                free_.erase(it);
            }
        }
    }
    uint64_t largest() const
    {
        uint64_t m = 0;
        for (auto &f : free_) m = std::max(m, f.second);
        return m;
    }
    uint64_t size() const { return size_; }
    uint64_t peak() const { return peak_; }

private:
    std::map<uint64_t, uint64_t> free_;
    uint64_t size_ = 0, used_ = 0, peak_ = 0;
};

struct Request {
    int64_t id;
    std::string plan;
    Clock::time_point arrival;
    bool sized = false;
    sdb::BatchSize size;
    uint64_t dev_need = 0;  // arena + zeroed region + result region, this plan alone
};

struct Done {
    int64_t id;
    int status;
    std::string error;
    sdb_result *res;
    double latency_ms;
};

struct Slot {
    sdb::SlotStreams ss;
    cudaEvent_t done = nullptr;
    bool busy = false;
    sdb_batch *batch = nullptr;
    std::vector<Request> reqs;
    uint64_t dev_off = 0, dev_bytes = 0, pin_off = 0, pin_bytes = 0;
};

}  // namespace

struct sdb_server {
    sdb_engine *eng = nullptr;
    sdb_server_config cfg{};
    char *dev = nullptr;
    char *pinned = nullptr;
    RegionPool dev_pool, pin_pool;
    std::vector<Slot> slots;

    std::mutex mu;
    std::condition_variable cv_in, cv_out;
    std::deque<Request> incoming;
    std::deque<Done> done;
    int64_t next_id = 0;
    bool stop = false;
    std::thread worker;

    // dispatcher-only state
    std::deque<Request> waiting;
    sdb_server_stats st{};
    uint64_t inflight_plans = 0;

    void finish(Request &r, int status, const std::string &err, sdb_result *res)
    {
        const double ms = std::chrono::duration<double, std::milli>(Clock::now() - r.arrival).count();
        std::lock_guard<std::mutex> g(mu);
        done.push_back({r.id, status, err, res, ms});
        if (status == SDB_OK)
            st.completed++;
        else
            st.failed++;
        cv_out.notify_all();
    }

    void complete_slot(Slot &s, cudaError_t e)
    {
        for (size_t p = 0; p < s.reqs.size(); p++) {
            if (e != cudaSuccess) {
                finish(s.reqs[p], SDB_ERR_CUDA, cudaGetErrorString(e), nullptr);
                continue;
            }
            try {
                finish(s.reqs[p], SDB_OK, "", sdb::batch_take_result(s.batch, p));
            } catch (const sdb::Error &x) {
                finish(s.reqs[p], x.status, x.what(), nullptr);
            } catch (const std::exception &x) {
                finish(s.reqs[p], SDB_ERR_INVALID, x.what(), nullptr);
            }
        }
        inflight_plans -= s.reqs.size();
        sdb::batch_destroy(s.batch);
        s.batch = nullptr;
        s.reqs.clear();
        dev_pool.release(s.dev_off, s.dev_bytes);
        pin_pool.release(s.pin_off, s.pin_bytes);
        s.busy = false;
    }

    bool size_request(Request &r)
    {
        const auto t0 = Clock::now();
        struct Tally {  // the pass's host time, however it ends
            Clock::time_point t0;
            sdb_server *s;
            ~Tally()
            {
                const auto us = std::chrono::duration_cast<std::chrono::microseconds>(Clock::now() - t0).count();
                std::lock_guard<std::mutex> g(s->mu);
                s->st.sizing_us += (uint64_t)us;
            }
        } tally{t0, this};
        try {
            r.size = sdb::batch_size(eng, {r.plan});
            r.dev_need = RegionPool::round(r.size.arena) + RegionPool::round(r.size.zero) +
                         RegionPool::round(r.size.staging);
            r.sized = true;
            return true;
        } catch (const sdb::Error &x) {
            finish(r, x.status, x.what(), nullptr);
        } catch (const std::exception &x) {
            finish(r, SDB_ERR_INVALID, x.what(), nullptr);
        }
        return false;
    }

    // Admits the longest fitting prefix of `waiting` into slot s; false if
    // nothing could be admitted now.
    bool admit(Slot &s)
    {
        size_t k = 0;
        uint64_t need = 0;
        const uint64_t room = dev_pool.largest();
        while (k < waiting.size() && k < (size_t)cfg.max_batch && need + waiting[k].dev_need <= room) {
            need += waiting[k].dev_need;
            k++;
        }
        if (k == 0) {
            // the head alone does not fit now; if it never can, fail it
            const uint64_t alone = waiting.front().dev_need + sdb::batch_chain_bytes(waiting.front().size.chains);
            bool any_busy = false;
            for (auto &o : slots) any_busy |= o.busy;
            if (!any_busy && alone > dev_pool.largest()) {
                Request r = std::move(waiting.front());
                waiting.pop_front();
                finish(r, SDB_ERR_NOMEM,
                       "plan needs " + std::to_string(alone) + " device bytes, the server budget has " +
                           std::to_string(dev_pool.size()),
                       nullptr);
                return true;
            }
            return false;
        }
        for (; k > 0; k--) {
            sdb::BatchSize z;
            std::vector<std::string> plans;
            for (size_t i = 0; i < k; i++) {
                const sdb::BatchSize &q = waiting[i].size;
                z.arena += q.arena;
                z.zero += q.zero;
                z.staging += q.staging;
                z.chains.insert(z.chains.end(), q.chains.begin(), q.chains.end());
                plans.push_back(waiting[i].plan);
            }
            const uint64_t cb = sdb::batch_chain_bytes(z.chains);
            const uint64_t dev_bytes = RegionPool::round(z.arena) + RegionPool::round(z.zero) +
                                       RegionPool::round(z.staging) + RegionPool::round(cb);
            const uint64_t pin_bytes = RegionPool::round(cb) + RegionPool::round(z.staging);
            uint64_t doff = 0, poff = 0;
            if (!dev_pool.alloc(dev_bytes, doff)) continue;
            if (!pin_pool.alloc(pin_bytes, poff)) {
                dev_pool.release(doff, dev_bytes);
                continue;
            }
            s.dev_off = doff;
            s.dev_bytes = dev_bytes;
            s.pin_off = poff;
            s.pin_bytes = pin_bytes;
            s.reqs.assign(std::make_move_iterator(waiting.begin()), std::make_move_iterator(waiting.begin() + k));
            waiting.erase(waiting.begin(), waiting.begin() + k);
            const auto t_launch = Clock::now();
            try {
                s.batch = sdb::batch_launch_external(eng, plans, z, dev + doff, dev_bytes, pinned + poff, pin_bytes, s.ss);
                {
                    const auto us =
                        std::chrono::duration_cast<std::chrono::microseconds>(Clock::now() - t_launch).count();
                    std::lock_guard<std::mutex> g(mu);
                    st.launch_us += (uint64_t)us;
                    st.paired_chains += (uint64_t)sdb::batch_paired_chains(s.batch);
                }
                cudaError_t e = cudaEventRecord(s.done, s.ss.main);
                if (e != cudaSuccess) throw sdb::Error(SDB_ERR_CUDA, cudaGetErrorString(e));
            } catch (const std::exception &x) {
                // whatever was enqueued must finish before the memory is reused
                cudaStreamSynchronize(s.ss.main);
                for (auto &ss : s.ss.side) cudaStreamSynchronize(ss);
                const int status = dynamic_cast<const sdb::Error *>(&x) ? static_cast<const sdb::Error &>(x).status
                                                                       : SDB_ERR_INVALID;
                for (auto &r : s.reqs) finish(r, status, x.what(), nullptr);
                if (s.batch) sdb::batch_destroy(s.batch);
                s.batch = nullptr;
                s.reqs.clear();
                dev_pool.release(doff, dev_bytes);
                pin_pool.release(poff, pin_bytes);
                return true;
            }
            s.busy = true;
            inflight_plans += k;
            std::lock_guard<std::mutex> g(mu);
            st.batches++;
            st.batched_plans += k;
            st.max_batch_plans = std::max<uint64_t>(st.max_batch_plans, k);
            st.max_inflight_plans = std::max(st.max_inflight_plans, inflight_plans);
            st.peak_device_bytes = dev_pool.peak();
            st.peak_pinned_bytes = pin_pool.peak();
            return true;
        }
        bool any_busy = false;
        for (auto &o : slots) any_busy |= o.busy;
        if (!any_busy) {  // not even the head fits an idle server (chain tables or staging)
            Request r = std::move(waiting.front());
            waiting.pop_front();
            finish(r, SDB_ERR_NOMEM, "plan does not fit the server's device budget or pinned staging", nullptr);
            return true;
        }
        return false;
    }

    // Longest queue an idle server still serves one request at a time.
    static constexpr size_t kDirectQueue = 4;

    void run()
    {
        cudaSetDevice(device);
        const bool direct = !cfg.no_direct && cfg.budget_bytes >= sdb::engine_memory_bytes(eng);
        for (;;) {
            bool progress = false;
            int busy = 0;
            for (auto &s : slots) {
                if (!s.busy) continue;
                cudaError_t q = cudaEventQuery(s.done);
                if (q == cudaSuccess) {
                    complete_slot(s, cudaSuccess);
                    progress = true;
                } else if (q != cudaErrorNotReady) {
                    cudaGetLastError();
                    complete_slot(s, q);
                    progress = true;
                } else {
                    busy++;
                }
            }
            {
                std::lock_guard<std::mutex> g(mu);
                while (!incoming.empty()) {
                    waiting.push_back(std::move(incoming.front()));
                    incoming.pop_front();
                }
            }
            // An idle server with a short queue (at most kDirectQueue
            // waiting) runs the oldest request at once through the plain
            // path: no sizing pass, no batch set-up, first come first served.
            // While the device keeps up with the arrivals a request then
            // waits no longer than on the plain path, and none waits for a
            // batch that fills up behind it; once the queue grows past that
            // (the device falls behind), the waiting requests go into
            // batches, whose shared builds and scans raise throughput.
            // (Only when the budget covers the engine's own memory, which a
            // plain execution uses: no plan then goes past the budget.)
            if (direct && busy == 0 && !waiting.empty() && waiting.size() <= kDirectQueue) {
                Request r = std::move(waiting.front());
                waiting.pop_front();
                try {
                    sdb_result *res = sdb::execute_plain(eng, r.plan);
                    finish(r, SDB_OK, "", res);
                } catch (const sdb::Error &x) {
                    finish(r, x.status, x.what(), nullptr);
                } catch (const std::exception &x) {
                    finish(r, SDB_ERR_INVALID, x.what(), nullptr);
                }
                std::lock_guard<std::mutex> g(mu);
                st.direct_plans++;
                continue;
            }
            for (size_t i = 0; i < waiting.size();) {
                if (waiting[i].sized || size_request(waiting[i])) {
                    i++;
                } else {
                    waiting.erase(waiting.begin() + i);
                    progress = true;
                }
            }
            for (auto &s : slots) {
                if (waiting.empty()) break;
                if (s.busy) continue;
                if (admit(s)) {
                    progress = true;
                    if (s.busy) busy++;
                } else {
                    break;
                }
            }
            if (progress) continue;
            std::unique_lock<std::mutex> lk(mu);
            if (stop && incoming.empty() && waiting.empty() && busy == 0) return;
            if (busy)
                cv_in.wait_for(lk, std::chrono::microseconds(20));
            else
                cv_in.wait_for(lk, std::chrono::milliseconds(5), [&] { return stop || !incoming.empty(); });
        }
    }

    int device = 0;
};

namespace {

int submit_at(sdb_server *s, const char *plan, Clock::time_point arrival, int64_t *id)
{
    std::lock_guard<std::mutex> g(s->mu);
    if (s->stop) return sdb_set_error(SDB_ERR_INVALID, "sdb_server_submit: server is stopping");
    Request r;
    r.id = s->next_id++;
    r.plan = plan;
    r.arrival = arrival;
    *id = r.id;
    s->incoming.push_back(std::move(r));
    s->st.submitted++;
    s->cv_in.notify_one();
    return SDB_OK;
}

}  // namespace

extern "C" {

int sdb_server_create(sdb_engine *eng, const sdb_server_config *cfg, sdb_server **out)
{
    if (!eng || !out) return sdb_set_error(SDB_ERR_INVALID, "sdb_server_create: NULL argument");
    *out = nullptr;
    auto S = std::make_unique<sdb_server>();
    S->eng = eng;
    if (cfg) S->cfg = *cfg;
    if (!S->cfg.budget_bytes) S->cfg.budget_bytes = 60ull << 30;
    if (!S->cfg.pinned_bytes) S->cfg.pinned_bytes = 1ull << 30;
    if (S->cfg.slots <= 0) S->cfg.slots = 4;
    if (S->cfg.max_batch <= 0) S->cfg.max_batch = 64;
    if (S->cfg.streams_per_slot <= 0) S->cfg.streams_per_slot = 4;
    cudaGetDevice(&S->device);
    cudaError_t e = cudaMalloc(&S->dev, S->cfg.budget_bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return sdb_set_error(SDB_ERR_NOMEM, "sdb_server_create: device budget of %llu bytes: %s",
                             (unsigned long long)S->cfg.budget_bytes, cudaGetErrorString(e));
    }
    e = cudaHostAlloc(reinterpret_cast<void **>(&S->pinned), S->cfg.pinned_bytes, cudaHostAllocDefault);
    if (e != cudaSuccess) {
        cudaFree(S->dev);
        return sdb_set_error(SDB_ERR_NOMEM, "sdb_server_create: pinned staging: %s", cudaGetErrorString(e));
    }
    S->dev_pool.init(S->cfg.budget_bytes);
    S->pin_pool.init(S->cfg.pinned_bytes);
    S->slots.resize(S->cfg.slots);
    for (auto &sl : S->slots) {
        bool ok = cudaStreamCreateWithFlags(&sl.ss.main, cudaStreamNonBlocking) == cudaSuccess &&
                  cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming) == cudaSuccess &&
                  cudaEventCreateWithFlags(&sl.ss.fork, cudaEventDisableTiming) == cudaSuccess;
        for (int i = 0; ok && i < S->cfg.streams_per_slot; i++) {
            cudaStream_t st;
            cudaEvent_t ev;
            ok = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) == cudaSuccess &&
                 cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) == cudaSuccess;
            if (ok) {
                sl.ss.side.push_back(st);
                sl.ss.join.push_back(ev);
            }
        }
        if (!ok) {
            sdb_server_destroy(S.release());
            return sdb_set_error(SDB_ERR_CUDA, "sdb_server_create: stream setup failed");
        }
    }
    sdb_server *raw = S.get();
    raw->worker = std::thread([raw] { raw->run(); });
    *out = S.release();
    return SDB_OK;
}

int sdb_server_submit(sdb_server *s, const char *plan_json, int64_t *id)
{
    if (!s || !plan_json || !id) return sdb_set_error(SDB_ERR_INVALID, "sdb_server_submit: NULL argument");
    return submit_at(s, plan_json, Clock::now(), id);
}

int sdb_server_next(sdb_server *s, int timeout_ms, int64_t *id, int *status, sdb_result **res, double *latency_ms)
{
    if (!s || !id || !status || !res) return sdb_set_error(SDB_ERR_INVALID, "sdb_server_next: NULL argument");
    std::unique_lock<std::mutex> lk(s->mu);
    auto ready = [&] { return !s->done.empty(); };
    if (timeout_ms < 0)
        s->cv_out.wait(lk, ready);
    else if (!s->cv_out.wait_for(lk, std::chrono::milliseconds(timeout_ms), ready))
        return sdb_set_error(SDB_ERR_TIMEOUT, "sdb_server_next: nothing finished within %d ms", timeout_ms);
    Done d = std::move(s->done.front());
    s->done.pop_front();
    lk.unlock();
    *id = d.id;
    *status = d.status;
    *res = d.res;
    if (latency_ms) *latency_ms = d.latency_ms;
    if (d.status != SDB_OK) sdb_set_error(d.status, "%s", d.error.c_str());
    return SDB_OK;
}

int sdb_server_stats_get(sdb_server *s, sdb_server_stats *out)
{
    if (!s || !out) return sdb_set_error(SDB_ERR_INVALID, "sdb_server_stats_get: NULL argument");
    std::lock_guard<std::mutex> g(s->mu);
    *out = s->st;
    out->budget_bytes = s->cfg.budget_bytes;
    return SDB_OK;
}

int sdb_server_destroy(sdb_server *s)
{
    if (!s) return SDB_OK;
    {
        std::lock_guard<std::mutex> g(s->mu);
        s->stop = true;
        s->cv_in.notify_all();
    }
    if (s->worker.joinable()) s->worker.join();
    for (auto &d : s->done)
        if (d.res) sdb_result_free(d.res);
    for (auto &sl : s->slots) {
        if (sl.ss.main) cudaStreamDestroy(sl.ss.main);
        for (auto st : sl.ss.side) cudaStreamDestroy(st);
        for (auto ev : sl.ss.join) cudaEventDestroy(ev);
        if (sl.ss.fork) cudaEventDestroy(sl.ss.fork);
        if (sl.done) cudaEventDestroy(sl.done);
    }
    if (s->dev) cudaFree(s->dev);
    if (s->pinned) cudaFreeHost(s->pinned);
    delete s;
    return SDB_OK;
}

int sdb_server_replay(sdb_server *s, const char *const *plans, const double *arrival_s, int n, int *status,
                      sdb_result **results, double *latency_ms, double *wall_s)
{
    if (!s || (n > 0 && (!plans || !arrival_s || !status || !latency_ms)) || n < 0)
        return sdb_set_error(SDB_ERR_INVALID, "sdb_server_replay: bad argument");
    // nothing else submits during a replay, so request i gets id base + i
    int64_t base;
    {
        std::lock_guard<std::mutex> g(s->mu);
        base = s->next_id;
    }
    std::atomic<int> submit_status{SDB_OK};
    const Clock::time_point t0 = Clock::now();
    std::thread feeder([&] {
        for (int i = 0; i < n; i++) {
            const auto at = t0 + std::chrono::duration_cast<Clock::duration>(std::chrono::duration<double>(arrival_s[i]));
            std::this_thread::sleep_until(at);
            int64_t id;
            int st = submit_at(s, plans[i], at, &id);
            if (st == SDB_OK && id != base + i) st = sdb_set_error(SDB_ERR_INVALID, "sdb_server_replay: concurrent submissions");
            if (st != SDB_OK) {
                submit_status = st;
                return;
            }
        }
    });
    int got = 0;
    int rc = SDB_OK;
    Clock::time_point last = t0;
    while (got < n) {
        int64_t id = -1;
        int stt = 0;
        sdb_result *r = nullptr;
        double ms = 0;
        if (sdb_server_next(s, 50, &id, &stt, &r, &ms) != SDB_OK) {
            if (submit_status != SDB_OK) {
                rc = submit_status;
                break;
            }
            continue;
        }
        const int64_t i = id - base;
        if (i < 0 || i >= n) {
            if (r) sdb_result_free(r);
            continue;
        }
        status[i] = stt;
        latency_ms[i] = ms;
        if (results)
            results[i] = r;
        else if (r)
            sdb_result_free(r);
        last = Clock::now();
        got++;
    }
    feeder.join();
    if (wall_s) *wall_s = std::chrono::duration<double>(last - t0).count();
    return rc;
}

int sdb_engine_replay_plain(sdb_engine *eng, const char *const *plans, const double *arrival_s, int n, int *status,
                            sdb_result **results, double *latency_ms, double *wall_s)
{
    if (!eng || (n > 0 && (!plans || !arrival_s || !status || !latency_ms)) || n < 0)
        return sdb_set_error(SDB_ERR_INVALID, "sdb_engine_replay_plain: bad argument");
    const Clock::time_point t0 = Clock::now();
    for (int i = 0; i < n; i++) {
        const auto at = t0 + std::chrono::duration_cast<Clock::duration>(std::chrono::duration<double>(arrival_s[i]));
        std::this_thread::sleep_until(at);
        sdb_result *r = nullptr;
        int st = SDB_OK;
        try {
            r = sdb::execute_plain(eng, plans[i]);
        } catch (const sdb::Error &x) {
            st = sdb_set_error(x.status, "%s", x.what());
        } catch (const std::exception &x) {
            st = sdb_set_error(SDB_ERR_INVALID, "%s", x.what());
        }
        status[i] = st;
        latency_ms[i] = std::chrono::duration<double, std::milli>(Clock::now() - at).count();
        if (results)
            results[i] = r;
        else if (r)
            sdb_result_free(r);
    }
    if (wall_s) *wall_s = std::chrono::duration<double>(Clock::now() - t0).count();
    return SDB_OK;
}

}  // extern "C"
