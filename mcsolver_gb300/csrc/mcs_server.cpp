// mcs_server.cpp -- continuous-batching request loop (C ABI mcs_server_*).
//
// submit(): compiles the request on the caller's thread (validation,
//           colouring, tables, the arena image) and queues it; nothing touches
//           the device yet.  submit(), poll(), cancel() and stats() may be
//           called from any number of threads while another thread runs
//           step(): they hold the queue lock only to insert or look up, never
//           across device work.
// step():   1. retires cancelled requests;
//           2. admits queued requests in arrival order while a slot is free and
//              the HBM budget holds the request's arena (allocation + upload).
//              A request takes a slot of one persistent batch and joins (or
//              forms) the launch group of its configuration; the other groups
//              are left as they are;
//           3. advances every active request by its own quota of units, sized
//              so that each request's share of a step takes about the same
//              device time on its schedule (a small lattice does many sweeps
//              per step, a large one few), all groups side by side;
//           4. retires requests that reached their last unit: results are kept
//              for poll(), the arena is freed and its bytes return to the budget.
// A request that fails (its upload, its group's launch, its result read-back)
// is retired with its own status and message, which poll() returns; the other
// requests go on.  A request's spin trajectory depends only on its own problem
// and seed, so its result is the same alone and in any mix (tested).
#include <cuda_runtime.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "../../include/mcsgpu.h"
#include "mcs_engine.h"

using namespace mcs;

struct mcs_server {
    int device = 0;
    uint64_t budget = 0;
    int max_slots = 0;
    uint64_t next_ticket = 1;
    double step_us = 2000.0;  // target device time of a request's share of one step
    struct Done {
        int status = MCS_OK;
        std::string msg;
        mcs_result r;
        std::vector<double> groups;
    };
    // guarded by qmu: the queue, finished results, tickets not yet finished,
    // cancellations, counters
    std::mutex qmu;
    std::deque<std::pair<uint64_t, std::unique_ptr<Replica>>> queue;
    std::unordered_map<uint64_t, Done> done;
    std::unordered_set<uint64_t> pending;  // queued or active
    std::unordered_set<uint64_t> cancels;  // active tickets to retire at the next step
    uint64_t in_use = 0;
    long long site_updates = 0;
    int n_active = 0;
    // guarded by smu: the device side (one step at a time)
    std::mutex smu;
    Batch batch;                         // replicas indexed by slot (null = free)
    std::vector<uint64_t> slot_ticket;   // ticket of each slot (0 = free)
    // host-side fault injection for tests (MCSGPU_SERVER_INJECT="upload:k" or
    // "results:k": the k-th upload or result read-back of this server reports
    // failure before touching the device); never set in production
    long long inject_upload = 0, inject_results = 0, n_upload = 0, n_results = 0;
};

static uint64_t request_bytes(const Replica &r) { return r.bytes + sizeof(Rep); }

// Record a finished or failed request (qmu held by the caller).
static void finish_locked(mcs_server *s, uint64_t t, mcs_server::Done &&d)
{
    s->pending.erase(t);
    s->cancels.erase(t);
    s->done[t] = std::move(d);
}

static mcs_server::Done failed_done(int status, const std::string &msg)
{
    mcs_server::Done d;
    // poll's 1 means pending: a failure is never reported with that value
    d.status = (status == MCS_OK || status == 1) ? MCS_EFAILED : status;
    d.msg = msg;
    memset(&d.r, 0, sizeof d.r);
    return d;
}

extern "C" int mcs_server_create(int32_t device, uint64_t hbm_budget_bytes, int32_t max_slots, mcs_server **out)
{
    if (!out || max_slots < 1 || hbm_budget_bytes == 0) { set_error("server needs a budget and >= 1 slot"); return MCS_EINVAL; }
    mcs_server *s = new mcs_server();
    s->device = device;
    s->budget = hbm_budget_bytes;
    s->max_slots = max_slots;
    s->batch.init(device);
    s->batch.no_autotune = 1;  // membership changes often; each group runs its first candidate
    s->batch.slot_capacity = max_slots;
    s->batch.replicas.resize(max_slots);
    s->slot_ticket.assign(max_slots, 0);
    if (const char *e = getenv("MCSGPU_SERVER_STEP_US")) s->step_us = std::max(1.0, atof(e));
    // the engine's kernels are loaded now rather than at the first launch of
    // each, inside some request's step (where no device is present, nothing
    // happens: requests are still compiled and queued on the host)
    {
        int cur = 0;
        if (cudaGetDevice(&cur) == cudaSuccess && cudaSetDevice(device) == cudaSuccess) {
            if (preload_kernels_main() == cudaSuccess) preload_kernels_cluster();
            cudaSetDevice(cur);
        }
        cudaGetLastError();
    }
    if (const char *e = getenv("MCSGPU_SERVER_INJECT")) {
        long long k = 0;
        if (sscanf(e, "upload:%lld", &k) == 1) s->inject_upload = k;
        if (sscanf(e, "results:%lld", &k) == 1) s->inject_results = k;
    }
    *out = s;
    return MCS_OK;
}

extern "C" int mcs_server_submit(mcs_server *s, const mcs_problem *problem, const mcs_options *options, uint64_t *ticket)
{
    if (!s || !problem) { set_error("server and problem are required"); return MCS_EINVAL; }
    mcs_options def;
    memset(&def, 0, sizeof def);
    if (!options) options = &def;
    std::unique_ptr<Replica> r(new Replica());
    r->device = s->device;
    int rc = build_replica(problem, options, r.get(), false);
    if (rc != MCS_OK) return rc;
    if (request_bytes(*r) > s->budget) { set_error("request larger than the server's HBM budget"); return MCS_ENOMEM; }
    std::lock_guard<std::mutex> lock(s->qmu);
    const uint64_t t = s->next_ticket++;
    s->queue.emplace_back(t, std::move(r));
    s->pending.insert(t);
    if (ticket) *ticket = t;
    return MCS_OK;
}

extern "C" int mcs_server_cancel(mcs_server *s, uint64_t ticket)
{
    if (!s) { set_error("server is required"); return MCS_EINVAL; }
    std::lock_guard<std::mutex> lock(s->qmu);
    if (s->done.count(ticket)) return MCS_OK;  // already finished: poll returns its result
    if (!s->pending.count(ticket)) { set_error("unknown ticket"); return MCS_ENOTFOUND; }
    for (auto it = s->queue.begin(); it != s->queue.end(); ++it)
        if (it->first == ticket) {  // never admitted: nothing on the device
            s->queue.erase(it);
            finish_locked(s, ticket, failed_done(MCS_ECANCELLED, "request cancelled"));
            return MCS_OK;
        }
    s->cancels.insert(ticket);  // active: retired at the start of the next step
    return MCS_OK;
}

// Retire the requests of `slots` (results already gathered in `fin`, or a
// failure status): take them out of their groups, free their arenas, return
// their bytes, and record them.  Replicas left without a group are failed too.
static void retire_slots(mcs_server *s, std::vector<int> slots, std::vector<std::pair<int, mcs_server::Done>> &fin)
{
    Batch &b = s->batch;
    std::vector<int> orphans;
    b.drop(slots, &orphans);
    for (int o : orphans)
        if (std::find(slots.begin(), slots.end(), o) == slots.end()) {
            slots.push_back(o);
            fin.emplace_back(o, failed_done(MCS_ECUDA, "kernel group of this request could not be rebuilt: " + get_error()));
        }
    std::vector<std::unique_ptr<Replica>> freed;
    {
        std::lock_guard<std::mutex> lock(s->qmu);
        for (auto &f : fin) {
            const int slot = f.first;
            Replica *r = b.replicas[slot].get();
            if (!r) continue;
            s->in_use -= request_bytes(*r);
            if (f.second.status == MCS_OK) s->site_updates += f.second.r.site_updates;
            finish_locked(s, s->slot_ticket[slot], std::move(f.second));
            s->slot_ticket[slot] = 0;
            freed.push_back(std::move(b.replicas[slot]));
        }
        int n = 0;
        for (auto &r : b.replicas) n += r != nullptr;
        s->n_active = n;
    }
    freed.clear();  // frees the arenas outside the lock (no device work is in flight between steps)
}

extern "C" int mcs_server_step(mcs_server *s, int32_t *completed)
{
    if (!s) { set_error("server is required"); return MCS_EINVAL; }
    std::lock_guard<std::mutex> slock(s->smu);
    if (completed) *completed = 0;
    Batch &b = s->batch;
    // MCSGPU_TRACE=1: host time of the step's phases on stderr
    const bool trace = getenv("MCSGPU_TRACE") != nullptr;
    const auto t0 = std::chrono::steady_clock::now();
    auto ms_since = [&](std::chrono::steady_clock::time_point t) {
        return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t).count();
    };
    // 1. cancelled requests that are on the device
    {
        std::vector<int> cs;
        {
            std::lock_guard<std::mutex> lock(s->qmu);
            for (int k = 0; k < s->max_slots; ++k)
                if (s->slot_ticket[k] && s->cancels.count(s->slot_ticket[k])) cs.push_back(k);
        }
        if (!cs.empty()) {
            std::vector<std::pair<int, mcs_server::Done>> fin;
            for (int k : cs) fin.emplace_back(k, failed_done(MCS_ECANCELLED, "request cancelled"));
            retire_slots(s, cs, fin);
        }
    }
    // 2. admission by slots and HBM budget, in arrival order
    std::vector<std::pair<uint64_t, std::unique_ptr<Replica>>> admit;
    {
        std::lock_guard<std::mutex> lock(s->qmu);
        int free_slots = 0;
        for (int k = 0; k < s->max_slots; ++k) free_slots += s->slot_ticket[k] == 0;
        while (!s->queue.empty() && free_slots > 0) {
            Replica &r = *s->queue.front().second;
            if (s->in_use + request_bytes(r) > s->budget) break;
            s->in_use += request_bytes(r);
            admit.push_back(std::move(s->queue.front()));
            s->queue.pop_front();
            --free_slots;
        }
    }
    if (!admit.empty()) {
        std::vector<int> slots;
        int next = 0;
        for (auto &a : admit) {
            int rc = MCS_OK;
            if (s->inject_upload > 0 && ++s->n_upload == s->inject_upload) {
                rc = MCS_ENOMEM;
                set_error("injected upload failure");
            } else {
                rc = upload_replica(a.second.get());
            }
            if (rc != MCS_OK) {
                // this request fails alone; its bytes go back to the budget
                cudaGetLastError();
                std::lock_guard<std::mutex> lock(s->qmu);
                s->in_use -= request_bytes(*a.second);
                finish_locked(s, a.first, failed_done(rc, get_error()));
                continue;
            }
            while (s->slot_ticket[next]) ++next;
            s->slot_ticket[next] = a.first;
            b.replicas[next] = std::move(a.second);
            slots.push_back(next);
        }
        int rc = b.admit(slots, s->step_us);
        if (rc != MCS_OK) {
            // the admitted requests fail together (their groups may be half
            // built); the running ones keep theirs
            const std::string msg = get_error();
            cudaGetLastError();
            std::vector<std::pair<int, mcs_server::Done>> fin;
            for (int k : slots) fin.emplace_back(k, failed_done(rc, "admission: " + msg));
            retire_slots(s, slots, fin);
        } else {
            std::lock_guard<std::mutex> lock(s->qmu);
            int n = 0;
            for (auto &r : b.replicas) n += r != nullptr;
            s->n_active = n;
        }
    }
    const double t_admit = ms_since(t0);
    if (trace && !admit.empty()) fprintf(stderr, "mcsgpu trace: server admitted %zu in %.3f ms\n", admit.size(), t_admit);
    if (b.groups.empty()) return MCS_OK;
    // 3. every active request by its own quota
    std::vector<int> failed;
    int rc = b.advance_quota(&failed);
    if (rc != MCS_OK) {
        // an error at the synchronisation leaves the context unusable: every
        // active request fails with it and the server reports it
        const std::string msg = get_error();
        std::vector<int> all;
        std::vector<std::pair<int, mcs_server::Done>> fin;
        for (int k = 0; k < s->max_slots; ++k)
            if (b.replicas[k]) { all.push_back(k); fin.emplace_back(k, failed_done(rc, msg)); }
        retire_slots(s, all, fin);
        set_error(msg);
        return rc;
    }
    // 4. retire failed and finished requests
    std::vector<int> out;
    std::vector<std::pair<int, mcs_server::Done>> fin;
    {
        std::vector<char> bad(s->max_slots, 0);
        for (int k : failed) {
            if (bad[k]) continue;
            bad[k] = 1;
            out.push_back(k);
            fin.emplace_back(k, failed_done(MCS_ECUDA, "launch of this request's kernel group failed"));
        }
        std::vector<int> fs;
        for (int k = 0; k < s->max_slots; ++k) {
            Replica *r = b.replicas[k].get();
            if (r && !bad[k] && r->rep.u >= r->hm.units_total) fs.push_back(k);
        }
        if (!fs.empty()) {
            // descriptors (frames written) and result blocks of the finished
            // requests, one synchronisation for all of them
            std::vector<Rep> fr(fs.size());
            for (size_t i = 0; i < fs.size(); ++i)
                if (cudaMemcpyAsync(&fr[i], b.d_reps + fs[i], sizeof(Rep), cudaMemcpyDeviceToHost, b.stream) != cudaSuccess)
                    rc = MCS_ECUDA;
            if (rc == MCS_OK && cudaStreamSynchronize(b.stream) != cudaSuccess) rc = MCS_ECUDA;
            std::vector<Replica *> rs;
            for (int k : fs) rs.push_back(b.replicas[k].get());
            if (rc == MCS_OK) rc = fetch_result_blocks(rs, s->device);
            for (size_t i = 0; i < fs.size(); ++i) {
                const int k = fs[i];
                Replica *r = b.replicas[k].get();
                out.push_back(k);
                if (rc != MCS_OK) {
                    fin.emplace_back(k, failed_done(MCS_ECUDA, "result read-back failed"));
                    continue;
                }
                mcs_server::Done d;
                memset(&d.r, 0, sizeof d.r);
                const int G = r->hm.ngroup;
                d.groups.assign((size_t)(G + 1) * (G + 1) + (G + 1), 0.0);
                d.r.group_values = d.groups.data();
                d.r.group_capacity = (int)d.groups.size();
                int rr = MCS_OK;
                if (s->inject_results > 0 && ++s->n_results == s->inject_results) {
                    rr = MCS_ECUDA;
                    set_error("injected result failure");
                } else {
                    rr = replica_results(r, fr[i], &d.r);
                }
                d.r.group_values = nullptr;
                d.r.frames = nullptr;
                d.r.series = nullptr;
                if (rr != MCS_OK) {
                    fin.emplace_back(k, failed_done(rr, get_error()));
                    continue;
                }
                fin.emplace_back(k, std::move(d));
            }
        }
    }
    if (out.empty()) return MCS_OK;
    int ok = 0;
    for (auto &f : fin) ok += f.second.status == MCS_OK;
    retire_slots(s, out, fin);
    if (completed) *completed = ok;
    if (trace) fprintf(stderr, "mcsgpu trace: server step %.3f ms (admission %.3f), retired %zu\n", ms_since(t0), t_admit,
                       out.size());
    // the remaining requests are placed again for the lighter load (a large
    // lattice left alone moves to a larger cluster)
    std::vector<int> orphans;
    if (b.rebalance(s->step_us, &orphans) != MCS_OK) {
        cudaGetLastError();
        for (int k = 0; k < s->max_slots; ++k)
            if (b.replicas[k]) {
                bool grouped = false;
                for (auto &G : b.groups) grouped |= std::find(G->ids.begin(), G->ids.end(), k) != G->ids.end();
                if (!grouped) orphans.push_back(k);
            }
    }
    if (trace) fprintf(stderr, "mcsgpu trace: server step with rebalance %.3f ms\n", ms_since(t0));
    if (!orphans.empty()) {
        std::vector<std::pair<int, mcs_server::Done>> ofin;
        for (int k : orphans) ofin.emplace_back(k, failed_done(MCS_ECUDA, "re-placing this request failed: " + get_error()));
        retire_slots(s, orphans, ofin);
    }
    return MCS_OK;
}

extern "C" int mcs_server_poll(mcs_server *s, uint64_t ticket, mcs_result *result)
{
    if (!s) { set_error("server is required"); return MCS_EINVAL; }
    std::lock_guard<std::mutex> lock(s->qmu);
    auto it = s->done.find(ticket);
    if (it == s->done.end()) {
        if (s->pending.count(ticket)) return 1;
        set_error("unknown ticket");
        return MCS_ENOTFOUND;
    }
    if (it->second.status != MCS_OK) {
        // a failed or cancelled request: its own status and message
        const int st = it->second.status;
        set_error(it->second.msg);
        s->done.erase(it);
        return st;
    }
    if (result) {
        double *g = result->group_values;
        int cap = result->group_capacity;
        float *fr = result->frames;
        double *se = result->series;
        *result = it->second.r;
        result->group_values = g;
        result->group_capacity = cap;
        result->frames = fr;
        result->series = se;
        result->frames_written = 0;
        if (g)
            for (int k = 0; k < cap && k < (int)it->second.groups.size(); ++k) g[k] = it->second.groups[k];
    }
    s->done.erase(it);
    return 0;
}

extern "C" int mcs_server_stats(mcs_server *s, int32_t *active, int32_t *queued, uint64_t *bytes_in_use,
                                int64_t *site_updates)
{
    if (!s) { set_error("server is required"); return MCS_EINVAL; }
    std::lock_guard<std::mutex> lock(s->qmu);
    if (active) *active = (int32_t)s->n_active;
    if (queued) *queued = (int32_t)s->queue.size();
    if (bytes_in_use) *bytes_in_use = s->in_use;
    if (site_updates) *site_updates = s->site_updates;
    return MCS_OK;
}

extern "C" void mcs_server_destroy(mcs_server *s)
{
    if (!s) return;
    {
        std::lock_guard<std::mutex> slock(s->smu);
        if (s->batch.stream) cudaStreamSynchronize(s->batch.stream);
        s->batch.groups.clear();
    }
    delete s;
}
