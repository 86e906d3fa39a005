// mcs_server.cpp -- continuous-batching request loop (C ABI mcs_server_*).
//
// submit(): compiles the request on the caller's thread (validation,
//           colouring, tables, the arena image) and queues it; nothing touches
//           the device yet.  submit() and poll() may be called from any number
//           of threads while another thread runs step(): they hold the queue
//           lock only to insert or look up, never across device work.
// step():   1. admits queued requests in arrival order while a slot is free and
//              the HBM budget holds the request's arena (allocation + upload);
//           2. advances every active request in one persistent batch: its
//              launch groups (and captured graphs) are rebuilt only when the
//              set of active requests changes, and each step runs as many
//              units as the chunk allows but never past the next completion,
//              so a finished request is retired at once;
//           3. retires requests that reached their last unit: results are kept
//              for poll(), the arena is freed and its bytes return to the budget.
// A request's spin trajectory depends only on its own problem and seed, so its
// result is the same alone and in any mix (tested).
#include <cuda_runtime.h>
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
    long long chunk = 50;
    struct Done {
        mcs_result r;
        std::vector<double> groups;
    };
    // guarded by qmu: the queue, finished results, tickets not yet finished, counters
    std::mutex qmu;
    std::deque<std::pair<uint64_t, std::unique_ptr<Replica>>> queue;
    std::unordered_map<uint64_t, Done> done;
    std::unordered_set<uint64_t> pending;
    uint64_t in_use = 0;
    long long site_updates = 0;
    int n_active = 0;
    // guarded by smu: the device side (one step at a time)
    std::mutex smu;
    Batch batch;                       // replicas = active requests
    std::vector<uint64_t> tickets;     // ticket of batch.replicas[i]
};

extern "C" int mcs_server_create(int32_t device, uint64_t hbm_budget_bytes, int32_t max_slots, mcs_server **out)
{
    if (!out || max_slots < 1 || hbm_budget_bytes == 0) { set_error("server needs a budget and >= 1 slot"); return MCS_EINVAL; }
    mcs_server *s = new mcs_server();
    s->device = device;
    s->budget = hbm_budget_bytes;
    s->max_slots = max_slots;
    s->batch.init(device);
    s->batch.no_autotune = 1;  // membership changes often; the first candidate of each group runs
    if (const char *e = getenv("MCSGPU_SERVER_CHUNK")) s->chunk = std::max(1LL, atoll(e));
    *out = s;
    return MCS_OK;
}

extern "C" int mcs_server_submit(mcs_server *s, const mcs_problem *problem, const mcs_options *options, uint64_t *ticket)
{
    if (!s || !problem) return MCS_EINVAL;
    mcs_options def;
    memset(&def, 0, sizeof def);
    if (!options) options = &def;
    std::unique_ptr<Replica> r(new Replica());
    r->device = s->device;
    int rc = build_replica(problem, options, r.get(), false);
    if (rc != MCS_OK) return rc;
    if (r->bytes + sizeof(Rep) > s->budget) { set_error("request larger than the server's HBM budget"); return MCS_ENOMEM; }
    std::lock_guard<std::mutex> lock(s->qmu);
    const uint64_t t = s->next_ticket++;
    s->queue.emplace_back(t, std::move(r));
    s->pending.insert(t);
    if (ticket) *ticket = t;
    return MCS_OK;
}

extern "C" int mcs_server_step(mcs_server *s, int32_t *completed)
{
    if (!s) return MCS_EINVAL;
    std::lock_guard<std::mutex> slock(s->smu);
    if (completed) *completed = 0;
    Batch &b = s->batch;
    // 1. admission by slots and HBM budget, in arrival order
    std::vector<std::pair<uint64_t, std::unique_ptr<Replica>>> admit;
    {
        std::lock_guard<std::mutex> lock(s->qmu);
        int slots = s->max_slots - (int)b.replicas.size();
        while (!s->queue.empty() && slots > 0) {
            Replica &r = *s->queue.front().second;
            const uint64_t need = r.bytes + sizeof(Rep);
            if (s->in_use + need > s->budget) break;
            s->in_use += need;
            admit.push_back(std::move(s->queue.front()));
            s->queue.pop_front();
            --slots;
        }
    }
    if (!admit.empty()) {
        // progress of the running requests goes back to their host descriptors
        // before the groups are rebuilt around the new set
        int rc = b.sync_descriptors();
        if (rc != MCS_OK) return rc;
        b.release_groups();
        for (auto &a : admit) {
            rc = upload_replica(a.second.get());
            if (rc != MCS_OK) {
                std::lock_guard<std::mutex> lock(s->qmu);
                s->in_use -= a.second->bytes + sizeof(Rep);
                s->pending.erase(a.first);
                return rc;
            }
            s->tickets.push_back(a.first);
            b.replicas.push_back(std::move(a.second));
        }
        std::lock_guard<std::mutex> lock(s->qmu);
        s->n_active = (int)b.replicas.size();
    }
    if (b.replicas.empty()) return MCS_OK;
    // 2. one chunk of units, ending at the next completion at the latest
    long long units = s->chunk;
    for (auto &r : b.replicas) units = std::min(units, std::max(1LL, r->hm.units_total - r->rep.u));
    int rc = b.advance(units);
    if (rc != MCS_OK) return rc;
    for (auto &r : b.replicas) r->rep.u = std::min(r->hm.units_total, r->rep.u + units);
    // 3. retire finished requests
    bool any = false;
    for (auto &r : b.replicas) any |= r->rep.u >= r->hm.units_total;
    if (!any) return MCS_OK;
    rc = b.sync_descriptors();
    if (rc != MCS_OK) return rc;
    {
        std::vector<Replica *> done_r;
        for (auto &r : b.replicas)
            if (r->rep.u >= r->hm.units_total) done_r.push_back(r.get());
        rc = fetch_result_blocks(done_r, s->device);  // one synchronisation for all of them
        if (rc != MCS_OK) return rc;
    }
    std::vector<std::pair<uint64_t, mcs_server::Done>> fin;
    std::vector<std::unique_ptr<Replica>> keep;
    std::vector<uint64_t> keep_t;
    uint64_t freed = 0;
    long long su = 0;
    for (size_t i = 0; i < b.replicas.size(); ++i) {
        std::unique_ptr<Replica> &r = b.replicas[i];
        if (r->rep.u < r->hm.units_total) {
            keep.push_back(std::move(r));
            keep_t.push_back(s->tickets[i]);
            continue;
        }
        mcs_server::Done d;
        memset(&d.r, 0, sizeof d.r);
        const int G = r->hm.ngroup;
        d.groups.assign((size_t)(G + 1) * (G + 1) + (G + 1), 0.0);
        d.r.group_values = d.groups.data();
        d.r.group_capacity = (int)d.groups.size();
        int rr = replica_results(r.get(), r->rep, &d.r);
        d.r.group_values = nullptr;
        d.r.frames = nullptr;
        d.r.series = nullptr;
        if (rr != MCS_OK) return rr;
        su += d.r.site_updates;
        freed += r->bytes + sizeof(Rep);
        fin.emplace_back(s->tickets[i], std::move(d));
    }
    b.release_groups();
    b.replicas.swap(keep);
    s->tickets.swap(keep_t);
    keep.clear();  // frees the retired arenas
    std::lock_guard<std::mutex> lock(s->qmu);
    for (auto &f : fin) {
        s->pending.erase(f.first);
        s->done.emplace(f.first, std::move(f.second));
    }
    s->site_updates += su;
    s->in_use -= freed;
    s->n_active = (int)b.replicas.size();
    if (completed) *completed = (int32_t)fin.size();
    return MCS_OK;
}

extern "C" int mcs_server_poll(mcs_server *s, uint64_t ticket, mcs_result *result)
{
    if (!s) return MCS_EINVAL;
    std::lock_guard<std::mutex> lock(s->qmu);
    auto it = s->done.find(ticket);
    if (it == s->done.end()) {
        if (s->pending.count(ticket)) return 1;
        set_error("unknown ticket");
        return MCS_ENOTFOUND;
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
    if (!s) return MCS_EINVAL;
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
        s->batch.release_groups();
    }
    delete s;
}
