// mcs_server.cpp -- continuous-batching request loop (C ABI mcs_server_*).
//
// submit(): compiles the request on the host (validation, colouring, tables,
//           the arena image) and queues it; nothing touches the device yet.
// step():   1. admits queued requests in arrival order while a slot is free and
//              the HBM budget holds the request's arena (allocation + upload);
//           2. advances every active request by a chunk of units in one batched
//              launch sequence (the kernels of mcs_batch_*), so requests that
//              arrived at different times run side by side on the device;
//           3. retires requests that reached their last unit: results are kept
//              for poll(), the arena is freed and its bytes return to the budget.
// A request's spin trajectory depends only on its own problem and seed, so its
// result is the same alone and in any mix (tested).
#include <cuda_runtime.h>
#include <string.h>

#include <chrono>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <unordered_map>
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
    std::deque<std::pair<uint64_t, std::unique_ptr<Replica>>> queue;
    std::vector<std::pair<uint64_t, std::unique_ptr<Replica>>> active;
    struct Done {
        mcs_result r;
        std::vector<double> groups;
    };
    std::unordered_map<uint64_t, Done> done;
    uint64_t in_use = 0;
    long long site_updates = 0;
    std::mutex mu;
};

extern "C" int mcs_server_create(int32_t device, uint64_t hbm_budget_bytes, int32_t max_slots, mcs_server **out)
{
    if (!out || max_slots < 1 || hbm_budget_bytes == 0) { set_error("server needs a budget and >= 1 slot"); return MCS_EINVAL; }
    mcs_server *s = new mcs_server();
    s->device = device;
    s->budget = hbm_budget_bytes;
    s->max_slots = max_slots;
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
    std::lock_guard<std::mutex> lock(s->mu);
    const uint64_t t = s->next_ticket++;
    s->queue.emplace_back(t, std::move(r));
    if (ticket) *ticket = t;
    return MCS_OK;
}

extern "C" int mcs_server_step(mcs_server *s, int32_t *completed)
{
    if (!s) return MCS_EINVAL;
    std::lock_guard<std::mutex> lock(s->mu);
    if (completed) *completed = 0;
    // 1. admission by slots and HBM budget, in arrival order
    while (!s->queue.empty() && (int)s->active.size() < s->max_slots) {
        Replica &r = *s->queue.front().second;
        const uint64_t need = r.bytes + sizeof(Rep);
        if (s->in_use + need > s->budget) break;
        int rc = upload_replica(&r);
        if (rc != MCS_OK) return rc;
        s->in_use += need;
        s->active.push_back(std::move(s->queue.front()));
        s->queue.pop_front();
    }
    if (s->active.empty()) return MCS_OK;
    // 2. one chunk of units for every active request
    Batch b;
    b.init(s->device);
    b.no_autotune = 1;
    std::vector<uint64_t> tickets;
    for (auto &a : s->active) {
        tickets.push_back(a.first);
        b.replicas.push_back(std::move(a.second));
    }
    s->active.clear();
    int rc = b.advance(s->chunk);
    if (rc == MCS_OK) rc = b.collect();
    // 3. retire finished requests, keep the rest
    int ndone = 0;
    for (size_t i = 0; i < b.replicas.size(); ++i) {
        std::unique_ptr<Replica> r = std::move(b.replicas[i]);
        if (rc == MCS_OK && r->rep.u >= r->hm.units_total) {
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
            s->site_updates += d.r.site_updates;
            s->in_use -= r->bytes + sizeof(Rep);
            s->done.emplace(tickets[i], std::move(d));
            ++ndone;
        } else {
            s->active.emplace_back(tickets[i], std::move(r));
        }
    }
    b.replicas.clear();
    if (completed) *completed = ndone;
    return rc;
}

extern "C" int mcs_server_poll(mcs_server *s, uint64_t ticket, mcs_result *result)
{
    if (!s) return MCS_EINVAL;
    std::lock_guard<std::mutex> lock(s->mu);
    auto it = s->done.find(ticket);
    if (it == s->done.end()) {
        for (auto &q : s->queue) if (q.first == ticket) return 1;
        for (auto &a : s->active) if (a.first == ticket) return 1;
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
    std::lock_guard<std::mutex> lock(s->mu);
    if (active) *active = (int32_t)s->active.size();
    if (queued) *queued = (int32_t)s->queue.size();
    if (bytes_in_use) *bytes_in_use = s->in_use;
    if (site_updates) *site_updates = s->site_updates;
    return MCS_OK;
}

extern "C" void mcs_server_destroy(mcs_server *s) { delete s; }
