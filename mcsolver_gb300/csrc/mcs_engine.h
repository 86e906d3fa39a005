// mcs_engine.h -- host engine objects behind the C ABI.
#pragma once
#include <cuda_runtime.h>

#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/mcsgpu.h"
#include "mcs_internal.h"
#include "mcs_model.h"

namespace mcs {

void set_error(const std::string &s);
const std::string &get_error();

// Device copy of a lattice's index arrays (geometry, classes, measurement
// lists), shared by every replica of a batch compiled from that lattice's
// template: the replicas of a temperature grid or a parallel-tempering ladder
// then read one copy of them (from L2) instead of one each.
struct SharedLists {
    void *d = nullptr;
    size_t bytes = 0;
    const int *nbr = nullptr;
    const unsigned short *lcode = nullptr, *rjc = nullptr;
    const unsigned char *deg = nullptr, *stype = nullptr, *rdeg = nullptr, *gmask = nullptr, *sflag = nullptr;
    const int *cpair = nullptr, *rorb = nullptr, *rcl = nullptr, *rlink = nullptr, *rindex = nullptr, *circ = nullptr,
              *rtgt = nullptr;
    const float *slen = nullptr, *sval = nullptr;
    ~SharedLists();
};
int make_shared_lists(const HostModel &m, int device, std::unique_ptr<SharedLists> *out);

// One solve on the device.
struct Replica {
    HostModel hm;
    Rep rep;                 // descriptor (device pointers into the arena)
    void *arena = nullptr;   // one device allocation per replica
    size_t bytes = 0;
    size_t acc_off = 0, icnt_off = 0, stats_off = 0, series_off = 0, spins_off = 0;
    void *frames_host = nullptr;       // spin frames: page-locked host memory mapped into the device
    size_t frames_bytes = 0;
    size_t nacc = 0;
    int schedule = 0;        // 1 plain, 2 resident, 3 tiled, 4/5 Wolff, 6 cluster
    int requested_schedule = 0;
    int record_series = 0;
    int recheck = 32;
    int device = 0;
    bool initialized = false;          // initial-state kernel has run
    int pref_C = 0;                    // cluster size chosen by the load balancer (0: none)
    const SharedLists *shared = nullptr; // index arrays shared with other replicas of the batch (or null)
    std::vector<unsigned char> staging; // host image of the arena until upload
    std::vector<unsigned char> rblock;  // host copy of the result block (acc, icnt, stats)
    bool rblock_fresh = false;          // rblock matches the device (set by a batched readback)
    ~Replica();
};

int build_replica(const mcs_problem *p, const mcs_options *o, Replica *r, bool upload,
                  const ModelTemplate *tmpl = nullptr, bool *reused = nullptr, const SharedLists *shared = nullptr);
int upload_replica(Replica *r);
int replica_results(Replica *r, const Rep &Rfinal, mcs_result *res);
// Read the result blocks of many replicas with one synchronisation.
int fetch_result_blocks(const std::vector<Replica *> &rs, int device);
int replica_spins(Replica *r, std::vector<double> &out);
int replica_set_spins(Replica *r, const double *in);
size_t replica_acc_count(const HostModel &m);

// A set of replicas advanced by one kernel family.
struct Group {
    int kind = 0;              // 1 plain, 2 resident, 3 tiled
    int dim = 0, geom = 0;
    std::vector<int> ids;
    int *d_ids = nullptr;      // device copy of ids (capacity ids_cap)
    int ids_cap = 0;
    long long max_units = 0, done_units = 0;
    // resident / cluster
    int threads = 0;
    size_t smem = 0;
    long long chunk = 0;
    int C = 0;                 // CTAs per replica of the cluster kernel (0 = the resident kernel)
    int tuned = 0;             // autotuner has chosen (C, threads)
    int can_cluster = 0;
    std::vector<std::pair<int, int>> candidates;  // (C, threads)
    std::string tune_key;      // autotuner cache key (group shape and candidates)
    std::vector<double> cand_ms;
    // tiled
    int maxcol = 0, nmeas = 0;
    std::vector<size_t> cofs;
    std::vector<int> ccount;
    Item *d_sw = nullptr, *d_mi = nullptr;
    int *d_ioff = nullptr, *d_moff = nullptr;
    double *d_dE = nullptr, *d_fp = nullptr;
    long long *d_ip = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int K = 0;
    long long per_graph = 0;
    std::vector<void *> bufs;
    ~Group();
};

// Many replicas of uneven sizes run together.
struct Batch {
    int device = 0;
    std::vector<std::unique_ptr<Replica>> replicas;
    Rep *d_reps = nullptr;
    StopItem *d_stop = nullptr;  // slot mode: (replica, quota) of the current step
    StopItem *h_stop = nullptr;  // page-locked staging of the same
    void *d_scratch = nullptr;
    bool prepared = false;
    std::vector<std::unique_ptr<Group>> groups;
    double last_ms = 0;
    cudaStream_t stream = nullptr, stream2 = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, ev_a = nullptr, ev_b = nullptr, ev_fork = nullptr;
    std::mutex add_mutex;       // mcs_batch_add may be called from several threads
    std::vector<std::shared_ptr<const ModelTemplate>> templates;  // compiled lattices of this batch (O(n))
    std::map<const ModelTemplate *, std::unique_ptr<SharedLists>> shared_lists;  // their index arrays on the device
    int cluster_override = 0;   // 1: never cluster; 2/4/8: only that size
    int no_autotune = 0;
    int balance = 1;            // place replicas by the load balancer (off for parallel tempering)
    std::vector<cudaStream_t> gstreams;  // one stream per group: groups run side by side
    std::vector<cudaStream_t> gstreams_hi;  // the same at the device's highest stream priority (tiled groups)
    std::vector<cudaEvent_t> gevents;
    double device_ms = 0;
    long long site_updates = 0;
    long long launches = 0;
    int threads_override = 0;
    long long chunk_override = 0;
    std::vector<Rep> final_reps;
    ~Batch();
    int init(int dev);
    int ensure_streams();
    int add(const mcs_problem *p, const mcs_options *o, int *idx);
    int prepare();                 // upload descriptors, initial energies, build groups
    int advance(long long units);  // every replica runs up to `units` more units
    // pieces of prepare(), also used by the server's slot mode
    int setup_device();
    void assign_schedules(const std::vector<int> &ids, int max_smem);
    int init_states(const std::vector<int> &ids);
    int build_groups(const std::vector<int> &ids, bool merge);
    int upload_ids(Group &G);
    int reset_tiled(Group &G);
    // slot mode (server): replicas[i] may be null; d_reps holds slot_capacity descriptors
    int slot_capacity = 0;
    int admit(const std::vector<int> &ids, double step_us);        // new replicas in these slots
    void drop(const std::vector<int> &ids, std::vector<int> *orphans);  // replicas leaving their groups
    int rebalance(double step_us, std::vector<int> *orphans);          // re-place the remaining replicas
    void set_quotas(const std::vector<int> &ids, double step_us);
    // every replica of the groups advances by its own quota (Rep::quota); the
    // replicas of a group whose launch failed are added to *failed
    int advance_quota(std::vector<int> *failed);
    int run_groups(const std::vector<long long> &todo, const std::vector<long long> &pre, std::vector<int> *failed,
                   std::vector<float> *group_ms = nullptr);
    double quota_ms = 0;             // slot mode: target device time of a group's share of a step
    std::vector<cudaEvent_t> tev;    // per-group timing events (start, end)
    int collect();                 // read back descriptors and counters
    int sync_descriptors();        // read back descriptors: progress travels with each replica
    void release_groups();         // drop groups and descriptor arrays; the next advance re-prepares
    int run();                     // prepare + advance to completion + collect
    int result(int i, mcs_result *res);
    int setup_tiled(Group &G);
    void place_replicas(int max_smem, const std::vector<int> &ids, double base_crit = 0, double base_smsec = 0,
                        double base_ctas = 0);
    cudaError_t tiled_unit(Group &G, cudaStream_t s, long long *nl);
    cudaError_t launch_group(Group &G, int C, int threads, long long units, cudaStream_t s);
};

}  // namespace mcs
