// Internals shared by the runtime translation units of libkungpu.so.
#pragma once
#include <cuda_runtime.h>

#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <tuple>
#include <unordered_map>
#include <vector>

#include "kun_gpu.h"
#include "kun_module_abi.h"

#define KUN_EXPORT extern "C" __attribute__((visibility("default")))

namespace kungpu {

void set_error(const char *fmt, ...);
void clear_error();
const char *last_error();

// buffer name -> user pointer (kunSetBufferNameMap)
using NameMap = std::unordered_map<std::string, float *>;

struct Library {
    void *handle = nullptr;
    std::string path;
};

struct Arena {
    void *ptr = nullptr;
    size_t bytes = 0;
    ~Arena() {
        if (ptr) cudaFree(ptr);
    }
    bool ensure(size_t need) {
        if (need <= bytes) return true;
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
        if (need == 0) return true;
        if (cudaMalloc(&ptr, need) != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
        bytes = need;
        return true;
    }
};

// Static execution plan of one module for a (num_stocks, length) shape.
struct Plan {
    std::vector<int> order;                 // stage ids in a topological order
    std::vector<std::vector<int>> preds;    // stage -> stages producing its inputs
    std::vector<int> temp_slot;             // per buffer: arena slot or -1
    std::vector<std::vector<int>> scratch;  // per stage: slots of its scratch
    std::vector<int> stream_of;             // per stage: stream index
    int num_streams = 1;
    int num_slots = 0;
    size_t slot_bytes = 0;
};

// Number of kunUnloadLibrary calls so far.  Caches keyed by a module
// descriptor's address (plans, captured graphs, tuned shapes) are dropped
// when it changes: another library can be loaded at the same address.
uint64_t library_epoch();

// Builds the stage order and the slot assignment of temporaries and scratch
// for `nstreams` streams; false (with the error set) on a cyclic stage graph.
bool make_plan(const KunGpuModuleDesc *m, long long S, long long length, int nstreams, Plan &p);

// A captured CUDA graph of one run, valid for the exact buffers it was
// captured with.
struct GraphEntry {
    std::vector<void *> key;
    cudaGraphExec_t exec = nullptr;
    int64_t launches = 0;
};

struct Executor {
    int device = 0;
    std::vector<cudaStream_t> streams;
    cudaStream_t user_stream = nullptr;
    Arena arena;
    Arena staging;
    int64_t last_launches = 0;
    int32_t *d_error = nullptr;  // set by a kernel whose bounded wait ran out
    uint64_t epoch = 0;  // library_epoch() the module caches below belong to
    std::map<std::tuple<const void *, long long, long long, int>, Plan> plans;
    std::mutex mu;
    // optional per-stage timing (CUDA events around every launch)
    bool profile = false;
    std::vector<cudaEvent_t> ev;
    std::vector<int> ev_stage;
    // stage completion events for cross-stream dependencies
    std::vector<cudaEvent_t> done;
    cudaEvent_t fork = nullptr;
    // graph replay: a run whose key was seen before is captured once
    bool use_graphs = true;
    std::map<std::vector<void *>, int> seen;
    std::vector<GraphEntry> graphs;
    // ordering with a caller's stream: work always runs on streams[0] and is
    // bridged to the caller's stream with these events
    bool has_user_stream = false;
    cudaEvent_t bridge_in = nullptr, bridge_out = nullptr;
    // tuned launch shapes per module and stage (time tile, threads per
    // block, per kernel); empty vectors mean the generated defaults
    struct StageTune {
        std::vector<int32_t> tile, block;
    };
    std::map<const void *, std::vector<StageTune>> tuning;
    // pinned host and device staging of grouped-launch parameter blocks
    void *group_host = nullptr;
    Arena group_dev;
    size_t group_host_bytes = 0;
    // copy streams for device-to-host output copies overlapping the stages
    std::vector<cudaStream_t> copy_streams;
    std::vector<cudaEvent_t> copy_ev;    // per stage: its outputs are ready
    std::vector<cudaEvent_t> copy_done;  // per copy stream: all copies issued so far are done
    cudaStream_t stream() const { return streams[0]; }
    // drops plans, graphs and tuned shapes if a library was unloaded since
    // they were made (call with `mu` held)
    void check_epoch();
};

// Device state of a stream module for `cap` stock columns: per buffer a ring
// of `window` rows ([window][cap], row n % window holds tick n) and per stage
// its op states as arrays of `cap` (float/double, then int32).
struct StreamStore {
    const KunGpuModuleDesc *m = nullptr;
    long long cap = 0;
    std::vector<void *> rings;
    std::vector<void *> st_t, st_i;
    void *d_init = nullptr;  // segment table of one reset
    void **d_rows = nullptr;  // start of every ring row (all buffers)
    long long n_rows = 0;
    bool alloc(const KunGpuModuleDesc *mod, long long capacity);
    void release();
    size_t bytes_per_stock() const;
    KunStatus reset(long long stock0, long long count, cudaStream_t st);
};

// Stage order of a stream module (false on a cycle).
bool stream_order(const KunGpuModuleDesc *m, std::vector<int> &order);

// Concurrent stages of one tick: stage -> stream, with completion events.
struct TickSchedule {
    std::vector<int> stream_of;
    std::vector<std::vector<int>> preds;
    std::vector<cudaStream_t> streams;  // [0] is the caller's stream (unused slot)
    std::vector<cudaEvent_t> done;      // per stage
    std::vector<cudaEvent_t> join;      // per stream
    cudaEvent_t fork = nullptr;
};
bool make_tick_schedule(const KunGpuModuleDesc *m, const std::vector<int> &order, int nstreams, TickSchedule &s);
void free_tick_schedule(TickSchedule &s);

// A tick as a chain of stage-graph levels: level d holds the stages whose
// longest path from a source has d stages, so the stages of a level do not
// depend on each other.  The Rank stages of a level run as one launch over
// (segment, stage) blocks; every other stage keeps its own launch.  All on
// one stream: a tick is a short chain of launches instead of one launch per
// stage with cross-stream events.
struct TickLevels {
    std::vector<std::vector<int>> other;  // per level: non-Rank stages
    std::vector<int> rank_off, rank_cnt;  // per level: slice of the job table
    void *d_jobs = nullptr;               // device RankJob table
    // the Rank launch of long segments runs beside the short ones' on
    // `side` (forked from and joined to the tick's stream at each level)
    cudaStream_t side = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
    bool ok = false;
};
// false when a Rank stage does not read and write exactly one ring
bool make_tick_levels(const StreamStore &store, const std::vector<int> &order, TickLevels &lv);
void free_tick_levels(TickLevels &lv);

// Enqueue one tick of every stage of `store` for the segments described by
// the device arrays; with `d_seg_count` the host counts are upper bounds.
// With `levels` the tick runs level by level on `st` (TickLevels), else
// stage by stage on `sched`'s streams (or on `st` alone).
KunStatus enqueue_tick(const StreamStore &store, const std::vector<int> &order, const int32_t *d_seg_off,
                       const int32_t *d_seg_stock0, const int64_t *d_tick, int nseg, long long n_active,
                       int max_len, cudaStream_t st, const int32_t *d_seg_count = nullptr,
                       const TickSchedule *sched = nullptr, const TickLevels *levels = nullptr);

}  // namespace kungpu
