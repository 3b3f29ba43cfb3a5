// Many universes of one module in one run, and the launch-shape autotuner.
//
// kunRunGraphBatch runs `njobs` jobs (universes of their own stock count and
// length) of one batch module.  Stage by stage in the module's order, a
// time-series stage that supports grouped launches runs each of its kernels
// ONCE over the tiles of all jobs (the job of a block is found from a tile
// table passed by value); a Rank stage ranks every job's rows in one launch;
// other stages run job by job.  The jobs' parameter
// blocks go to the device with one copy per stage.  This replaces the
// reference's one runGraph per universe (cpp/Kun/Runtime.cpp:311-352).
//
// kunExecutorTune picks, per stage, the time tile of the time-parallel
// kernels and the threads per block by timing candidate shapes on the jobs
// given (CUDA events on the executor's stream), keeping the fastest.  The
// executor then uses those shapes in kunRunGraphBatch and kunRunGraphEx.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "kun_runtime_internal.h"
#include "kun_xsec.cuh"

namespace kungpu {

// jobs per grouped launch (the modules' tile tables hold this many)
static constexpr int KUN_GROUP_MAX = 256;

static bool batch_device_pointer(const void *p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

struct BatchJob {
    long long S, total_time, cur_time, length;
    const Plan *plan;
    std::vector<void *> ptrs;
    size_t arena_off;
};

struct BatchRun {
    Executor *ex;
    const KunGpuModuleDesc *m;
    std::vector<BatchJob> jobs;
    std::vector<int> order;
    size_t host_off = 0;  // parameter blocks staged so far in this run
};

static KunStatus batch_setup(Executor *ex, const KunGpuModuleDesc *m, int njobs, const NameMap *const *maps,
                             const size_t *S, const size_t *total_time, const size_t *cur_time,
                             const size_t *length, BatchRun &br) {
    if (!ex || !m || njobs <= 0 || !maps || !S || !total_time || !cur_time || !length) {
        set_error("kunRunGraphBatch: bad arguments");
        return KUN_INVALID_ARGUMENT;
    }
    if (m->abi != KUN_GPU_MODULE_ABI) {
        set_error("The required version in the module does not match the runtime version");
        return KUN_INVALID_ARGUMENT;
    }
    if (m->output_layout == KUN_LAYOUT_STREAM) {
        set_error("Cannot run stream mode module via runGraph()");
        return KUN_INVALID_ARGUMENT;
    }
    br.ex = ex;
    br.m = m;
    br.jobs.resize(njobs);
    size_t total = 0;
    for (int j = 0; j < njobs; j++) {
        BatchJob &jb = br.jobs[j];
        jb.S = (long long)S[j];
        jb.total_time = (long long)total_time[j];
        jb.cur_time = (long long)cur_time[j];
        jb.length = (long long)length[j];
        if (jb.S <= 0 || jb.length <= 0 || jb.cur_time + jb.length > jb.total_time || !maps[j]) {
            set_error("kunRunGraphBatch: bad shape of job %d", j);
            return KUN_INVALID_ARGUMENT;
        }
        if (m->aligned && m->input_layout == KUN_LAYOUT_TS && (jb.S % m->blocking_len) != 0) {
            set_error("Bad shape: num_stocks %lld of job %d is not a multiple of %d", jb.S, j, m->blocking_len);
            return KUN_INVALID_ARGUMENT;
        }
        auto key = std::make_tuple((const void *)m, jb.S, jb.length, 1);
        auto it = ex->plans.find(key);
        if (it == ex->plans.end()) {
            Plan p;
            if (!make_plan(m, jb.S, jb.length, 1, p)) return KUN_INVALID_ARGUMENT;
            it = ex->plans.emplace(key, std::move(p)).first;
        }
        jb.plan = &it->second;
        jb.arena_off = total;
        total += (jb.plan->slot_bytes * (size_t)jb.plan->num_slots + 255) / 256 * 256;
    }
    br.order = br.jobs[0].plan->order;
    if (!ex->arena.ensure(total)) {
        set_error("out of device memory for the temporaries of %d jobs (%zu bytes)", njobs, total);
        return KUN_OUT_OF_MEMORY;
    }
    for (int j = 0; j < njobs; j++) {
        BatchJob &jb = br.jobs[j];
        jb.ptrs.assign(m->num_buffers, nullptr);
        for (int b = 0; b < m->num_buffers; b++) {
            const KunGpuBufferDesc &bd = m->buffers[b];
            if (bd.kind == KUN_BUF_TEMP) {
                if (jb.plan->temp_slot[b] >= 0)
                    jb.ptrs[b] = (char *)ex->arena.ptr + jb.arena_off +
                                 jb.plan->slot_bytes * (size_t)jb.plan->temp_slot[b];
                continue;
            }
            auto f = maps[j]->find(bd.name);
            if (f == maps[j]->end() || !f->second) {
                set_error("Buffer name not found: %s (job %d)", bd.name, j);
                return KUN_INVALID_ARGUMENT;
            }
            if (!batch_device_pointer(f->second)) {
                set_error("kunRunGraphBatch: buffer %s of job %d is not device memory", bd.name, j);
                return KUN_INVALID_ARGUMENT;
            }
            jb.ptrs[b] = f->second;
        }
    }
    return KUN_SUCCESS;
}

static bool ensure_group_staging(Executor *ex, size_t need) {
    if (need <= ex->group_host_bytes) return ex->group_dev.ensure(need);
    if (ex->group_host) cudaFreeHost(ex->group_host);
    ex->group_host = nullptr;
    ex->group_host_bytes = 0;
    if (cudaHostAlloc(&ex->group_host, need, cudaHostAllocDefault) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    ex->group_host_bytes = need;
    return ex->group_dev.ensure(need);
}

// Enqueue stage `si` for every job; `tile`/`block` override the tuning table.
static KunStatus batch_stage(BatchRun &br, int si, cudaStream_t st, const int32_t *tile, const int32_t *block,
                             int64_t &launches) {
    Executor *ex = br.ex;
    const KunGpuModuleDesc *m = br.m;
    const KunGpuStageDesc &d = m->stages[si];
    const int n = (int)br.jobs.size();
    std::vector<std::vector<void *>> scratch(n);
    std::vector<KunGpuStageArgs> args(n);
    auto tn = ex->tuning.find((const void *)m);
    for (int j = 0; j < n; j++) {
        BatchJob &jb = br.jobs[j];
        for (int sl : jb.plan->scratch[si])
            scratch[j].push_back((char *)ex->arena.ptr + jb.arena_off + jb.plan->slot_bytes * (size_t)sl);
        KunGpuStageArgs &a = args[j];
        memset(&a, 0, sizeof a);
        a.buffers = jb.ptrs.data();
        a.scratch = scratch[j].data();
        a.num_stocks = jb.S;
        a.total_time = jb.total_time;
        a.start = jb.cur_time;
        a.length = jb.length;
        a.error_flag = ex->d_error;
        if (tile) {
            a.tune_tile = tile;
            a.tune_block = block;
        } else if (tn != ex->tuning.end() && si < (int)tn->second.size() && !tn->second[si].tile.empty()) {
            a.tune_tile = tn->second[si].tile.data();
            a.tune_block = tn->second[si].block.data();
        }
    }
    // Rank stages in the TS layout: every job's rows in one launch
    const bool ts_rank = d.kind == KUN_STAGE_RANK && n > 1 && d.num_in == 1 && d.num_out == 1 &&
                         (m->buffers[d.in_bufs[0]].kind != KUN_BUF_INPUT || m->input_layout == KUN_LAYOUT_TS) &&
                         (m->buffers[d.out_bufs[0]].kind != KUN_BUF_OUTPUT || m->output_layout == KUN_LAYOUT_TS);
    if (ts_rank) {
        const int bi = d.in_bufs[0], bo = d.out_bufs[0];
        const size_t esz = m->dtype == 0 ? 4 : 8;
        std::vector<kun::RankRowsJob> jobs;
        long long rows = 0, max_S = 0;
        for (int j = 0; j < n; j++) {
            const BatchJob &jb = br.jobs[j];
            if (jb.S <= 0 || jb.length <= 0) continue;
            kun::RankRowsJob rj;
            const long long row_off = m->buffers[bi].kind == KUN_BUF_INPUT ? jb.cur_time : 0;
            rj.in = (const char *)jb.ptrs[bi] + (size_t)row_off * (size_t)jb.S * esz;
            rj.out = jb.ptrs[bo];
            rj.S = jb.S;
            rj.length = jb.length;
            rj.row0 = rows;
            rows += jb.length;
            max_S = std::max(max_S, jb.S);
            jobs.push_back(rj);
        }
        const size_t bytes = jobs.size() * sizeof(kun::RankRowsJob);
        const size_t off = (br.host_off + 255) / 256 * 256;
        if (off + bytes > ex->group_host_bytes) {
            set_error("grouped launch staging exhausted");
            return KUN_OUT_OF_MEMORY;
        }
        memcpy((char *)ex->group_host + off, jobs.data(), bytes);
        char *dev = (char *)ex->group_dev.ptr + off;
        cudaMemcpyAsync(dev, (char *)ex->group_host + off, bytes, cudaMemcpyHostToDevice, st);
        int rc = m->dtype == 0 ? kun::launch_rank_rows_multi<float>((const kun::RankRowsJob *)dev, (int)jobs.size(),
                                                                    rows, max_S, st)
                               : kun::launch_rank_rows_multi<double>((const kun::RankRowsJob *)dev,
                                                                     (int)jobs.size(), rows, max_S, st);
        if (rc) {
            set_error("stage %d (%s) grouped Rank failed: %s", si, d.name, cudaGetErrorString((cudaError_t)rc));
            return KUN_CUDA_ERROR;
        }
        br.host_off = off + bytes;
        launches += 1;
        return KUN_SUCCESS;
    }
    if (d.launch_group && n > 1) {
        for (int j0 = 0; j0 < n; j0 += KUN_GROUP_MAX) {
            const int nj = std::min(KUN_GROUP_MAX, n - j0);
            const size_t bytes = d.prepare(&args[j0], nj, nullptr);
            const size_t off = (br.host_off + 255) / 256 * 256;
            if (off + bytes > ex->group_host_bytes) {
                set_error("grouped launch staging exhausted");
                return KUN_OUT_OF_MEMORY;
            }
            d.prepare(&args[j0], nj, (char *)ex->group_host + off);
            char *dev = (char *)ex->group_dev.ptr + off;
            cudaMemcpyAsync(dev, (char *)ex->group_host + off, bytes, cudaMemcpyHostToDevice, st);
            int rc = d.launch_group(&args[j0], nj, dev, (void *)st);
            if (rc) {
                set_error("stage %d (%s) grouped launch failed: %s", si, d.name, cudaGetErrorString((cudaError_t)rc));
                return KUN_CUDA_ERROR;
            }
            br.host_off = off + bytes;
            launches += d.num_kernels > 0 ? d.num_kernels : 1;
        }
        return KUN_SUCCESS;
    }
    for (int j = 0; j < n; j++) {
        int rc = d.launch(&args[j], (void *)st);
        if (rc) {
            set_error("stage %d (%s) launch failed for job %d: %s", si, d.name, j,
                      cudaGetErrorString((cudaError_t)rc));
            return KUN_CUDA_ERROR;
        }
        launches += d.num_kernels > 0 ? d.num_kernels : 1;
    }
    return KUN_SUCCESS;
}

// bytes of the parameter blocks of one pass over all stages
static size_t batch_staging_bytes(const BatchRun &br) {
    size_t need = 0;
    const int n = (int)br.jobs.size();
    for (int si = 0; si < br.m->num_stages; si++) {
        const KunGpuStageDesc &d = br.m->stages[si];
        if (d.kind == KUN_STAGE_RANK && n > 1) {  // the grouped Rank's job table
            need += ((size_t)n * sizeof(kun::RankRowsJob) + 255) / 256 * 256;
            continue;
        }
        if (!d.launch_group || n <= 1) continue;
        std::vector<KunGpuStageArgs> args(n);
        memset(args.data(), 0, sizeof(KunGpuStageArgs) * n);
        for (int j0 = 0; j0 < n; j0 += KUN_GROUP_MAX)
            need += (d.prepare(&args[j0], std::min(KUN_GROUP_MAX, n - j0), nullptr) + 255) / 256 * 256;
    }
    return need + 256;
}

static KunStatus batch_begin(Executor *ex, BatchRun &br, size_t passes) {
    if (!ensure_group_staging(ex, batch_staging_bytes(br) * passes)) {
        set_error("out of memory for grouped launch staging");
        return KUN_OUT_OF_MEMORY;
    }
    br.host_off = 0;
    return KUN_SUCCESS;
}

static KunStatus batch_finish(Executor *ex, cudaStream_t st, bool sync) {
    if (ex->has_user_stream) {
        cudaEventRecord(ex->bridge_out, st);
        cudaStreamWaitEvent(ex->user_stream, ex->bridge_out, 0);
    }
    // the pinned staging is reused by the next run: always wait for the copies
    (void)sync;
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        set_error("CUDA error: %s", cudaGetErrorString(e));
        return KUN_CUDA_ERROR;
    }
    return KUN_SUCCESS;
}

}  // namespace kungpu

using namespace kungpu;

KUN_EXPORT KunStatus kunRunGraphBatch(KunExecutorHandle exec, KunModuleHandle mod, int njobs,
                                      const KunBufferNameMapHandle *buffers, const size_t *num_stocks,
                                      const size_t *total_time, const size_t *cur_time, const size_t *length,
                                      int synchronize) {
    clear_error();
    auto *ex = (Executor *)exec;
    if (!ex) return KUN_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(ex->mu);
    cudaSetDevice(ex->device);
    ex->check_epoch();
    BatchRun br;
    KunStatus rs = batch_setup(ex, (const KunGpuModuleDesc *)mod, njobs, (const NameMap *const *)buffers,
                               num_stocks, total_time, cur_time, length, br);
    if (rs != KUN_SUCCESS) return rs;
    if ((rs = batch_begin(ex, br, 1)) != KUN_SUCCESS) return rs;
    cudaStream_t st = ex->stream();
    if (ex->has_user_stream) {
        cudaEventRecord(ex->bridge_in, ex->user_stream);
        cudaStreamWaitEvent(st, ex->bridge_in, 0);
    }
    int64_t launches = 0;
    for (int si : br.order)
        if ((rs = batch_stage(br, si, st, nullptr, nullptr, launches)) != KUN_SUCCESS) return rs;
    ex->last_launches = launches;
    return batch_finish(ex, st, synchronize != 0);
}

// Tune the launch shapes of every grouped-capable stage on these jobs (the
// jobs' outputs are computed along the way).  Candidates: time tiles
// {default, 16, 32, 64, 128, 256} x {64, 128} threads per block for all the
// time-parallel kernels of a stage together, {32, 64, 128} threads for its
// scan kernels; then per time-parallel kernel, with the others held: its
// 64-register instance or not x block size, then its tile.  Each candidate
// runs the stage `reps` times after one warm-up; the fastest mean wins.
// Returns the number of stages tuned, or -1 on error.
KUN_EXPORT int kunExecutorTune(KunExecutorHandle exec, KunModuleHandle mod, int njobs,
                               const KunBufferNameMapHandle *buffers, const size_t *num_stocks,
                               const size_t *total_time, const size_t *cur_time, const size_t *length, int reps) {
    clear_error();
    auto *ex = (Executor *)exec;
    if (!ex) return -1;
    std::lock_guard<std::mutex> lk(ex->mu);
    cudaSetDevice(ex->device);
    ex->check_epoch();
    const auto *m = (const KunGpuModuleDesc *)mod;
    BatchRun br;
    if (batch_setup(ex, m, njobs, (const NameMap *const *)buffers, num_stocks, total_time, cur_time, length, br) !=
        KUN_SUCCESS)
        return -1;
    reps = std::max(1, reps);
    const int tiles[] = {0, 16, 32, 64, 128, 256};
    const int blocks[] = {64, 128};
    const int sblocks[] = {32, 64, 128};
    // each candidate run stages its parameter blocks once per repetition
    const size_t passes = (sizeof(tiles) / sizeof(int)) * (sizeof(blocks) / sizeof(int)) * (size_t)(reps + 1) + 4;
    if (batch_begin(ex, br, passes) != KUN_SUCCESS) return -1;
    cudaStream_t st = ex->stream();
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    auto &table = ex->tuning[(const void *)m];
    table.assign(m->num_stages, Executor::StageTune());
    int tuned = 0;
    int64_t launches = 0;
    for (int si : br.order) {
        const KunGpuStageDesc &d = m->stages[si];
        if (!d.kernel_info || d.num_kernels <= 0) {
            if (batch_stage(br, si, st, nullptr, nullptr, launches) != KUN_SUCCESS) return -1;
            continue;
        }
        const int nk = d.num_kernels;
        bool has_par = false, has_scan = false;
        for (int k = 0; k < nk; k++) (d.kernel_info[k] & 1 ? has_scan : has_par) = true;
        std::vector<int32_t> best_t(nk, 0), best_b(nk, 0), t(nk), b(nk);
        float best = -1.f;
        // times the stage with shape (t, b); keeps it when fastest so far
        auto run = [&]() -> bool {
            // the staging area is reused from its start: the copies of every
            // earlier launch (this stage's trials, and the untuned stages
            // enqueued before it) must have left it
            if (cudaStreamSynchronize(st) != cudaSuccess) return false;
            br.host_off = 0;
            if (batch_stage(br, si, st, t.data(), b.data(), launches) != KUN_SUCCESS) return false;
            cudaEventRecord(e0, st);
            for (int r = 0; r < reps; r++) {
                if (batch_stage(br, si, st, t.data(), b.data(), launches) != KUN_SUCCESS) return false;
            }
            cudaEventRecord(e1, st);
            if (cudaEventSynchronize(e1) != cudaSuccess) return false;
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            if (best < 0 || ms < best) {
                best = ms;
                best_t = t;
                best_b = b;
            }
            return true;
        };
        auto trial = [&](int tile, int blk, int sblk) -> bool {
            for (int k = 0; k < nk; k++) {
                const bool scan = d.kernel_info[k] & 1;
                t[k] = scan ? 0 : tile;
                b[k] = scan ? sblk : blk;
            }
            return run();
        };
        // one shape for every kernel of the stage first
        for (int tile : tiles) {
            if (!has_par && tile != 0) continue;
            for (int blk : blocks) {
                if (!has_par && blk != 128) continue;
                if (!trial(tile, blk, 128)) return -1;
            }
        }
        if (has_scan) {
            std::vector<int32_t> pt = best_t, pb = best_b;
            for (int sblk : sblocks) {
                int tile = 0, blk = 128;
                for (int k = 0; k < nk; k++)
                    if (!(d.kernel_info[k] & 1)) {
                        tile = pt[k];
                        blk = pb[k];
                    }
                if (!trial(tile, blk, sblk)) return -1;
            }
        }
        // then each time-parallel kernel on its own: the 64-register
        // instance and the block size, then the tile, the others held at
        // their best
        for (int k = 0; k < nk && has_par; k++) {
            if (d.kernel_info[k] & 1) continue;
            for (int cap : {0, (int)KUN_BLOCK_REGCAP}) {
                for (int blk : blocks) {
                    t = best_t;
                    b = best_b;
                    b[k] = blk | cap;
                    if (b[k] == best_b[k]) continue;
                    if (!run()) return -1;
                }
            }
            for (int tile : tiles) {
                t = best_t;
                b = best_b;
                if (tile == t[k]) continue;
                t[k] = tile;
                if (!run()) return -1;
            }
        }
        table[si].tile = best_t;
        table[si].block = best_b;
        // leave the stage's outputs from the chosen shape
        br.host_off = 0;
        if (batch_stage(br, si, st, best_t.data(), best_b.data(), launches) != KUN_SUCCESS) return -1;
        if (cudaStreamSynchronize(st) != cudaSuccess) return -1;
        tuned++;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    // graphs captured before tuning used the old shapes
    for (auto &g : ex->graphs) cudaGraphExecDestroy(g.exec);
    ex->graphs.clear();
    ex->seen.clear();
    if (cudaStreamSynchronize(st) != cudaSuccess) return -1;
    return tuned;
}

// The tuned shape of one stage: fills up to `cap` kernels' tiles and blocks;
// returns the kernel count, 0 when the stage has no tuned shape.
KUN_EXPORT int kunExecutorTunedShape(KunExecutorHandle exec, KunModuleHandle mod, int stage, int32_t *tile,
                                     int32_t *block, int cap) {
    auto *ex = (Executor *)exec;
    if (!ex) return -1;
    auto it = ex->tuning.find((const void *)mod);
    if (it == ex->tuning.end() || stage < 0 || stage >= (int)it->second.size()) return 0;
    const auto &tn = it->second[stage];
    int n = (int)tn.tile.size();
    for (int k = 0; k < std::min(n, cap); k++) {
        if (tile) tile[k] = tn.tile[k];
        if (block) block[k] = tn.block[k];
    }
    return n;
}

KUN_EXPORT KunStatus kunExecutorClearTuning(KunExecutorHandle exec) {
    auto *ex = (Executor *)exec;
    if (!ex) return KUN_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(ex->mu);
    ex->tuning.clear();
    for (auto &g : ex->graphs) cudaGraphExecDestroy(g.exec);
    ex->graphs.clear();
    ex->seen.clear();
    return KUN_SUCCESS;
}
