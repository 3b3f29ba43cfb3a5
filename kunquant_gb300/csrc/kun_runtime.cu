// libkungpu.so: the runtime behind the C ABI of include/kun_gpu.h.
//
// Batch execution (replaces cpp/Kun/Runtime.cpp:311-352 + Executor.cpp): the
// stage DAG of a module is ordered once; temporaries between stages live in a
// device arena whose slots are reused by liveness (a temp's slot is released
// after its last consumer, like the reference frees on last deref,
// Runtime.cpp:84-93), and the stage kernels are enqueued on the executor's
// CUDA stream.  Host buffers are staged to the device inside the call.
#include <cuda_runtime.h>

#include <atomic>
#include <dlfcn.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "kun_runtime_internal.h"

namespace kungpu {

static thread_local std::string g_last_error;

void set_error(const char *fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
}
void clear_error() { g_last_error.clear(); }
const char *last_error() { return g_last_error.c_str(); }

static size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

static bool topo_order(const KunGpuModuleDesc *m, std::vector<int> &order) {
    std::vector<int> pending(m->num_stages);
    for (int i = 0; i < m->num_stages; i++) pending[i] = m->stages[i].pending;
    std::vector<int> ready;
    for (int i = 0; i < m->num_stages; i++)
        if (pending[i] == 0) ready.push_back(i);
    size_t head = 0;
    while (head < ready.size()) {
        int i = ready[head++];
        order.push_back(i);
        const KunGpuStageDesc &s = m->stages[i];
        for (int d = 0; d < s.num_deps; d++) {
            int j = s.deps[d];
            if (j < 0) continue;
            if (--pending[j] == 0) ready.push_back(j);
        }
    }
    return (int)order.size() == m->num_stages;
}

// Plan: topological order, stage -> stream assignment and slot assignment of
// temporaries and scratch.  A slot is reused by stage P only when every stage
// that last touched it is an ancestor of P in the stage DAG, so the plan is
// safe however the streams interleave (the reference frees a temporary on its
// last deref, cpp/Kun/Runtime.cpp:84-93).
bool make_plan(const KunGpuModuleDesc *m, long long S, long long length, int nstreams, Plan &p) {
    if (!topo_order(m, p.order)) {
        set_error("module %s: cyclic stage graph", m->name);
        return false;
    }
    int ns = m->num_stages;
    p.preds.assign(ns, {});
    for (int i = 0; i < ns; i++) {
        const KunGpuStageDesc &s = m->stages[i];
        for (int d = 0; d < s.num_deps; d++)
            if (s.deps[d] >= 0) p.preds[s.deps[d]].push_back(i);
    }
    int words = (ns + 63) / 64;
    std::vector<std::vector<uint64_t>> anc(ns, std::vector<uint64_t>(words, 0));
    for (int i : p.order)
        for (int d : p.preds[i]) {
            anc[i][d / 64] |= 1ull << (d % 64);
            for (int w = 0; w < words; w++) anc[i][w] |= anc[d][w];
        }
    auto is_anc = [&](int a, int of) { return (anc[of][a / 64] >> (a % 64)) & 1ull; };
    size_t elem = m->dtype == 0 ? 4 : 8;
    p.slot_bytes = align_up((size_t)S * (size_t)length * elem, 256);
    int nb = m->num_buffers;
    std::vector<std::vector<int>> consumers(nb);
    for (int i = 0; i < ns; i++) {
        const KunGpuStageDesc &s = m->stages[i];
        for (int k = 0; k < s.num_in; k++) {
            int b = s.in_bufs[k];
            if (std::find(consumers[b].begin(), consumers[b].end(), i) == consumers[b].end())
                consumers[b].push_back(i);
        }
    }
    std::vector<int> remaining(nb);
    for (int b = 0; b < nb; b++) remaining[b] = (int)consumers[b].size();
    p.temp_slot.assign(nb, -1);
    p.scratch.assign(ns, {});
    struct Slot {
        bool busy = false;
        std::vector<int> releasers;
    };
    std::vector<Slot> slots;
    auto take = [&](int stage) {
        for (size_t k = 0; k < slots.size(); k++) {
            if (slots[k].busy) continue;
            bool ok = true;
            for (int r : slots[k].releasers)
                if (!is_anc(r, stage)) { ok = false; break; }
            if (ok) {
                slots[k].busy = true;
                return (int)k;
            }
        }
        slots.push_back(Slot());
        slots.back().busy = true;
        return (int)slots.size() - 1;
    };
    for (int si : p.order) {
        const KunGpuStageDesc &s = m->stages[si];
        for (int k = 0; k < s.num_out; k++) {
            int b = s.out_bufs[k];
            if (m->buffers[b].kind == KUN_BUF_TEMP) p.temp_slot[b] = take(si);
        }
        for (int k = 0; k < s.num_scratch; k++) p.scratch[si].push_back(take(si));
        for (int sl : p.scratch[si]) {
            slots[sl].busy = false;
            slots[sl].releasers = {si};
        }
        for (int k = 0; k < s.num_in; k++) {
            int b = s.in_bufs[k];
            bool first = true;
            for (int q = 0; q < k; q++) first &= s.in_bufs[q] != b;
            if (!first || m->buffers[b].kind != KUN_BUF_TEMP || p.temp_slot[b] < 0) continue;
            if (--remaining[b] == 0) {
                slots[p.temp_slot[b]].busy = false;
                slots[p.temp_slot[b]].releasers = consumers[b];
            }
        }
        for (int k = 0; k < s.num_out; k++) {
            int b = s.out_bufs[k];
            if (m->buffers[b].kind == KUN_BUF_TEMP && consumers[b].empty()) {
                slots[p.temp_slot[b]].busy = false;
                slots[p.temp_slot[b]].releasers = {si};
            }
        }
    }
    p.num_slots = (int)slots.size();
    // streams: continue a predecessor's chain when it is that stream's tail,
    // otherwise take the stream with the least work queued
    p.num_streams = std::max(1, nstreams);
    p.stream_of.assign(ns, 0);
    std::vector<int> tail(p.num_streams, -1), load(p.num_streams, 0);
    for (int si : p.order) {
        int pick = -1;
        for (int d : p.preds[si])
            for (int k = 0; k < p.num_streams; k++)
                if (tail[k] == d) pick = k;
        if (pick < 0) pick = (int)(std::min_element(load.begin(), load.end()) - load.begin());
        p.stream_of[si] = pick;
        tail[pick] = si;
        load[pick] += m->stages[si].num_kernels > 0 ? m->stages[si].num_kernels : 1;
    }
    return true;
}

static bool is_device_pointer(const void *ptr) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, ptr) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

static size_t user_buffer_elems(const KunGpuModuleDesc *m, const KunGpuBufferDesc &b, long long S,
                                long long total_time, long long length) {
    bool input = b.kind == KUN_BUF_INPUT;
    long long rows = input ? total_time : length;
    int layout = input ? m->input_layout : m->output_layout;
    long long cols = S;
    if (layout == KUN_LAYOUT_STS) cols = (S + m->blocking_len - 1) / m->blocking_len * m->blocking_len;
    if (input && !strncmp(b.name, "__init", 6)) rows = 1;
    return (size_t)rows * (size_t)cols;
}

static void ensure_events(std::vector<cudaEvent_t> &v, size_t n, unsigned flags) {
    while (v.size() < n) {
        cudaEvent_t e;
        cudaEventCreateWithFlags(&e, flags);
        v.push_back(e);
    }
}

// Enqueue all stages.  Single stream: in plan order.  Several streams: each
// stage on its assigned stream after its predecessors' completion events.
// Device-to-host copies of host output buffers, issued on copy streams as
// soon as the stage producing each buffer has finished, so the copies of
// early outputs overlap the kernels of later stages.
struct OutputCopies {
    struct Item {
        void *host;
        const void *dev;
        size_t bytes;
    };
    std::vector<std::vector<Item>> by_stage;  // stage -> outputs it produces
    int next = 0;
};

static void issue_stage_copies(Executor *ex, OutputCopies &oc, int si, cudaStream_t st) {
    auto &items = oc.by_stage[si];
    if (items.empty()) return;
    cudaEvent_t ev = ex->copy_ev[si];
    cudaEventRecord(ev, st);
    for (auto &it : items) {
        cudaStream_t cs = ex->copy_streams[oc.next++ % ex->copy_streams.size()];
        cudaStreamWaitEvent(cs, ev, 0);
        cudaMemcpyAsync(it.host, it.dev, it.bytes, cudaMemcpyDeviceToHost, cs);
    }
}

static KunStatus enqueue_stages(Executor *ex, const KunGpuModuleDesc *m, const Plan &plan, void **ptrs,
                                long long S, long long total_time, long long cur_time, long long length,
                                cudaStream_t origin, bool multi, int64_t &launches, OutputCopies *oc = nullptr) {
    std::vector<void *> scratch;
    int ev_idx = 0;
    if (ex->profile) {
        ensure_events(ex->ev, plan.order.size() + 1, cudaEventDefault);
        ex->ev_stage.assign(plan.order.begin(), plan.order.end());
        cudaEventRecord(ex->ev[0], origin);
    }
    if (multi) {
        ensure_events(ex->done, m->num_stages, cudaEventDisableTiming);
        if (!ex->fork) cudaEventCreateWithFlags(&ex->fork, cudaEventDisableTiming);
        cudaEventRecord(ex->fork, origin);
        for (int k = 0; k < plan.num_streams; k++)
            if (ex->streams[k] != origin) cudaStreamWaitEvent(ex->streams[k], ex->fork, 0);
    }
    std::vector<int> last_on(plan.num_streams, -1);
    for (int si : plan.order) {
        const KunGpuStageDesc &s = m->stages[si];
        cudaStream_t st = origin;
        if (multi) {
            int k = plan.stream_of[si];
            st = (k == 0) ? origin : ex->streams[k];
            for (int d : plan.preds[si])
                if (plan.stream_of[d] != k) cudaStreamWaitEvent(st, ex->done[d], 0);
        }
        scratch.clear();
        for (int sl : plan.scratch[si]) scratch.push_back((char *)ex->arena.ptr + plan.slot_bytes * (size_t)sl);
        KunGpuStageArgs a;
        memset(&a, 0, sizeof a);
        a.buffers = ptrs;
        a.scratch = scratch.data();
        a.num_stocks = S;
        a.total_time = total_time;
        a.start = cur_time;
        a.length = length;
        a.error_flag = ex->d_error;
        auto tn = ex->tuning.find((const void *)m);
        if (tn != ex->tuning.end() && si < (int)tn->second.size() && !tn->second[si].tile.empty()) {
            a.tune_tile = tn->second[si].tile.data();
            a.tune_block = tn->second[si].block.data();
        }
        int rc = s.launch(&a, (void *)st);
        launches += s.num_kernels > 0 ? s.num_kernels : 1;
        if (rc != 0) {
            set_error("stage %d (%s) launch failed: %s", si, s.name, cudaGetErrorString((cudaError_t)rc));
            return KUN_CUDA_ERROR;
        }
        if (ex->profile) cudaEventRecord(ex->ev[++ev_idx], st);
        if (oc) issue_stage_copies(ex, *oc, si, st);
        if (multi) {
            cudaEventRecord(ex->done[si], st);
            last_on[plan.stream_of[si]] = si;
        }
    }
    if (multi)
        for (int k = 1; k < plan.num_streams; k++)
            if (last_on[k] >= 0) cudaStreamWaitEvent(origin, ex->done[last_on[k]], 0);
    return KUN_SUCCESS;
}

static std::atomic<uint64_t> g_library_epoch{0};
uint64_t library_epoch() { return g_library_epoch.load(); }

void Executor::check_epoch() {
    uint64_t e = library_epoch();
    if (e == epoch) return;
    for (auto &s : streams) cudaStreamSynchronize(s);
    for (auto &g : graphs) cudaGraphExecDestroy(g.exec);
    graphs.clear();
    seen.clear();
    plans.clear();
    tuning.clear();
    epoch = e;
}

KunStatus run_graph(Executor *ex, const KunGpuModuleDesc *m, const NameMap &names, long long S,
                    long long total_time, long long cur_time, long long length, bool sync) {
    clear_error();
    if (!ex || !m) {
        set_error("null executor or module");
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
    if (S <= 0 || length <= 0 || cur_time < 0 || cur_time + length > total_time) {
        set_error("Bad parameter: num_stocks=%lld total_time=%lld cur_time=%lld length=%lld", S, total_time,
                  cur_time, length);
        return KUN_INVALID_ARGUMENT;
    }
    if (m->aligned && m->input_layout == KUN_LAYOUT_TS && (S % m->blocking_len) != 0) {
        // the reference rejects unaligned stock counts for aligned modules
        // (cpp/Python/PyBinding.cpp:322-327)
        set_error("Bad shape: num_stocks %lld is not a multiple of %d", S, m->blocking_len);
        return KUN_INVALID_ARGUMENT;
    }
    std::lock_guard<std::mutex> lk(ex->mu);
    cudaSetDevice(ex->device);
    ex->check_epoch();
    bool multi = ex->streams.size() > 1 && !ex->profile;
    int nstreams = multi ? (int)ex->streams.size() : 1;
    auto key = std::make_tuple((const void *)m, S, length, nstreams);
    auto it = ex->plans.find(key);
    if (it == ex->plans.end()) {
        Plan p;
        if (!make_plan(m, S, length, nstreams, p)) return KUN_INVALID_ARGUMENT;
        it = ex->plans.emplace(key, std::move(p)).first;
    }
    const Plan &plan = it->second;
    size_t elem = m->dtype == 0 ? 4 : 8;
    if (!ex->arena.ensure(plan.slot_bytes * (size_t)plan.num_slots)) {
        set_error("out of device memory for %d temporaries of %zu bytes", plan.num_slots, plan.slot_bytes);
        return KUN_OUT_OF_MEMORY;
    }
    cudaStream_t st = ex->stream();
    if (ex->has_user_stream) {
        cudaEventRecord(ex->bridge_in, ex->user_stream);
        cudaStreamWaitEvent(st, ex->bridge_in, 0);
    }
    // resolve user buffers; stage host ones
    std::vector<void *> ptrs(m->num_buffers, nullptr);
    struct HostCopy {
        int buf;
        void *host;
        size_t bytes;
        size_t off;
    };
    std::vector<HostCopy> host_in, host_out;
    size_t staging_need = 0;
    for (int b = 0; b < m->num_buffers; b++) {
        const KunGpuBufferDesc &bd = m->buffers[b];
        if (bd.kind == KUN_BUF_TEMP) {
            if (plan.temp_slot[b] >= 0)
                ptrs[b] = (char *)ex->arena.ptr + plan.slot_bytes * (size_t)plan.temp_slot[b];
            continue;
        }
        auto f = names.find(bd.name);
        if (f == names.end() || !f->second) {
            set_error("Buffer name not found: %s", bd.name);
            return KUN_INVALID_ARGUMENT;
        }
        if (is_device_pointer(f->second)) {
            ptrs[b] = f->second;
        } else {
            size_t bytes = user_buffer_elems(m, bd, S, total_time, length) * elem;
            HostCopy hc{b, f->second, bytes, staging_need};
            staging_need += align_up(bytes, 256);
            (bd.kind == KUN_BUF_INPUT ? host_in : host_out).push_back(hc);
        }
    }
    if (staging_need) {
        if (!ex->staging.ensure(staging_need)) {
            set_error("out of device memory for %zu staging bytes", staging_need);
            return KUN_OUT_OF_MEMORY;
        }
        for (auto &hc : host_in) {
            ptrs[hc.buf] = (char *)ex->staging.ptr + hc.off;
            cudaMemcpyAsync(ptrs[hc.buf], hc.host, hc.bytes, cudaMemcpyHostToDevice, st);
        }
        for (auto &hc : host_out) ptrs[hc.buf] = (char *)ex->staging.ptr + hc.off;
    }
    int64_t launches = 0;
    // graph key: module, shape and every device address the kernels see
    std::vector<void *> gkey(ptrs.begin(), ptrs.end());
    gkey.push_back((void *)m);
    gkey.push_back((void *)(intptr_t)S);
    gkey.push_back((void *)(intptr_t)total_time);
    gkey.push_back((void *)(intptr_t)cur_time);
    gkey.push_back((void *)(intptr_t)length);
    gkey.push_back(ex->arena.ptr);
    gkey.push_back((void *)(intptr_t)nstreams);
    KunStatus rs = KUN_SUCCESS;
    GraphEntry *ge = nullptr;
    // host outputs: copy each one out as soon as its stage is done (no graph
    // replay for such runs; the copies are not part of the captured work)
    OutputCopies oc;
    bool overlap = !host_out.empty() && !ex->profile;
    if (overlap) {
        if (ex->copy_streams.empty()) {
            for (int k = 0; k < 4; k++) {
                cudaStream_t cs;
                if (cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) != cudaSuccess) break;
                ex->copy_streams.push_back(cs);
            }
            if (ex->copy_streams.empty()) {
                cudaGetLastError();
                overlap = false;
            }
        }
    }
    if (overlap) {
        ensure_events(ex->copy_ev, m->num_stages, cudaEventDisableTiming);
        ensure_events(ex->copy_done, ex->copy_streams.size(), cudaEventDisableTiming);
        oc.by_stage.assign(m->num_stages, {});
        std::vector<int> producer(m->num_buffers, -1);
        for (int si = 0; si < m->num_stages; si++)
            for (int k = 0; k < m->stages[si].num_out; k++) producer[m->stages[si].out_bufs[k]] = si;
        for (auto &hc : host_out) {
            if (producer[hc.buf] < 0) {
                overlap = false;
                break;
            }
            oc.by_stage[producer[hc.buf]].push_back({hc.host, ptrs[hc.buf], hc.bytes});
        }
    }
    if (overlap) {
        rs = enqueue_stages(ex, m, plan, ptrs.data(), S, total_time, cur_time, length, st, multi, launches, &oc);
        if (rs != KUN_SUCCESS) return rs;
        for (size_t k = 0; k < ex->copy_streams.size(); k++) {
            cudaEventRecord(ex->copy_done[k], ex->copy_streams[k]);
            cudaStreamWaitEvent(st, ex->copy_done[k], 0);
        }
        host_out.clear();
    } else if (ex->use_graphs && !ex->profile) {
        for (auto &g : ex->graphs)
            if (g.key == gkey) ge = &g;
        if (!ge && ++ex->seen[gkey] >= 2) {
            // second run with these buffers: capture it once
            cudaStreamCaptureStatus cs;
            cudaStreamIsCapturing(st, &cs);
            if (cs == cudaStreamCaptureStatusNone &&
                cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
                int64_t l2 = 0;
                rs = enqueue_stages(ex, m, plan, ptrs.data(), S, total_time, cur_time, length, st, multi, l2);
                cudaGraph_t g = nullptr;
                cudaError_t e = cudaStreamEndCapture(st, &g);
                cudaGraphExec_t exec = nullptr;
                if (rs == KUN_SUCCESS && e == cudaSuccess && g &&
                    cudaGraphInstantiate(&exec, g, 0) == cudaSuccess) {
                    GraphEntry ent;
                    ent.key = gkey;
                    ent.exec = exec;
                    ent.launches = l2;
                    if (ex->graphs.size() >= 16) {
                        cudaGraphExecDestroy(ex->graphs.front().exec);
                        ex->graphs.erase(ex->graphs.begin());
                    }
                    ex->graphs.push_back(ent);
                    ge = &ex->graphs.back();
                } else {
                    cudaGetLastError();
                }
                if (g) cudaGraphDestroy(g);
                if (rs != KUN_SUCCESS) return rs;
            }
        }
    }
    if (overlap) {
        // stages and copies are enqueued
    } else if (ge) {
        cudaError_t e = cudaGraphLaunch(ge->exec, st);
        if (e != cudaSuccess) {
            set_error("graph launch failed: %s", cudaGetErrorString(e));
            return KUN_CUDA_ERROR;
        }
        launches = ge->launches;
    } else {
        rs = enqueue_stages(ex, m, plan, ptrs.data(), S, total_time, cur_time, length, st, multi, launches);
        if (rs != KUN_SUCCESS) return rs;
    }
    ex->last_launches = launches;
    bool had_host_out = overlap || !host_out.empty();
    for (auto &hc : host_out) cudaMemcpyAsync(hc.host, ptrs[hc.buf], hc.bytes, cudaMemcpyDeviceToHost, st);
    if (ex->has_user_stream) {
        cudaEventRecord(ex->bridge_out, st);
        cudaStreamWaitEvent(ex->user_stream, ex->bridge_out, 0);
    }
    if (sync || !host_in.empty() || had_host_out) {
        cudaError_t e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) {
            set_error("CUDA error: %s", cudaGetErrorString(e));
            return KUN_CUDA_ERROR;
        }
        if (ex->d_error) {
            // a kernel whose bounded wait for a bulk copy ran out (never
            // expected: a hardware or launch-setup fault) reports it here
            int32_t flag = 0;
            cudaMemcpy(&flag, ex->d_error, sizeof flag, cudaMemcpyDeviceToHost);
            if (flag) {
                cudaMemset(ex->d_error, 0, sizeof(int32_t));
                set_error("a staged (bulk-copy) kernel timed out waiting for its copies; outputs are not valid");
                return KUN_CUDA_ERROR;
            }
        }
    }
    return KUN_SUCCESS;
}

Executor *create_executor(int nstreams) {
    auto *ex = new Executor();
    cudaGetDevice(&ex->device);
    if (nstreams < 1) nstreams = 1;
    for (int i = 0; i < nstreams; i++) {
        cudaStream_t s;
        if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) {
            set_error("cannot create a CUDA stream: %s", cudaGetErrorString(cudaGetLastError()));
            for (auto x : ex->streams) cudaStreamDestroy(x);
            delete ex;
            return nullptr;
        }
        ex->streams.push_back(s);
    }
    ex->epoch = library_epoch();
    if (cudaMalloc(&ex->d_error, sizeof(int32_t)) == cudaSuccess)
        cudaMemset(ex->d_error, 0, sizeof(int32_t));
    else
        cudaGetLastError();
    return ex;
}

void destroy_executor(Executor *ex) {
    if (!ex) return;
    for (auto s : ex->streams) {
        cudaStreamSynchronize(s);
        cudaStreamDestroy(s);
    }
    for (auto &g : ex->graphs) cudaGraphExecDestroy(g.exec);
    for (auto e : ex->ev) cudaEventDestroy(e);
    for (auto e : ex->done) cudaEventDestroy(e);
    if (ex->fork) cudaEventDestroy(ex->fork);
    if (ex->bridge_in) cudaEventDestroy(ex->bridge_in);
    if (ex->bridge_out) cudaEventDestroy(ex->bridge_out);
    if (ex->d_error) cudaFree(ex->d_error);
    for (auto cs : ex->copy_streams) {
        cudaStreamSynchronize(cs);
        cudaStreamDestroy(cs);
    }
    if (ex->group_host) cudaFreeHost(ex->group_host);
    for (auto e : ex->copy_ev) cudaEventDestroy(e);
    for (auto e : ex->copy_done) cudaEventDestroy(e);
    delete ex;
}

}  // namespace kungpu

using namespace kungpu;

static const KunGpuModuleDesc *M(KunModuleHandle m) { return (const KunGpuModuleDesc *)m; }

KUN_EXPORT KunExecutorHandle kunCreateSingleThreadExecutor(void) { return create_executor(1); }
KUN_EXPORT KunExecutorHandle kunCreateMultiThreadExecutor(int numthreads) { return create_executor(numthreads); }
KUN_EXPORT void kunDestoryExecutor(KunExecutorHandle ptr) { destroy_executor((Executor *)ptr); }

KUN_EXPORT KunLibraryHandle kunLoadLibrary(const char *path_or_name) {
    clear_error();
    void *h = dlopen(path_or_name, RTLD_LOCAL | RTLD_NOW);
    if (!h) {
        set_error("Cannot load library: %s", dlerror());
        return nullptr;
    }
    auto *lib = new Library();
    lib->handle = h;
    lib->path = path_or_name;
    return lib;
}

KUN_EXPORT KunModuleHandle kunGetModuleFromLibrary(KunLibraryHandle lib, const char *name) {
    clear_error();
    if (!lib || !name) return nullptr;
    std::string sym = std::string("kun_module_") + name;
    auto *m = (const KunGpuModuleDesc *)dlsym(((Library *)lib)->handle, sym.c_str());
    if (!m) {
        set_error("Module name not found: %s", name);
        return nullptr;
    }
    if (m->abi != KUN_GPU_MODULE_ABI) {
        set_error("The required version in the module does not match the runtime version");
        return nullptr;
    }
    return (KunModuleHandle)m;
}

KUN_EXPORT void kunUnloadLibrary(KunLibraryHandle ptr) {
    auto *lib = (Library *)ptr;
    if (!lib) return;
    if (lib->handle) dlclose(lib->handle);
    delete lib;
    g_library_epoch.fetch_add(1);
}

KUN_EXPORT KunBufferNameMapHandle kunCreateBufferNameMap(void) { return new NameMap(); }
KUN_EXPORT void kunDestoryBufferNameMap(KunBufferNameMapHandle ptr) { delete (NameMap *)ptr; }
KUN_EXPORT void kunSetBufferNameMap(KunBufferNameMapHandle ptr, const char *name, float *buffer) {
    (*(NameMap *)ptr)[name] = buffer;
}
KUN_EXPORT void kunEraseBufferNameMap(KunBufferNameMapHandle ptr, const char *name) {
    ((NameMap *)ptr)->erase(name);
}

KUN_EXPORT KunStatus kunRunGraphEx(KunExecutorHandle exec, KunModuleHandle m, KunBufferNameMapHandle buffers,
                                   size_t num_stocks, size_t total_time, size_t cur_time, size_t length,
                                   int synchronize) {
    if (!buffers) {
        set_error("null buffer map");
        return KUN_INVALID_ARGUMENT;
    }
    return run_graph((Executor *)exec, M(m), *(NameMap *)buffers, (long long)num_stocks, (long long)total_time,
                     (long long)cur_time, (long long)length, synchronize != 0);
}

KUN_EXPORT void kunRunGraph(KunExecutorHandle exec, KunModuleHandle m, KunBufferNameMapHandle buffers,
                            size_t num_stocks, size_t total_time, size_t cur_time, size_t length) {
    kunRunGraphEx(exec, m, buffers, num_stocks, total_time, cur_time, length, 1);
}

KUN_EXPORT KunStatus kunExecutorSetStream(KunExecutorHandle exec, void *cuda_stream) {
    auto *ex = (Executor *)exec;
    if (!ex) return KUN_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(ex->mu);
    if (!ex->bridge_in) {
        cudaEventCreateWithFlags(&ex->bridge_in, cudaEventDisableTiming);
        cudaEventCreateWithFlags(&ex->bridge_out, cudaEventDisableTiming);
    }
    ex->user_stream = (cudaStream_t)cuda_stream;
    ex->has_user_stream = true;
    return KUN_SUCCESS;
}

// Stop ordering with a caller's stream.
KUN_EXPORT KunStatus kunExecutorClearStream(KunExecutorHandle exec) {
    auto *ex = (Executor *)exec;
    if (!ex) return KUN_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(ex->mu);
    ex->has_user_stream = false;
    ex->user_stream = nullptr;
    return KUN_SUCCESS;
}

KUN_EXPORT KunStatus kunExecutorSynchronize(KunExecutorHandle exec) {
    auto *ex = (Executor *)exec;
    if (!ex) return KUN_INVALID_ARGUMENT;
    cudaError_t e = cudaStreamSynchronize(ex->stream());
    if (e != cudaSuccess) {
        set_error("CUDA error: %s", cudaGetErrorString(e));
        return KUN_CUDA_ERROR;
    }
    return KUN_SUCCESS;
}

// Capture repeated runs into CUDA graphs (default on).
KUN_EXPORT KunStatus kunExecutorSetGraphs(KunExecutorHandle exec, int enable) {
    auto *ex = (Executor *)exec;
    if (!ex) return KUN_INVALID_ARGUMENT;
    ex->use_graphs = enable != 0;
    return KUN_SUCCESS;
}

KUN_EXPORT int64_t kunExecutorLastLaunchCount(KunExecutorHandle exec) {
    auto *ex = (Executor *)exec;
    return ex ? ex->last_launches : -1;
}

KUN_EXPORT const char *kunGetLastError(void) { return last_error(); }

// Per-stage timing (GPU extension used by the benchmark): when enabled, every
// run records a CUDA event after each stage launch on the executor's stream.
KUN_EXPORT KunStatus kunExecutorSetProfiling(KunExecutorHandle exec, int enable) {
    auto *ex = (Executor *)exec;
    if (!ex) return KUN_INVALID_ARGUMENT;
    ex->profile = enable != 0;
    return KUN_SUCCESS;
}

// Milliseconds of each stage of the last profiled run, by stage id; returns
// the number of stages written.
KUN_EXPORT int kunExecutorStageTimes(KunExecutorHandle exec, int32_t *stage_ids, float *ms, int cap) {
    auto *ex = (Executor *)exec;
    if (!ex || !ex->profile) return -1;
    cudaStreamSynchronize(ex->stream());
    int n = std::min((int)ex->ev_stage.size(), cap);
    for (int i = 0; i < n; i++) {
        float t = 0;
        cudaEventElapsedTime(&t, ex->ev[i], ex->ev[i + 1]);
        stage_ids[i] = ex->ev_stage[i];
        ms[i] = t;
    }
    return n;
}

KUN_EXPORT int kunModuleNumBuffers(KunModuleHandle m) { return M(m)->num_buffers; }
KUN_EXPORT const char *kunModuleBufferName(KunModuleHandle m, int idx) { return M(m)->buffers[idx].name; }
KUN_EXPORT int kunModuleBufferKind(KunModuleHandle m, int idx) { return M(m)->buffers[idx].kind; }
KUN_EXPORT int kunModuleBufferUnreliableCount(KunModuleHandle m, int idx) {
    return M(m)->buffers[idx].unreliable_count;
}
KUN_EXPORT int kunModuleBufferWindow(KunModuleHandle m, int idx) { return M(m)->buffers[idx].window; }
KUN_EXPORT int kunModuleInputLayout(KunModuleHandle m) { return M(m)->input_layout; }
KUN_EXPORT int kunModuleOutputLayout(KunModuleHandle m) { return M(m)->output_layout; }
KUN_EXPORT int kunModuleBlockingLen(KunModuleHandle m) { return M(m)->blocking_len; }
KUN_EXPORT int kunModuleDtype(KunModuleHandle m) { return M(m)->dtype; }
KUN_EXPORT int kunModuleNumStages(KunModuleHandle m) { return M(m)->num_stages; }

