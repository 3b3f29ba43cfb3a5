// libkungpu.so: the runtime behind the C ABI of include/kun_gpu.h.
//
// Batch execution (replaces cpp/Kun/Runtime.cpp:311-352 + Executor.cpp): the
// stage DAG of a module is ordered once; temporaries between stages live in a
// device arena whose slots are reused by liveness (a temp's slot is released
// after its last consumer, like the reference frees on last deref,
// Runtime.cpp:84-93), and the stage kernels are enqueued on the executor's
// CUDA stream.  Host buffers are staged to the device inside the call.
#include <cuda_runtime.h>
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

#include "kun_gpu.h"
#include "kun_module_abi.h"

#define KUN_EXPORT extern "C" __attribute__((visibility("default")))

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
    std::vector<int> order;                 // stage ids in launch order
    std::vector<int> temp_slot;             // per buffer: arena slot or -1
    std::vector<std::vector<int>> scratch;  // per stage: slots of its scratch
    int num_slots = 0;
    size_t slot_bytes = 0;
};

struct Executor {
    int device = 0;
    std::vector<cudaStream_t> streams;
    cudaStream_t user_stream = nullptr;
    Arena arena;
    Arena staging;
    int32_t *d_error = nullptr;
    int64_t last_launches = 0;
    std::map<std::tuple<const void *, long long, long long>, Plan> plans;
    std::mutex mu;
    // optional per-stage timing (CUDA events around every launch)
    bool profile = false;
    std::vector<cudaEvent_t> ev;
    std::vector<int> ev_stage;
    cudaStream_t stream() const { return user_stream ? user_stream : streams[0]; }
};

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

// Liveness-based slot assignment of temporaries and stage scratch.
static bool make_plan(const KunGpuModuleDesc *m, long long S, long long length, Plan &p) {
    if (!topo_order(m, p.order)) {
        set_error("module %s: cyclic stage graph", m->name);
        return false;
    }
    size_t elem = m->dtype == 0 ? 4 : 8;
    p.slot_bytes = align_up((size_t)S * (size_t)length * elem, 256);
    int nb = m->num_buffers;
    std::vector<int> last_use(nb, -1), producer_pos(nb, -1);
    for (int pos = 0; pos < (int)p.order.size(); pos++) {
        const KunGpuStageDesc &s = m->stages[p.order[pos]];
        for (int k = 0; k < s.num_in; k++) last_use[s.in_bufs[k]] = pos;
        for (int k = 0; k < s.num_out; k++) producer_pos[s.out_bufs[k]] = pos;
    }
    p.temp_slot.assign(nb, -1);
    p.scratch.assign(m->num_stages, {});
    std::vector<int> free_slots;
    int next = 0;
    auto take = [&]() {
        if (!free_slots.empty()) {
            int s = free_slots.back();
            free_slots.pop_back();
            return s;
        }
        return next++;
    };
    for (int pos = 0; pos < (int)p.order.size(); pos++) {
        int si = p.order[pos];
        const KunGpuStageDesc &s = m->stages[si];
        for (int k = 0; k < s.num_out; k++) {
            int b = s.out_bufs[k];
            if (m->buffers[b].kind == KUN_BUF_TEMP) p.temp_slot[b] = take();
        }
        for (int k = 0; k < s.num_scratch; k++) p.scratch[si].push_back(take());
        // release scratch and temps whose last consumer is this stage
        for (int sl : p.scratch[si]) free_slots.push_back(sl);
        for (int k = 0; k < s.num_in; k++) {
            int b = s.in_bufs[k];
            if (m->buffers[b].kind == KUN_BUF_TEMP && last_use[b] == pos && p.temp_slot[b] >= 0) {
                bool dup = false;
                for (int q = 0; q < k; q++) dup |= s.in_bufs[q] == b;
                if (!dup) free_slots.push_back(p.temp_slot[b]);
            }
        }
        // a temp nobody reads is dead right away
        for (int k = 0; k < s.num_out; k++) {
            int b = s.out_bufs[k];
            if (m->buffers[b].kind == KUN_BUF_TEMP && last_use[b] < 0) free_slots.push_back(p.temp_slot[b]);
        }
    }
    p.num_slots = next;
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

using NameMap = std::unordered_map<std::string, float *>;

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
    auto key = std::make_tuple((const void *)m, S, length);
    auto it = ex->plans.find(key);
    if (it == ex->plans.end()) {
        Plan p;
        if (!make_plan(m, S, length, p)) return KUN_INVALID_ARGUMENT;
        it = ex->plans.emplace(key, std::move(p)).first;
    }
    const Plan &plan = it->second;
    size_t elem = m->dtype == 0 ? 4 : 8;
    if (!ex->arena.ensure(plan.slot_bytes * (size_t)plan.num_slots)) {
        set_error("out of device memory for %d temporaries of %zu bytes", plan.num_slots, plan.slot_bytes);
        return KUN_OUT_OF_MEMORY;
    }
    cudaStream_t st = ex->stream();
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
    std::vector<void *> scratch;
    if (ex->profile) {
        while (ex->ev.size() < plan.order.size() + 1) {
            cudaEvent_t e;
            cudaEventCreate(&e);
            ex->ev.push_back(e);
        }
        ex->ev_stage.assign(plan.order.begin(), plan.order.end());
        cudaEventRecord(ex->ev[0], st);
    }
    for (int si : plan.order) {
        const KunGpuStageDesc &s = m->stages[si];
        scratch.clear();
        for (int sl : plan.scratch[si]) scratch.push_back((char *)ex->arena.ptr + plan.slot_bytes * (size_t)sl);
        KunGpuStageArgs a;
        memset(&a, 0, sizeof a);
        a.buffers = ptrs.data();
        a.scratch = scratch.data();
        a.num_stocks = S;
        a.total_time = total_time;
        a.start = cur_time;
        a.length = length;
        a.error_flag = ex->d_error;
        int rc = s.launch(&a, (void *)st);
        launches++;
        if (ex->profile) cudaEventRecord(ex->ev[launches], st);
        if (rc != 0) {
            set_error("stage %d (%s) launch failed: %s", si, s.name, cudaGetErrorString((cudaError_t)rc));
            return KUN_CUDA_ERROR;
        }
    }
    ex->last_launches = launches;
    for (auto &hc : host_out) cudaMemcpyAsync(hc.host, ptrs[hc.buf], hc.bytes, cudaMemcpyDeviceToHost, st);
    if (sync || !host_in.empty() || !host_out.empty()) {
        cudaError_t e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) {
            set_error("CUDA error: %s", cudaGetErrorString(e));
            return KUN_CUDA_ERROR;
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
    if (cudaMalloc(&ex->d_error, sizeof(int32_t)) == cudaSuccess) cudaMemset(ex->d_error, 0, sizeof(int32_t));
    else cudaGetLastError();
    return ex;
}

void destroy_executor(Executor *ex) {
    if (!ex) return;
    for (auto s : ex->streams) {
        cudaStreamSynchronize(s);
        cudaStreamDestroy(s);
    }
    if (ex->d_error) cudaFree(ex->d_error);
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
    ex->user_stream = (cudaStream_t)cuda_stream;
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

// ---------------- stream API (filled in by kun_stream.cu when built) -------
#ifndef KUN_HAVE_STREAM
KUN_EXPORT KunStreamContextHandle kunCreateStream(KunExecutorHandle, KunModuleHandle, size_t) {
    set_error("stream mode is not built");
    return nullptr;
}
KUN_EXPORT KunStatus kunCreateStreamEx(KunExecutorHandle, KunModuleHandle, size_t, const KunStreamExtraArgs *,
                                       KunStreamContextHandle *out) {
    if (out) *out = nullptr;
    set_error("stream mode is not built");
    return KUN_INIT_ERROR;
}
KUN_EXPORT KunStatus kunStreamSerializeStates(KunStreamContextHandle, KunStateBufferKind, char *, size_t *) {
    return KUN_INVALID_ARGUMENT;
}
KUN_EXPORT size_t kunQueryBufferHandle(KunStreamContextHandle, const char *) { return (size_t)-1; }
KUN_EXPORT const float *kunStreamGetCurrentBuffer(KunStreamContextHandle, size_t) { return nullptr; }
KUN_EXPORT void kunStreamPushData(KunStreamContextHandle, size_t, const float *) {}
KUN_EXPORT void kunStreamRun(KunStreamContextHandle) {}
KUN_EXPORT void kunDestoryStream(KunStreamContextHandle) {}
KUN_EXPORT KunStatus kunStreamPushDataDevice(KunStreamContextHandle, size_t, const void *) {
    return KUN_INVALID_ARGUMENT;
}
KUN_EXPORT const void *kunStreamGetCurrentBufferDevice(KunStreamContextHandle, size_t) { return nullptr; }
KUN_EXPORT KunStatus kunStreamRunEx(KunStreamContextHandle, int) { return KUN_INVALID_ARGUMENT; }
#endif
