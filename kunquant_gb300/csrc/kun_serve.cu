// Serving pool: many stream sessions of one stream module sharing one device
// store, advanced together.
//
// The reference runs one StreamContext per session (cpp/Kun/Runtime.cpp:
// 424-546), each a separate set of host rings.  Here a pool owns one
// StreamStore of `capacity` stock columns; a session holds a contiguous range
// of columns (first fit) for its whole life, so its ring and op state stay
// resident on the device between ticks.  A step advances any subset of the
// sessions by one tick each:
//   host: one copy of the segment table and of the sessions' input columns,
//   graph: scatter inputs into the rings -> every stage's tick kernel over the
//          batch of segments -> gather the output rows,
//   host: one copy of the sessions' output columns.
// The kernels read the batch's counts from the device table, so one captured
// graph per (stocks, sessions) size bucket serves every step.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "kun_runtime_internal.h"
#include "kun_xsec.cuh"

namespace kungpu {

// session k of the step: active stocks [off[k], off[k+1]) live in columns
// stock0[k] + (i - off[k])
__device__ __forceinline__ int serve_segment(const int32_t *off, int nseg, long long i) {
    int lo = 0, hi = nseg - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (off[mid] <= i) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// input table [nin][cap] -> ring row (tick % window) of each active column
template <typename T>
__global__ void serve_scatter(const T *__restrict__ cols, T *const *rings, const int32_t *wins,
                              const int32_t *off, const int32_t *stock0, const long long *tick,
                              const int32_t *cnt, long long cap) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int nseg = cnt[0];
    const long long n = cnt[1];
    if (i >= n) return;
    const int b = blockIdx.y;
    const int k = serve_segment(off, nseg, i);
    const long long s = stock0[k] + (i - off[k]);
    const long long row = tick[k] % wins[b];
    rings[b][row * cap + s] = cols[(long long)b * cap + s];
}

// ring row (tick % window) of each active column -> output table [nout][cap]
template <typename T>
__global__ void serve_gather(T *__restrict__ cols, T *const *rings, const int32_t *wins, const int32_t *off,
                             const int32_t *stock0, const long long *tick, const int32_t *cnt, long long cap) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int nseg = cnt[0];
    const long long n = cnt[1];
    if (i >= n) return;
    const int b = blockIdx.y;
    const int k = serve_segment(off, nseg, i);
    const long long s = stock0[k] + (i - off[k]);
    const long long row = tick[k] % wins[b];
    cols[(long long)b * cap + s] = rings[b][row * cap + s];
}

struct Session {
    long long stock0 = 0, len = 0;
    long long tick = 0;        // ticks completed
    bool pending = false;      // a tick is submitted or on the device
    uint64_t stamp = 0;        // last step that took it (duplicate check)
    std::chrono::steady_clock::time_point t_submit;
};

struct ServePool {
    Executor *ex = nullptr;
    const KunGpuModuleDesc *m = nullptr;
    long long cap = 0;
    int max_sessions = 0;
    int max_len = 0;
    StreamStore store;
    std::vector<int> order;
    std::vector<int> in_bufs, out_bufs;
    // device: segment table {off[max+1], stock0[max], cnt[3]} then ticks,
    // ring pointer/window arrays, input/output tables by column
    char *d_table = nullptr;
    char *h_table = nullptr;  // pinned mirror
    size_t table_bytes = 0, tick_off = 0;
    void **d_in_rings = nullptr, **d_out_rings = nullptr;
    int32_t *d_in_win = nullptr, *d_out_win = nullptr;
    void *d_in = nullptr, *d_out = nullptr;  // [nin][cap], [nout][cap]
    void *h_in = nullptr, *h_out = nullptr;  // pinned mirrors
    std::map<long long, long long> free_cols;  // start -> length
    std::map<int64_t, Session> sessions;
    int64_t next_id = 1;
    uint64_t steps = 0;
    std::map<std::pair<long long, int>, cudaGraphExec_t> graphs;
    TickSchedule sched;            // concurrent stages inside the step graph
    TickLevels levels;             // the step as a chain of stage-graph levels
    std::mutex mu;                 // sessions, columns, queue
    std::mutex gpu_mu;             // one step on the device at a time
    // request loop (continuous batching)
    std::thread loop;
    bool running = false;
    int batch_window_us = 0;
    std::condition_variable cv_ready, cv_done;
    std::vector<int64_t> ready;
    KunStatus failed = KUN_SUCCESS;
    std::string fail_msg;
    std::vector<float> lat_us;     // per completed tick: submit -> done
    std::vector<int> step_sizes;
    cudaStream_t stream() const { return ex->streams[0]; }
    size_t elem() const { return m->dtype == 0 ? 4 : 8; }
    int32_t *off() const { return (int32_t *)d_table; }
    int32_t *stock0() const { return (int32_t *)d_table + (max_sessions + 1); }
    int32_t *cnt() const { return (int32_t *)d_table + (2 * max_sessions + 1); }
    long long *ticks() const { return (long long *)(d_table + tick_off); }
    ~ServePool();
};

static void stop_loop(ServePool *p) {
    {
        std::lock_guard<std::mutex> lk(p->mu);
        if (!p->running) return;
        p->running = false;
    }
    p->cv_ready.notify_all();
    if (p->loop.joinable()) p->loop.join();
    p->cv_done.notify_all();
}

ServePool::~ServePool() {
    stop_loop(this);
    cudaStreamSynchronize(stream());
    for (auto &g : graphs) cudaGraphExecDestroy(g.second);
    free_tick_schedule(sched);
    free_tick_levels(levels);
    void *dev[] = {d_table, d_in_rings, d_out_rings, d_in_win, d_out_win, d_in, d_out};
    for (void *q : dev)
        if (q) cudaFree(q);
    if (h_table) cudaFreeHost(h_table);
    if (h_in) cudaFreeHost(h_in);
    if (h_out) cudaFreeHost(h_out);
    store.release();
}

static constexpr int kStepLimitMs = 20000;
static constexpr int kStepStreams = 8;  // concurrent stage chains inside a step

// graph size buckets: powers of 4 from lo, capped at hi (a step of n uses
// the graph of the first bucket >= n; its kernels take the exact counts
// from the device table)
static long long bucket(long long n, long long lo, long long hi) {
    long long b = lo;
    while (b < n && b < hi) b <<= 2;
    return b < hi ? b : hi;
}

static KunStatus build_serve_graph(ServePool *p, long long nb, int sb, cudaGraphExec_t *out) {
    cudaStream_t st = p->stream();
    if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        set_error("cannot capture the serving graph");
        return KUN_CUDA_ERROR;
    }
    dim3 gin((unsigned)((nb + 255) / 256), (unsigned)p->in_bufs.size());
    dim3 gout((unsigned)((nb + 255) / 256), (unsigned)p->out_bufs.size());
    if (p->elem() == 4)
        serve_scatter<float><<<gin, 256, 0, st>>>((const float *)p->d_in, (float *const *)p->d_in_rings,
                                                  p->d_in_win, p->off(), p->stock0(), p->ticks(), p->cnt(), p->cap);
    else
        serve_scatter<double><<<gin, 256, 0, st>>>((const double *)p->d_in, (double *const *)p->d_in_rings,
                                                   p->d_in_win, p->off(), p->stock0(), p->ticks(), p->cnt(), p->cap);
    KunStatus rs = enqueue_tick(p->store, p->order, p->off(), p->stock0(), (const int64_t *)p->ticks(), sb, nb,
                                p->max_len, st, p->cnt(), &p->sched, &p->levels);
    if (!p->out_bufs.empty()) {
        if (p->elem() == 4)
            serve_gather<float><<<gout, 256, 0, st>>>((float *)p->d_out, (float *const *)p->d_out_rings,
                                                      p->d_out_win, p->off(), p->stock0(), p->ticks(), p->cnt(),
                                                      p->cap);
        else
            serve_gather<double><<<gout, 256, 0, st>>>((double *)p->d_out, (double *const *)p->d_out_rings,
                                                       p->d_out_win, p->off(), p->stock0(), p->ticks(), p->cnt(),
                                                       p->cap);
    }
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(st, &g);
    if (rs != KUN_SUCCESS || e != cudaSuccess || !g) {
        if (g) cudaGraphDestroy(g);
        cudaGetLastError();
        if (rs == KUN_SUCCESS) set_error("serving graph capture failed: %s", cudaGetErrorString(e));
        return rs == KUN_SUCCESS ? KUN_CUDA_ERROR : rs;
    }
    e = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        set_error("serving graph instantiate failed: %s", cudaGetErrorString(e));
        return KUN_CUDA_ERROR;
    }
    return KUN_SUCCESS;
}

// The device part of a step whose table (h_table) is filled: copies, graph,
// copies back, wait.  Holds gpu_mu, not mu.
struct StepShape {
    int nsess = 0;
    long long n = 0, lo = 0, hi = 0;
    // column runs [first, second) of the step's sessions, merged where adjacent
    std::vector<std::pair<long long, long long>> runs;
};

static KunStatus graph_for(ServePool *p, long long nb, int sb, cudaGraphExec_t *out);

// the graph of a (stocks, sessions) bucket, built on first use (gpu_mu held)
static KunStatus graph_for(ServePool *p, long long nb, int sb, cudaGraphExec_t *out) {
    auto key = std::make_pair(nb, sb);
    auto g = p->graphs.find(key);
    if (g == p->graphs.end()) {
        cudaGraphExec_t ge = nullptr;
        KunStatus rs = build_serve_graph(p, nb, sb, &ge);
        if (rs != KUN_SUCCESS) return rs;
        g = p->graphs.emplace(key, ge).first;
    }
    *out = g->second;
    return KUN_SUCCESS;
}

static KunStatus run_step(ServePool *p, const StepShape &sh, const void *dev_in, void *dev_out) {
    std::lock_guard<std::mutex> g_lk(p->gpu_mu);
    cudaStream_t st = p->stream();
    size_t elem = p->elem();
    // the table goes as two copies: ints up to cnt, then the ticks
    cudaMemcpyAsync(p->d_table, p->h_table, (2 * p->max_sessions + 5) * sizeof(int32_t), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(p->d_table + p->tick_off, p->h_table + p->tick_off, sh.nsess * sizeof(long long),
                    cudaMemcpyHostToDevice, st);
    // every input and output row moves as 2D copies: one over the column
    // span [lo, hi) when the step's sessions fill most of it, else one per
    // run of adjacent sessions
    size_t pitch = (size_t)p->cap * elem;
    std::vector<std::pair<long long, long long>> whole{{sh.lo, sh.hi}};
    const auto &runs = (sh.n * 2 >= sh.hi - sh.lo || sh.runs.empty()) ? whole : sh.runs;
    const char *h_in = (const char *)(dev_in ? dev_in : p->h_in);
    for (const auto &r : runs)
        cudaMemcpy2DAsync((char *)p->d_in + (size_t)r.first * elem, pitch, h_in + (size_t)r.first * elem, pitch,
                          (size_t)(r.second - r.first) * elem, p->in_bufs.size(),
                          dev_in ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, st);
    cudaGraphExec_t ge = nullptr;
    KunStatus rs = graph_for(p, bucket(sh.n, 256, p->cap), (int)bucket(sh.nsess, 4, p->max_sessions), &ge);
    if (rs != KUN_SUCCESS) return rs;
    cudaError_t e = cudaGraphLaunch(ge, st);
    if (e != cudaSuccess) {
        set_error("serving step launch failed: %s", cudaGetErrorString(e));
        return KUN_CUDA_ERROR;
    }
    if (!p->out_bufs.empty()) {
        char *h_out = (char *)(dev_out ? dev_out : p->h_out);
        for (const auto &r : runs)
            cudaMemcpy2DAsync(h_out + (size_t)r.first * elem, pitch, (const char *)p->d_out + (size_t)r.first * elem,
                              pitch, (size_t)(r.second - r.first) * elem, p->out_bufs.size(),
                              dev_out ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, st);
    }
    // wait with a limit, so a step that never finishes is reported instead
    // of blocking the loop and every client
    auto t0 = std::chrono::steady_clock::now();
    while ((e = cudaStreamQuery(st)) == cudaErrorNotReady) {
        if (std::chrono::steady_clock::now() - t0 > std::chrono::milliseconds(kStepLimitMs)) {
            set_error("serving step did not finish within %d ms", kStepLimitMs);
            return KUN_TIMEOUT;
        }
        std::this_thread::yield();
    }
    if (e != cudaSuccess) {
        set_error("CUDA error: %s", cudaGetErrorString(e));
        return KUN_CUDA_ERROR;
    }
    return KUN_SUCCESS;
}

// Fill the host table for the sessions `sids` (under mu).
static KunStatus prepare_step(ServePool *p, int nsess, const int64_t *sids, std::vector<Session *> &sel,
                              StepShape &sh) {
    if (nsess > p->max_sessions) {
        set_error("step of %d sessions exceeds the pool's %d", nsess, p->max_sessions);
        return KUN_INVALID_ARGUMENT;
    }
    int32_t *off = (int32_t *)p->h_table;
    int32_t *s0 = off + (p->max_sessions + 1);
    int32_t *cnt = off + (2 * p->max_sessions + 1);
    long long *tk = (long long *)(p->h_table + p->tick_off);
    long long n = 0, lo = p->cap, hi = 0;
    int longest = 0;
    uint64_t stamp = ++p->steps;
    sel.resize(nsess);
    for (int k = 0; k < nsess; k++) {
        auto it = p->sessions.find(sids[k]);
        if (it == p->sessions.end()) {
            set_error("unknown session %lld", (long long)sids[k]);
            return KUN_INVALID_ARGUMENT;
        }
        Session &s = it->second;
        if (s.stamp == stamp) {
            set_error("session %lld appears twice in one step", (long long)sids[k]);
            return KUN_INVALID_ARGUMENT;
        }
        s.stamp = stamp;
        sel[k] = &s;
    }
    // the sessions the small Rank blocks serve come first (cnt[3] of them)
    std::stable_partition(sel.begin(), sel.end(),
                          [](const Session *q) { return q->len <= (long long)kun::kRankSmallMax; });
    int nsmall = 0;
    for (int k = 0; k < nsess; k++) {
        Session &s = *sel[k];
        nsmall += s.len <= (long long)kun::kRankSmallMax;
        off[k] = (int32_t)n;
        s0[k] = (int32_t)s.stock0;
        tk[k] = s.tick;
        n += s.len;
        if (s.len > longest) longest = (int)s.len;
        lo = std::min(lo, s.stock0);
        hi = std::max(hi, s.stock0 + s.len);
    }
    off[nsess] = (int32_t)n;
    // column runs of the selected sessions
    sh.runs.clear();
    {
        std::vector<std::pair<long long, long long>> cols(nsess);
        for (int k = 0; k < nsess; k++) cols[k] = {sel[k]->stock0, sel[k]->stock0 + sel[k]->len};
        std::sort(cols.begin(), cols.end());
        for (const auto &c : cols) {
            if (!sh.runs.empty() && sh.runs.back().second == c.first)
                sh.runs.back().second = c.second;
            else
                sh.runs.push_back(c);
        }
    }
    cnt[0] = nsess;
    cnt[1] = (int32_t)n;
    cnt[2] = longest;
    cnt[3] = nsmall;
    sh.nsess = nsess;
    sh.n = n;
    sh.lo = lo;
    sh.hi = hi;
    return KUN_SUCCESS;
}

static KunStatus pool_step(ServePool *p, int nsess, const int64_t *sids, const void *dev_in, void *dev_out) {
    if (nsess <= 0) return KUN_SUCCESS;
    std::vector<Session *> sel;
    StepShape sh;
    std::unique_lock<std::mutex> lk(p->mu);
    if (p->running) {
        set_error("kunServeStep cannot be used while the request loop runs");
        return KUN_INVALID_ARGUMENT;
    }
    KunStatus rs = prepare_step(p, nsess, sids, sel, sh);
    if (rs != KUN_SUCCESS) return rs;
    rs = run_step(p, sh, dev_in, dev_out);
    if (rs != KUN_SUCCESS) return rs;
    for (auto *s : sel) s->tick++;
    return KUN_SUCCESS;
}

// The request loop: every submitted tick waits for the next step; a step
// takes every session submitted so far (after an optional batching window).
static void serve_loop(ServePool *p) {
    cudaSetDevice(p->ex->device);
    std::unique_lock<std::mutex> lk(p->mu);
    std::vector<int64_t> take;
    std::vector<Session *> sel;
    while (true) {
        p->cv_ready.wait(lk, [&] { return !p->running || !p->ready.empty(); });
        if (!p->running) break;
        if (p->batch_window_us > 0) {
            lk.unlock();
            std::this_thread::sleep_for(std::chrono::microseconds(p->batch_window_us));
            lk.lock();
        }
        take.swap(p->ready);
        p->ready.clear();
        StepShape sh;
        KunStatus rs = prepare_step(p, (int)take.size(), take.data(), sel, sh);
        if (rs == KUN_SUCCESS) {
            lk.unlock();
            rs = run_step(p, sh, nullptr, nullptr);
            lk.lock();
        }
        auto now = std::chrono::steady_clock::now();
        if (rs != KUN_SUCCESS) {
            p->failed = rs;
            p->fail_msg = last_error();
        }
        for (auto *s : sel) {
            if (rs == KUN_SUCCESS) {
                s->tick++;
                p->lat_us.push_back(
                    (float)std::chrono::duration<double, std::micro>(now - s->t_submit).count());
            }
            s->pending = false;
        }
        p->step_sizes.push_back((int)take.size());
        take.clear();
        p->cv_done.notify_all();
    }
}

}  // namespace kungpu

using namespace kungpu;

static ServePool *SP(KunServePoolHandle h) { return (ServePool *)h; }

KUN_EXPORT KunStatus kunCreateServePool(KunExecutorHandle exec, KunModuleHandle mod, size_t capacity_stocks,
                                        int max_sessions, int max_session_stocks, KunServePoolHandle *out) {
    clear_error();
    if (!out) return KUN_INVALID_ARGUMENT;
    *out = nullptr;
    auto *ex = (Executor *)exec;
    auto *m = (const KunGpuModuleDesc *)mod;
    if (!ex || !m) {
        set_error("null executor or module");
        return KUN_INVALID_ARGUMENT;
    }
    if (m->abi != KUN_GPU_MODULE_ABI) {
        set_error("The required version in the module does not match the runtime version");
        return KUN_INVALID_ARGUMENT;
    }
    if (m->output_layout != KUN_LAYOUT_STREAM) {
        set_error("Cannot run batch mode module via StreamContext");
        return KUN_INVALID_ARGUMENT;
    }
    if (capacity_stocks == 0 || capacity_stocks > (size_t)INT32_MAX || max_sessions <= 0 || max_session_stocks <= 0) {
        set_error("Bad serving pool size: capacity %zu stocks, %d sessions, %d stocks per session",
                  capacity_stocks, max_sessions, max_session_stocks);
        return KUN_INVALID_ARGUMENT;
    }
    cudaSetDevice(ex->device);
    std::unique_ptr<ServePool> p(new ServePool());
    p->ex = ex;
    p->m = m;
    p->cap = (long long)capacity_stocks;
    p->max_sessions = max_sessions;
    p->max_len = max_session_stocks;
    if (!stream_order(m, p->order)) {
        set_error("module %s: cyclic stage graph", m->name);
        return KUN_INVALID_ARGUMENT;
    }
    if (!make_tick_schedule(m, p->order, kStepStreams, p->sched)) {
        cudaGetLastError();
        set_error("cannot create the streams of a serving pool");
        return KUN_CUDA_ERROR;
    }
    for (int b = 0; b < m->num_buffers; b++) {
        if (m->buffers[b].kind == KUN_BUF_INPUT) p->in_bufs.push_back(b);
        if (m->buffers[b].kind == KUN_BUF_OUTPUT) p->out_bufs.push_back(b);
    }
    size_t elem = p->elem();
    size_t ints = (size_t)(2 * max_sessions + 5);
    p->tick_off = (ints * sizeof(int32_t) + 15) / 16 * 16;
    p->table_bytes = p->tick_off + (size_t)max_sessions * sizeof(long long);
    size_t nin = p->in_bufs.size(), nout = p->out_bufs.size();
    bool ok = p->store.alloc(m, p->cap) && cudaMalloc(&p->d_table, p->table_bytes) == cudaSuccess &&
              cudaMalloc((void **)&p->d_in_rings, std::max<size_t>(1, nin) * sizeof(void *)) == cudaSuccess &&
              cudaMalloc((void **)&p->d_out_rings, std::max<size_t>(1, nout) * sizeof(void *)) == cudaSuccess &&
              cudaMalloc((void **)&p->d_in_win, std::max<size_t>(1, nin) * sizeof(int32_t)) == cudaSuccess &&
              cudaMalloc((void **)&p->d_out_win, std::max<size_t>(1, nout) * sizeof(int32_t)) == cudaSuccess &&
              cudaMalloc(&p->d_in, std::max<size_t>(1, nin) * p->cap * elem) == cudaSuccess &&
              cudaMalloc(&p->d_out, std::max<size_t>(1, nout) * p->cap * elem) == cudaSuccess &&
              cudaHostAlloc((void **)&p->h_table, p->table_bytes, cudaHostAllocDefault) == cudaSuccess &&
              cudaHostAlloc(&p->h_in, std::max<size_t>(1, nin) * p->cap * elem, cudaHostAllocDefault) == cudaSuccess &&
              cudaHostAlloc(&p->h_out, std::max<size_t>(1, nout) * p->cap * elem, cudaHostAllocDefault) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        set_error("out of memory for a serving pool of %zu stocks", capacity_stocks);
        return KUN_OUT_OF_MEMORY;
    }
    memset(p->h_table, 0, p->table_bytes);
    // a module whose Rank stages do not fit the level form keeps the
    // stage-by-stage schedule
    if (!make_tick_levels(p->store, p->order, p->levels)) {
        cudaGetLastError();
        free_tick_levels(p->levels);
    }
    std::vector<void *> rin, rout;
    std::vector<int32_t> win, wout;
    for (int b : p->in_bufs) {
        rin.push_back(p->store.rings[b]);
        win.push_back(m->buffers[b].window > 0 ? m->buffers[b].window : 1);
    }
    for (int b : p->out_bufs) {
        rout.push_back(p->store.rings[b]);
        wout.push_back(m->buffers[b].window > 0 ? m->buffers[b].window : 1);
    }
    cudaStream_t st = p->stream();
    cudaMemcpyAsync(p->d_in_rings, rin.data(), nin * sizeof(void *), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(p->d_out_rings, rout.data(), nout * sizeof(void *), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(p->d_in_win, win.data(), nin * sizeof(int32_t), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(p->d_out_win, wout.data(), nout * sizeof(int32_t), cudaMemcpyHostToDevice, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) {
        set_error("CUDA error creating a serving pool");
        return KUN_CUDA_ERROR;
    }
    p->free_cols[0] = p->cap;
    *out = p.release();
    return KUN_SUCCESS;
}

KUN_EXPORT void kunDestroyServePool(KunServePoolHandle pool) { delete SP(pool); }

KUN_EXPORT KunStatus kunServeOpen(KunServePoolHandle pool, size_t num_stocks, int64_t *session_id) {
    ServePool *p = SP(pool);
    if (!p || !session_id) return KUN_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(p->mu);
    clear_error();
    *session_id = 0;
    if (num_stocks == 0 || (long long)num_stocks > p->max_len) {
        set_error("session of %zu stocks: the pool takes 1 to %d stocks per session", num_stocks, p->max_len);
        return KUN_INVALID_ARGUMENT;
    }
    if ((int)p->sessions.size() >= p->max_sessions) {
        set_error("all %d session slots are in use", p->max_sessions);
        return KUN_OUT_OF_MEMORY;
    }
    auto it = p->free_cols.begin();
    for (; it != p->free_cols.end(); ++it)
        if (it->second >= (long long)num_stocks) break;
    if (it == p->free_cols.end()) {
        set_error("no free range of %zu stock columns", num_stocks);
        return KUN_OUT_OF_MEMORY;
    }
    long long start = it->first, len = it->second;
    p->free_cols.erase(it);
    if (len > (long long)num_stocks) p->free_cols[start + (long long)num_stocks] = len - (long long)num_stocks;
    KunStatus rc;
    {
        std::lock_guard<std::mutex> g_lk(p->gpu_mu);
        rc = p->store.reset(start, (long long)num_stocks, p->stream());
    }
    if (rc != KUN_SUCCESS) {
        p->free_cols[start] = (long long)num_stocks;
        return rc;
    }
    Session s;
    s.stock0 = start;
    s.len = (long long)num_stocks;
    int64_t id = p->next_id++;
    p->sessions[id] = s;
    *session_id = id;
    return KUN_SUCCESS;
}

KUN_EXPORT KunStatus kunServeClose(KunServePoolHandle pool, int64_t session_id) {
    ServePool *p = SP(pool);
    if (!p) return KUN_INVALID_ARGUMENT;
    std::unique_lock<std::mutex> lk(p->mu);
    auto it = p->sessions.find(session_id);
    if (it == p->sessions.end()) {
        set_error("unknown session %lld", (long long)session_id);
        return KUN_INVALID_ARGUMENT;
    }
    // a tick still queued or on the device finishes first
    p->cv_done.wait(lk, [&] {
        auto f = p->sessions.find(session_id);
        return f == p->sessions.end() || !f->second.pending || !p->running;
    });
    it = p->sessions.find(session_id);
    if (it == p->sessions.end()) return KUN_SUCCESS;
    if (it->second.pending) {
        // the loop stopped with the tick queued: drop it
        p->ready.erase(std::remove(p->ready.begin(), p->ready.end(), session_id), p->ready.end());
        it->second.pending = false;
    }
    long long start = it->second.stock0, len = it->second.len;
    p->sessions.erase(it);
    // free the columns and merge with the neighbouring free ranges
    auto nx = p->free_cols.lower_bound(start);
    if (nx != p->free_cols.end() && nx->first == start + len) {
        len += nx->second;
        nx = p->free_cols.erase(nx);
    }
    if (nx != p->free_cols.begin()) {
        auto pv = std::prev(nx);
        if (pv->first + pv->second == start) {
            start = pv->first;
            len += pv->second;
            p->free_cols.erase(pv);
        }
    }
    p->free_cols[start] = len;
    return KUN_SUCCESS;
}

KUN_EXPORT KunStatus kunServeStep(KunServePoolHandle pool, int num_sessions, const int64_t *session_ids,
                                  const void *device_inputs, void *device_outputs) {
    ServePool *p = SP(pool);
    if (!p || (num_sessions > 0 && !session_ids)) return KUN_INVALID_ARGUMENT;
    clear_error();
    return pool_step(p, num_sessions, session_ids, device_inputs, device_outputs);  // takes mu
}

KUN_EXPORT KunStatus kunServeStart(KunServePoolHandle pool, int batch_window_us) {
    ServePool *p = SP(pool);
    if (!p) return KUN_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(p->mu);
    if (p->running) return KUN_SUCCESS;
    p->batch_window_us = batch_window_us > 0 ? batch_window_us : 0;
    // every size bucket's graph is built now, so no step of the loop waits
    // for a graph capture
    {
        std::lock_guard<std::mutex> g_lk(p->gpu_mu);
        cudaSetDevice(p->ex->device);
        for (long long nb = 256;; nb = std::min<long long>(nb << 2, p->cap)) {
            for (int sb = 4;; sb = std::min(sb << 2, p->max_sessions)) {
                cudaGraphExec_t ge;
                KunStatus rs = graph_for(p, std::min<long long>(nb, p->cap), std::min(sb, p->max_sessions), &ge);
                if (rs != KUN_SUCCESS) return rs;
                if (sb >= p->max_sessions) break;
            }
            if (nb >= p->cap) break;
        }
    }
    p->failed = KUN_SUCCESS;
    p->running = true;
    p->loop = std::thread(serve_loop, p);
    return KUN_SUCCESS;
}

KUN_EXPORT KunStatus kunServeStop(KunServePoolHandle pool) {
    ServePool *p = SP(pool);
    if (!p) return KUN_INVALID_ARGUMENT;
    stop_loop(p);
    return KUN_SUCCESS;
}

KUN_EXPORT KunStatus kunServeSubmit(KunServePoolHandle pool, int num_sessions, const int64_t *session_ids) {
    ServePool *p = SP(pool);
    if (!p || (num_sessions > 0 && !session_ids)) return KUN_INVALID_ARGUMENT;
    auto now = std::chrono::steady_clock::now();
    {
        std::lock_guard<std::mutex> lk(p->mu);
        clear_error();
        if (!p->running) {
            set_error("the serving loop is not running (kunServeStart)");
            return KUN_INVALID_ARGUMENT;
        }
        if (p->failed != KUN_SUCCESS) {
            set_error("serving loop failed: %s", p->fail_msg.c_str());
            return p->failed;
        }
        for (int k = 0; k < num_sessions; k++) {
            auto it = p->sessions.find(session_ids[k]);
            if (it == p->sessions.end()) {
                set_error("unknown session %lld", (long long)session_ids[k]);
                return KUN_INVALID_ARGUMENT;
            }
            if (it->second.pending) {
                set_error("session %lld already has a tick in flight", (long long)session_ids[k]);
                return KUN_INVALID_ARGUMENT;
            }
        }
        for (int k = 0; k < num_sessions; k++) {
            Session &s = p->sessions[session_ids[k]];
            s.pending = true;
            s.t_submit = now;
            p->ready.push_back(session_ids[k]);
        }
    }
    p->cv_ready.notify_one();
    return KUN_SUCCESS;
}

// Wait until the session has completed `min_tick` ticks (timeout in ms, <0 =
// no limit); KUN_TIMEOUT when the time runs out.
KUN_EXPORT KunStatus kunServeWait(KunServePoolHandle pool, int64_t session_id, int64_t min_tick, int timeout_ms) {
    ServePool *p = SP(pool);
    if (!p) return KUN_INVALID_ARGUMENT;
    std::unique_lock<std::mutex> lk(p->mu);
    clear_error();
    auto done = [&] {
        auto it = p->sessions.find(session_id);
        return it == p->sessions.end() || it->second.tick >= min_tick || p->failed != KUN_SUCCESS ||
               (!it->second.pending && !p->running);
    };
    if (timeout_ms < 0) p->cv_done.wait(lk, done);
    else if (!p->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), done)) {
        set_error("timed out waiting for session %lld", (long long)session_id);
        return KUN_TIMEOUT;
    }
    auto it = p->sessions.find(session_id);
    if (it == p->sessions.end()) {
        set_error("unknown session %lld", (long long)session_id);
        return KUN_INVALID_ARGUMENT;
    }
    if (p->failed != KUN_SUCCESS) {
        set_error("serving loop failed: %s", p->fail_msg.c_str());
        return p->failed;
    }
    if (it->second.tick < min_tick) {
        set_error("the serving loop stopped before session %lld reached tick %lld", (long long)session_id,
                  (long long)min_tick);
        return KUN_INVALID_ARGUMENT;
    }
    return KUN_SUCCESS;
}

// Tick latencies (microseconds, submit to completion) recorded by the loop
// since the last call; returns how many were written to `out` (at most cap)
// and clears them.  `step_sizes` (may be NULL) gets the sessions per step.
KUN_EXPORT int kunServeTakeLatencies(KunServePoolHandle pool, float *out, int cap, int32_t *step_sizes,
                                     int step_cap, int *num_steps) {
    ServePool *p = SP(pool);
    if (!p) return -1;
    std::lock_guard<std::mutex> lk(p->mu);
    int n = std::min(cap, (int)p->lat_us.size());
    if (out) std::copy(p->lat_us.begin(), p->lat_us.begin() + n, out);
    int ns = std::min(step_cap, (int)p->step_sizes.size());
    if (step_sizes) std::copy(p->step_sizes.begin(), p->step_sizes.begin() + ns, step_sizes);
    if (num_steps) *num_steps = ns;
    p->lat_us.clear();
    p->step_sizes.clear();
    return n;
}

KUN_EXPORT void *kunServeHostInputs(KunServePoolHandle pool) { return SP(pool) ? SP(pool)->h_in : nullptr; }
KUN_EXPORT void *kunServeHostOutputs(KunServePoolHandle pool) { return SP(pool) ? SP(pool)->h_out : nullptr; }

KUN_EXPORT int64_t kunServeSessionTick(KunServePoolHandle pool, int64_t session_id) {
    ServePool *p = SP(pool);
    if (!p) return -1;
    std::lock_guard<std::mutex> lk(p->mu);
    auto it = p->sessions.find(session_id);
    return it == p->sessions.end() ? -1 : it->second.tick;
}

KUN_EXPORT int64_t kunServeSessionStocks(KunServePoolHandle pool, int64_t session_id) {
    ServePool *p = SP(pool);
    if (!p) return -1;
    std::lock_guard<std::mutex> lk(p->mu);
    auto it = p->sessions.find(session_id);
    return it == p->sessions.end() ? -1 : it->second.len;
}

KUN_EXPORT int64_t kunServeSessionColumn(KunServePoolHandle pool, int64_t session_id) {
    ServePool *p = SP(pool);
    if (!p) return -1;
    std::lock_guard<std::mutex> lk(p->mu);
    auto it = p->sessions.find(session_id);
    return it == p->sessions.end() ? -1 : it->second.stock0;
}

// Free stock columns: total and the largest contiguous range.
KUN_EXPORT KunStatus kunServeFreeStocks(KunServePoolHandle pool, int64_t *total, int64_t *largest) {
    ServePool *p = SP(pool);
    if (!p) return KUN_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(p->mu);
    int64_t t = 0, l = 0;
    for (auto &f : p->free_cols) {
        t += f.second;
        l = std::max<int64_t>(l, f.second);
    }
    if (total) *total = t;
    if (largest) *largest = l;
    return KUN_SUCCESS;
}

// Device bytes a serving pool of `capacity_stocks` columns takes for module m.
KUN_EXPORT int64_t kunServePoolBytes(KunModuleHandle mod, size_t capacity_stocks) {
    auto *m = (const KunGpuModuleDesc *)mod;
    if (!m) return -1;
    StreamStore s;
    s.m = m;
    int nin = 0, nout = 0;
    for (int b = 0; b < m->num_buffers; b++) {
        nin += m->buffers[b].kind == KUN_BUF_INPUT;
        nout += m->buffers[b].kind == KUN_BUF_OUTPUT;
    }
    size_t elem = m->dtype == 0 ? 4 : 8;
    return (int64_t)((s.bytes_per_stock() + (size_t)(nin + nout) * elem) * capacity_stocks);
}
