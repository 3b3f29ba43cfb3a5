// Stream mode of libkungpu.so: the reference's StreamContext
// (cpp/Kun/Runtime.cpp:385-546, C API cpp/Kun/CApi.cpp:79-189) on the GPU.
//
// A StreamStore holds the device state of a stream module for `cap` stock
// columns: one ring of `window` rows per buffer (NaN filled, like
// StreamBuffer::make) and, per stage, the struct-of-arrays state of its ops.
// A stream context owns a store for its own stocks and replays one captured
// CUDA graph per tick; the graph ends with a kernel that advances the
// device-side tick counter, so ticks can be queued without host round trips.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include "kun_runtime_internal.h"
#include "kun_xsec.cuh"

namespace kungpu {

// NaN-fill columns [col0, col0 + ncols) of every ring row: row f of the
// flattened rows of all rings starts at rows[f]
template <typename T>
__global__ void fill_rows_nan(T *const *rows, long long col0, long long ncols) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncols) return;
    rows[blockIdx.y][col0 + c] = (T)__int_as_float(0x7fc00000);
}


__global__ void advance_tick(long long *tick, int nseg) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < nseg) tick[k] += 1;
}

static size_t elem_of(const KunGpuModuleDesc *m) { return m->dtype == 0 ? 4 : 8; }

bool StreamStore::alloc(const KunGpuModuleDesc *mod, long long capacity) {
    m = mod;
    cap = capacity;
    size_t elem = elem_of(m);
    rings.assign(m->num_buffers, nullptr);
    st_t.assign(m->num_stages, nullptr);
    st_i.assign(m->num_stages, nullptr);
    for (int b = 0; b < m->num_buffers; b++) {
        size_t w = (size_t)(m->buffers[b].window > 0 ? m->buffers[b].window : 1);
        if (cudaMalloc(&rings[b], w * (size_t)cap * elem) != cudaSuccess) return false;
    }
    for (int s = 0; s < m->num_stages; s++) {
        const KunGpuStageDesc &d = m->stages[s];
        if (d.state_t_vars && cudaMalloc(&st_t[s], (size_t)d.state_t_vars * cap * elem) != cudaSuccess) return false;
        if (d.state_i_vars && cudaMalloc(&st_i[s], (size_t)d.state_i_vars * cap * 4) != cudaSuccess) return false;
    }
    if (cudaMalloc(&d_init, 4 * sizeof(int64_t)) != cudaSuccess) return false;
    // row table for one-launch resets
    std::vector<void *> rowp;
    for (int b = 0; b < m->num_buffers; b++) {
        long long w = m->buffers[b].window > 0 ? m->buffers[b].window : 1;
        for (long long r = 0; r < w; r++) rowp.push_back((char *)rings[b] + (size_t)r * cap * elem);
    }
    n_rows = (long long)rowp.size();
    if (n_rows && cudaMalloc((void **)&d_rows, rowp.size() * sizeof(void *)) != cudaSuccess) return false;
    if (n_rows && cudaMemcpy(d_rows, rowp.data(), rowp.size() * sizeof(void *), cudaMemcpyHostToDevice) != cudaSuccess)
        return false;
    return true;
}

void StreamStore::release() {
    for (auto p : rings)
        if (p) cudaFree(p);
    for (auto p : st_t)
        if (p) cudaFree(p);
    for (auto p : st_i)
        if (p) cudaFree(p);
    if (d_init) cudaFree(d_init);
    if (d_rows) cudaFree(d_rows);
    d_rows = nullptr;
    rings.clear();
    st_t.clear();
    st_i.clear();
    d_init = nullptr;
}

size_t StreamStore::bytes_per_stock() const {
    size_t elem = elem_of(m), n = 0;
    for (int b = 0; b < m->num_buffers; b++) n += (size_t)(m->buffers[b].window > 0 ? m->buffers[b].window : 1) * elem;
    for (int s = 0; s < m->num_stages; s++)
        n += (size_t)m->stages[s].state_t_vars * elem + (size_t)m->stages[s].state_i_vars * 4;
    return n;
}

// NaN-fill the ring columns of stocks [stock0, stock0 + count) and reset
// their op states (the ops' constructors, cpp/Kun/Ops.hpp).
KunStatus StreamStore::reset(long long stock0, long long count, cudaStream_t st) {
    size_t elem = elem_of(m);
    // every ring row in one launch (rows go along grid y, at most 65535 per launch)
    for (long long r0 = 0; r0 < n_rows; r0 += 65535) {
        dim3 grid((unsigned)((count + 255) / 256), (unsigned)std::min<long long>(65535, n_rows - r0));
        if (elem == 4)
            fill_rows_nan<float><<<grid, 256, 0, st>>>((float *const *)d_rows + r0, stock0, count);
        else
            fill_rows_nan<double><<<grid, 256, 0, st>>>((double *const *)d_rows + r0, stock0, count);
    }
    int32_t h_seg[3] = {0, (int32_t)count, (int32_t)stock0};
    cudaMemcpyAsync(d_init, h_seg, sizeof h_seg, cudaMemcpyHostToDevice, st);
    for (int s = 0; s < m->num_stages; s++) {
        const KunGpuStageDesc &d = m->stages[s];
        if (!d.init) continue;
        KunGpuStageArgs a;
        memset(&a, 0, sizeof a);
        a.buffers = rings.data();
        a.num_stocks = cap;
        a.state = st_t[s];
        a.state_i = st_i[s];
        a.seg_off = (const int32_t *)d_init;
        a.seg_stock0 = (const int32_t *)d_init + 2;
        a.nseg = 1;
        a.n_active = count;
        int rc = d.init(&a, (void *)st);
        if (rc) {
            set_error("state init of stage %d failed: %s", s, cudaGetErrorString((cudaError_t)rc));
            return KUN_CUDA_ERROR;
        }
    }
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        set_error("CUDA error: %s", cudaGetErrorString(e));
        return KUN_CUDA_ERROR;
    }
    return KUN_SUCCESS;
}

bool make_tick_schedule(const KunGpuModuleDesc *m, const std::vector<int> &order, int nstreams, TickSchedule &s) {
    int ns = m->num_stages;
    nstreams = std::max(1, nstreams);
    s.preds.assign(ns, {});
    for (int i = 0; i < ns; i++)
        for (int d = 0; d < m->stages[i].num_deps; d++)
            if (m->stages[i].deps[d] >= 0) s.preds[m->stages[i].deps[d]].push_back(i);
    // continue a predecessor's chain when it is that stream's tail, else the
    // stream with the least work
    s.stream_of.assign(ns, 0);
    std::vector<int> tail(nstreams, -1), load(nstreams, 0);
    for (int si : order) {
        int pick = -1;
        for (int d : s.preds[si])
            for (int k = 0; k < nstreams; k++)
                if (tail[k] == d) pick = k;
        if (pick < 0) pick = (int)(std::min_element(load.begin(), load.end()) - load.begin());
        s.stream_of[si] = pick;
        tail[pick] = si;
        load[pick] += m->stages[si].num_kernels > 0 ? m->stages[si].num_kernels : 1;
    }
    s.streams.assign(nstreams, nullptr);
    for (int k = 1; k < nstreams; k++)
        if (cudaStreamCreateWithFlags(&s.streams[k], cudaStreamNonBlocking) != cudaSuccess) return false;
    s.done.assign(ns, nullptr);
    for (int i = 0; i < ns; i++)
        if (cudaEventCreateWithFlags(&s.done[i], cudaEventDisableTiming) != cudaSuccess) return false;
    s.join.assign(nstreams, nullptr);
    for (int k = 0; k < nstreams; k++)
        if (cudaEventCreateWithFlags(&s.join[k], cudaEventDisableTiming) != cudaSuccess) return false;
    return cudaEventCreateWithFlags(&s.fork, cudaEventDisableTiming) == cudaSuccess;
}

void free_tick_schedule(TickSchedule &s) {
    for (size_t k = 1; k < s.streams.size(); k++)
        if (s.streams[k]) cudaStreamDestroy(s.streams[k]);
    for (auto e : s.done)
        if (e) cudaEventDestroy(e);
    for (auto e : s.join)
        if (e) cudaEventDestroy(e);
    if (s.fork) cudaEventDestroy(s.fork);
    s = TickSchedule();
}

// Enqueue one tick of every stage for the segments in d_seg / d_tick: in
// order on `st`, or with `sched`, on its streams (forked from and joined back
// into `st`) with events for the cross-stream dependencies.
bool make_tick_levels(const StreamStore &store, const std::vector<int> &order, TickLevels &lv) {
    const KunGpuModuleDesc *m = store.m;
    const int ns = m->num_stages;
    std::vector<int> depth(ns, 0);
    for (int si : order)  // a topological order: predecessors come first
        for (int d = 0; d < m->stages[si].num_deps; d++) {
            const int j = m->stages[si].deps[d];
            if (j >= 0) depth[j] = std::max(depth[j], depth[si] + 1);
        }
    int nl = 0;
    for (int si : order) nl = std::max(nl, depth[si] + 1);
    std::vector<std::vector<int>> ranks(nl);
    lv.other.assign(nl, {});
    for (int si : order) {
        const KunGpuStageDesc &d = m->stages[si];
        if (d.kind == KUN_STAGE_RANK) {
            if (d.num_in != 1 || d.num_out != 1) return false;
            ranks[depth[si]].push_back(si);
        } else {
            lv.other[depth[si]].push_back(si);
        }
    }
    std::vector<kun::RankJob> jobs;
    lv.rank_off.assign(nl, 0);
    lv.rank_cnt.assign(nl, 0);
    for (int l = 0; l < nl; l++) {
        lv.rank_off[l] = (int)jobs.size();
        lv.rank_cnt[l] = (int)ranks[l].size();
        for (int si : ranks[l]) {
            const int bi = m->stages[si].in_bufs[0], bo = m->stages[si].out_bufs[0];
            kun::RankJob jb;
            jb.in = store.rings[bi];
            jb.out = store.rings[bo];
            jb.w_in = std::max(1, (int)m->buffers[bi].window);
            jb.w_out = std::max(1, (int)m->buffers[bo].window);
            jobs.push_back(jb);
        }
    }
    if (!jobs.empty()) {
        if (cudaMalloc(&lv.d_jobs, jobs.size() * sizeof(kun::RankJob)) != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
        if (cudaMemcpy(lv.d_jobs, jobs.data(), jobs.size() * sizeof(kun::RankJob), cudaMemcpyHostToDevice) !=
            cudaSuccess)
            return false;
    }
    if (cudaStreamCreateWithFlags(&lv.side, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&lv.fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&lv.join, cudaEventDisableTiming) != cudaSuccess)
        return false;
    lv.ok = true;
    return true;
}

void free_tick_levels(TickLevels &lv) {
    if (lv.d_jobs) cudaFree(lv.d_jobs);
    if (lv.side) cudaStreamDestroy(lv.side);
    if (lv.fork) cudaEventDestroy(lv.fork);
    if (lv.join) cudaEventDestroy(lv.join);
    lv.d_jobs = nullptr;
    lv.side = nullptr;
    lv.fork = lv.join = nullptr;
    lv.ok = false;
}

static KunStatus launch_stage(const StreamStore &store, int si, const int32_t *d_seg_off, const int32_t *d_seg_stock0,
                              const int64_t *d_tick, int nseg, long long n_active, int max_len, cudaStream_t sst,
                              const int32_t *d_seg_count) {
    const KunGpuStageDesc &d = store.m->stages[si];
    KunGpuStageArgs a;
    memset(&a, 0, sizeof a);
    a.buffers = store.rings.data();
    a.num_stocks = store.cap;
    a.total_time = 1;
    a.length = 1;
    a.state = store.st_t[si];
    a.state_i = store.st_i[si];
    a.seg_off = d_seg_off;
    a.seg_stock0 = d_seg_stock0;
    a.seg_tick = d_tick;
    a.nseg = nseg;
    a.n_active = n_active;
    a.max_seg_len = max_len;
    a.seg_count = d_seg_count;
    int rc = d.launch(&a, (void *)sst);
    if (rc) {
        set_error("stage %d (%s) failed: %s", si, d.name, cudaGetErrorString((cudaError_t)rc));
        return KUN_CUDA_ERROR;
    }
    return KUN_SUCCESS;
}

KunStatus enqueue_tick(const StreamStore &store, const std::vector<int> &order, const int32_t *d_seg_off,
                       const int32_t *d_seg_stock0, const int64_t *d_tick, int nseg, long long n_active,
                       int max_len, cudaStream_t st, const int32_t *d_seg_count, const TickSchedule *sched,
                       const TickLevels *levels) {
    const KunGpuModuleDesc *m = store.m;
    if (levels && levels->ok) {
        for (size_t l = 0; l < levels->other.size(); l++) {
            for (int si : levels->other[l]) {
                KunStatus rs = launch_stage(store, si, d_seg_off, d_seg_stock0, d_tick, nseg, n_active, max_len, st,
                                            d_seg_count);
                if (rs != KUN_SUCCESS) return rs;
            }
            if (levels->rank_cnt[l] > 0) {
                const kun::RankJob *jobs = (const kun::RankJob *)levels->d_jobs + levels->rank_off[l];
                // with a device table both size classes launch: the long
                // segments' launch on the side stream, concurrently
                const bool both = d_seg_count != nullptr && max_len > kun::kRankSmallMax;
                if (both) {
                    cudaEventRecord(levels->fork, st);
                    cudaStreamWaitEvent(levels->side, levels->fork, 0);
                }
                cudaStream_t sl = both ? levels->side : nullptr;
                int rc = m->dtype == 0
                             ? kun::launch_rank_multi_segments<float>(jobs, levels->rank_cnt[l], store.cap, d_seg_off,
                                                                      d_seg_stock0, (const long long *)d_tick, nseg,
                                                                      max_len, d_seg_count, st, sl)
                             : kun::launch_rank_multi_segments<double>(jobs, levels->rank_cnt[l], store.cap,
                                                                       d_seg_off, d_seg_stock0,
                                                                       (const long long *)d_tick, nseg, max_len,
                                                                       d_seg_count, st, sl);
                if (both) {
                    cudaEventRecord(levels->join, levels->side);
                    cudaStreamWaitEvent(st, levels->join, 0);
                }
                if (rc) {
                    set_error("rank stages of level %d failed: %s", (int)l, cudaGetErrorString((cudaError_t)rc));
                    return KUN_CUDA_ERROR;
                }
            }
        }
        return KUN_SUCCESS;
    }
    const bool multi = sched && sched->streams.size() > 1;
    if (multi) {
        cudaEventRecord(sched->fork, st);
        for (size_t k = 1; k < sched->streams.size(); k++) cudaStreamWaitEvent(sched->streams[k], sched->fork, 0);
    }
    for (int si : order) {
        const KunGpuStageDesc &d = m->stages[si];
        cudaStream_t sst = st;
        if (multi) {
            int k = sched->stream_of[si];
            sst = k == 0 ? st : sched->streams[k];
            for (int pd : sched->preds[si])
                if (sched->stream_of[pd] != k) cudaStreamWaitEvent(sst, sched->done[pd], 0);
        }
        KunGpuStageArgs a;
        memset(&a, 0, sizeof a);
        a.buffers = store.rings.data();
        a.num_stocks = store.cap;
        a.total_time = 1;
        a.length = 1;
        a.state = store.st_t[si];
        a.state_i = store.st_i[si];
        a.seg_off = d_seg_off;
        a.seg_stock0 = d_seg_stock0;
        a.seg_tick = d_tick;
        a.nseg = nseg;
        a.n_active = n_active;
        a.max_seg_len = max_len;
        a.seg_count = d_seg_count;
        int rc = d.launch(&a, (void *)sst);
        if (rc) {
            set_error("stage %d (%s) failed: %s", si, d.name, cudaGetErrorString((cudaError_t)rc));
            return KUN_CUDA_ERROR;
        }
        if (multi) cudaEventRecord(sched->done[si], sst);
    }
    if (multi)
        for (size_t k = 1; k < sched->streams.size(); k++) {
            cudaEventRecord(sched->join[k], sched->streams[k]);
            cudaStreamWaitEvent(st, sched->join[k], 0);
        }
    return KUN_SUCCESS;
}

bool stream_order(const KunGpuModuleDesc *m, std::vector<int> &order) {
    std::vector<int> pending(m->num_stages);
    for (int i = 0; i < m->num_stages; i++) pending[i] = m->stages[i].pending;
    std::vector<int> ready;
    for (int i = 0; i < m->num_stages; i++)
        if (pending[i] == 0) ready.push_back(i);
    size_t head = 0;
    while (head < ready.size()) {
        int i = ready[head++];
        order.push_back(i);
        for (int d = 0; d < m->stages[i].num_deps; d++) {
            int j = m->stages[i].deps[d];
            if (j >= 0 && --pending[j] == 0) ready.push_back(j);
        }
    }
    return (int)order.size() == m->num_stages;
}

struct StreamCtx {
    Executor *ex = nullptr;
    const KunGpuModuleDesc *m = nullptr;
    long long S = 0;
    long long tick = 0;
    StreamStore store;
    std::vector<int> order;
    int32_t *d_seg = nullptr;  // seg_off[2], seg_stock0[1]
    int64_t *d_tick = nullptr;
    std::vector<int> last_row;
    std::vector<std::vector<char>> mirror;
    cudaGraphExec_t graph = nullptr;
    TickLevels levels;
    cudaStream_t stream() const { return ex->streams[0]; }
    ~StreamCtx() {
        if (graph) cudaGraphExecDestroy(graph);
        free_tick_levels(levels);
        if (d_seg) cudaFree(d_seg);
        if (d_tick) cudaFree(d_tick);
        store.release();
    }
};

static int win_of(const KunGpuModuleDesc *m, int b) { return m->buffers[b].window > 0 ? m->buffers[b].window : 1; }

static KunStatus build_graph(StreamCtx *c) {
    cudaStream_t st = c->stream();
    if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        set_error("cannot capture the tick graph");
        return KUN_CUDA_ERROR;
    }
    KunStatus rs = enqueue_tick(c->store, c->order, c->d_seg, c->d_seg + 2, c->d_tick, 1, c->S, (int)c->S, st,
                                nullptr, nullptr, &c->levels);
    advance_tick<<<1, 32, 0, st>>>((long long *)c->d_tick, 1);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(st, &g);
    if (rs != KUN_SUCCESS || e != cudaSuccess || !g) {
        if (g) cudaGraphDestroy(g);
        if (rs == KUN_SUCCESS) set_error("tick graph capture failed: %s", cudaGetErrorString(e));
        cudaGetLastError();
        return rs == KUN_SUCCESS ? KUN_CUDA_ERROR : rs;
    }
    e = cudaGraphInstantiate(&c->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        set_error("tick graph instantiate failed: %s", cudaGetErrorString(e));
        return KUN_CUDA_ERROR;
    }
    return KUN_SUCCESS;
}

// ------------------------------------------------------------ serialisation
// Own format (the reference's is explicitly non-portable, doc/Stream.md):
//   "KUNGPUS1" | u32 version | u32 dtype | i64 stocks | i64 tick |
//   u32 buffers | u32 stages | char[64] module name |
//   per buffer: i32 window, i32 last row, window x stocks values |
//   per stage: i32 float vars, i32 int vars, the arrays (stocks columns).
static const char kMagic[8] = {'K', 'U', 'N', 'G', 'P', 'U', 'S', '1'};

struct Writer {
    virtual bool write(const void *p, size_t n) = 0;
    virtual ~Writer() = default;
};
struct MemWriter : Writer {
    char *buf;
    size_t cap, pos = 0;
    MemWriter(char *b, size_t c) : buf(b), cap(c) {}
    bool write(const void *p, size_t n) override {
        if (buf && pos + n <= cap) memcpy(buf + pos, p, n);
        pos += n;
        return true;
    }
};
struct FileWriter : Writer {
    std::ofstream f;
    explicit FileWriter(const char *path) : f(path, std::ios::binary) {}
    bool write(const void *p, size_t n) override {
        f.write((const char *)p, (std::streamsize)n);
        return (bool)f;
    }
};
struct Reader {
    virtual bool read(void *p, size_t n) = 0;
    virtual ~Reader() = default;
};
struct MemReader : Reader {
    const char *buf;
    size_t size, pos = 0;
    MemReader(const char *b, size_t s) : buf(b), size(s) {}
    bool read(void *p, size_t n) override {
        if (pos + n > size) return false;
        memcpy(p, buf + pos, n);
        pos += n;
        return true;
    }
};
struct FileReader : Reader {
    std::ifstream f;
    explicit FileReader(const char *path) : f(path, std::ios::binary) {}
    bool read(void *p, size_t n) override {
        f.read((char *)p, (std::streamsize)n);
        return (bool)f && (size_t)f.gcount() == n;
    }
};

// copy rows [0, rows) x columns [col0, col0 + n) of a pitched device array
static bool dev_to_host_cols(std::vector<char> &host, const void *dev, size_t elem, long long pitch, long long rows,
                             long long col0, long long n, cudaStream_t st) {
    host.resize((size_t)rows * n * elem);
    if (!rows || !n) return true;
    return cudaMemcpy2DAsync(host.data(), n * elem, (const char *)dev + col0 * elem, pitch * elem, n * elem, rows,
                             cudaMemcpyDeviceToHost, st) == cudaSuccess;
}
static bool host_to_dev_cols(void *dev, const std::vector<char> &host, size_t elem, long long pitch, long long rows,
                             long long col0, long long n, cudaStream_t st) {
    if (!rows || !n) return true;
    return cudaMemcpy2DAsync((char *)dev + col0 * elem, pitch * elem, host.data(), n * elem, n * elem, rows,
                             cudaMemcpyHostToDevice, st) == cudaSuccess;
}

bool serialize_range(const StreamStore &store, long long col0, long long n, long long tick,
                     const std::vector<int> &last_row, Writer &w, cudaStream_t st) {
    const KunGpuModuleDesc *m = store.m;
    size_t elem = elem_of(m);
    uint32_t ver = 1, dt = (uint32_t)m->dtype, nb = (uint32_t)m->num_buffers, ns = (uint32_t)m->num_stages;
    int64_t stocks = n, tk = tick;
    char name[64] = {0};
    strncpy(name, m->name, 63);
    w.write(kMagic, 8);
    w.write(&ver, 4);
    w.write(&dt, 4);
    w.write(&stocks, 8);
    w.write(&tk, 8);
    w.write(&nb, 4);
    w.write(&ns, 4);
    w.write(name, 64);
    std::vector<char> host;
    for (int b = 0; b < m->num_buffers; b++) {
        int32_t win = win_of(m, b), lr = last_row[b];
        w.write(&win, 4);
        w.write(&lr, 4);
        if (!dev_to_host_cols(host, store.rings[b], elem, store.cap, win, col0, n, st)) return false;
        cudaStreamSynchronize(st);
        if (!w.write(host.data(), host.size())) return false;
    }
    for (int s = 0; s < m->num_stages; s++) {
        const KunGpuStageDesc &d = m->stages[s];
        int32_t nt = d.state_t_vars, ni = d.state_i_vars;
        w.write(&nt, 4);
        w.write(&ni, 4);
        if (nt) {
            if (!dev_to_host_cols(host, store.st_t[s], elem, store.cap, nt, col0, n, st)) return false;
            cudaStreamSynchronize(st);
            if (!w.write(host.data(), host.size())) return false;
        }
        if (ni) {
            if (!dev_to_host_cols(host, store.st_i[s], 4, store.cap, ni, col0, n, st)) return false;
            cudaStreamSynchronize(st);
            if (!w.write(host.data(), host.size())) return false;
        }
    }
    return true;
}

// A dump read and checked on the host: every ring and state array of a
// range of `n` stocks, as laid out in the file.
struct ParsedDump {
    long long tick = 0;
    std::vector<int> last_row;
    std::vector<std::vector<char>> rings;         // per buffer [window][n]
    std::vector<std::vector<char>> st_t, st_i;    // per stage [vars][n]
};

// Reads a dump for `n` stocks of module `m` and checks every value a kernel
// would use as an index or a loop bound: ring rows in [0, window), the tick
// non-negative, and each int32 state within the bounds the module declares
// (state_i_max).  Touches no device memory; on failure sets the reference's
// error text (cpp/Kun/Runtime.cpp:418,456).
static bool parse_dump(const KunGpuModuleDesc *m, long long n, Reader &r, ParsedDump &d) {
    size_t elem = elem_of(m);
    char magic[8];
    uint32_t ver, dt, nb, ns;
    int64_t stocks, tk;
    char name[64];
    if (!r.read(magic, 8) || memcmp(magic, kMagic, 8) || !r.read(&ver, 4) || ver != 1 || !r.read(&dt, 4) ||
        dt != (uint32_t)m->dtype || !r.read(&stocks, 8) || stocks != n || !r.read(&tk, 8) || tk < 0 ||
        !r.read(&nb, 4) || nb != (uint32_t)m->num_buffers || !r.read(&ns, 4) || ns != (uint32_t)m->num_stages ||
        !r.read(name, 64) || strncmp(name, m->name, 63)) {
        set_error("Failed to read initial stream buffer");
        return false;
    }
    d.tick = tk;
    d.last_row.assign(m->num_buffers, 0);
    d.rings.assign(m->num_buffers, {});
    for (int b = 0; b < m->num_buffers; b++) {
        int32_t win, lr;
        if (!r.read(&win, 4) || win != win_of(m, b) || !r.read(&lr, 4) || lr < 0 || lr >= win) {
            set_error("Failed to read initial stream buffer");
            return false;
        }
        d.last_row[b] = lr;
        d.rings[b].resize((size_t)win * n * elem);
        if (!r.read(d.rings[b].data(), d.rings[b].size())) {
            set_error("Failed to read initial stream buffer");
            return false;
        }
    }
    d.st_t.assign(m->num_stages, {});
    d.st_i.assign(m->num_stages, {});
    for (int s = 0; s < m->num_stages; s++) {
        const KunGpuStageDesc &sd = m->stages[s];
        int32_t nt, ni;
        if (!r.read(&nt, 4) || nt != sd.state_t_vars || !r.read(&ni, 4) || ni != sd.state_i_vars) {
            set_error("Failed to deserialize state buffer");
            return false;
        }
        d.st_t[s].resize((size_t)nt * n * elem);
        d.st_i[s].resize((size_t)ni * n * 4);
        if ((nt && !r.read(d.st_t[s].data(), d.st_t[s].size())) ||
            (ni && !r.read(d.st_i[s].data(), d.st_i[s].size()))) {
            set_error("Failed to deserialize state buffer");
            return false;
        }
        if (ni && !sd.state_i_max) {
            set_error("Failed to deserialize state buffer");
            return false;
        }
        const int32_t *iv = (const int32_t *)d.st_i[s].data();
        for (int v = 0; v < ni; v++) {
            const int32_t mx = sd.state_i_max[v];
            if (mx < 0) continue;
            for (long long k = 0; k < n; k++) {
                const int32_t x = iv[(size_t)v * n + k];
                if (x < 0 || x > mx) {
                    set_error("Failed to deserialize state buffer");
                    return false;
                }
            }
        }
    }
    return true;
}

// Copies a checked dump into columns [col0, col0 + n) of the store.
static bool upload_dump(StreamStore &store, long long col0, long long n, const ParsedDump &d, cudaStream_t st) {
    const KunGpuModuleDesc *m = store.m;
    size_t elem = elem_of(m);
    bool ok = true;
    for (int b = 0; b < m->num_buffers; b++)
        ok = ok && host_to_dev_cols(store.rings[b], d.rings[b], elem, store.cap, win_of(m, b), col0, n, st);
    for (int s = 0; s < m->num_stages; s++) {
        const KunGpuStageDesc &sd = m->stages[s];
        if (sd.state_t_vars)
            ok = ok && host_to_dev_cols(store.st_t[s], d.st_t[s], elem, store.cap, sd.state_t_vars, col0, n, st);
        if (sd.state_i_vars)
            ok = ok && host_to_dev_cols(store.st_i[s], d.st_i[s], 4, store.cap, sd.state_i_vars, col0, n, st);
    }
    ok = cudaStreamSynchronize(st) == cudaSuccess && ok;
    if (!ok) set_error("Failed to deserialize state buffer");
    return ok;
}

static StreamCtx *create_ctx(Executor *ex, const KunGpuModuleDesc *m, long long S, Reader *init, KunStatus &rc) {
    rc = KUN_INVALID_ARGUMENT;
    if (!m) {
        set_error("null executor or module");
        return nullptr;
    }
    if (m->abi != KUN_GPU_MODULE_ABI) {
        set_error("The required version in the module does not match the runtime version");
        return nullptr;
    }
    if (m->output_layout != KUN_LAYOUT_STREAM) {
        set_error("Cannot run batch mode module via StreamContext");
        return nullptr;
    }
    if (S <= 0) {
        set_error("Bad num_stocks");
        return nullptr;
    }
    // a restored dump is read and checked in full before any device work
    ParsedDump dump;
    if (init && !parse_dump(m, S, *init, dump)) {
        rc = KUN_INIT_ERROR;
        return nullptr;
    }
    if (!ex) {
        set_error("null executor or module");
        return nullptr;
    }
    cudaSetDevice(ex->device);
    auto *c = new StreamCtx();
    c->ex = ex;
    c->m = m;
    c->S = S;
    rc = KUN_OUT_OF_MEMORY;
    if (!stream_order(m, c->order)) {
        set_error("module %s: cyclic stage graph", m->name);
        rc = KUN_INVALID_ARGUMENT;
        delete c;
        return nullptr;
    }
    if (!c->store.alloc(m, S) || cudaMalloc(&c->d_seg, 3 * sizeof(int32_t)) != cudaSuccess ||
        cudaMalloc(&c->d_tick, sizeof(int64_t)) != cudaSuccess) {
        cudaGetLastError();
        set_error("out of device memory for a stream of %lld stocks", S);
        delete c;
        return nullptr;
    }
    if (!make_tick_levels(c->store, c->order, c->levels)) {
        cudaGetLastError();
        free_tick_levels(c->levels);
    }
    cudaStream_t st = c->stream();
    int32_t seg[3] = {0, (int32_t)S, 0};
    cudaMemcpyAsync(c->d_seg, seg, sizeof seg, cudaMemcpyHostToDevice, st);
    rc = c->store.reset(0, S, st);
    if (rc != KUN_SUCCESS) {
        delete c;
        return nullptr;
    }
    c->last_row.resize(m->num_buffers);
    for (int b = 0; b < m->num_buffers; b++) c->last_row[b] = win_of(m, b) - 1;
    if (init) {
        c->tick = dump.tick;
        c->last_row = dump.last_row;
        if (!upload_dump(c->store, 0, S, dump, st)) {
            rc = KUN_INIT_ERROR;
            delete c;
            return nullptr;
        }
    }
    int64_t tk = c->tick;
    cudaMemcpyAsync(c->d_tick, &tk, sizeof tk, cudaMemcpyHostToDevice, st);
    cudaStreamSynchronize(st);
    c->mirror.resize(m->num_buffers);
    rc = build_graph(c);
    if (rc != KUN_SUCCESS) {
        delete c;
        return nullptr;
    }
    rc = KUN_SUCCESS;
    return c;
}

static KunStatus ctx_run(StreamCtx *c, bool sync) {
    cudaStream_t st = c->stream();
    cudaError_t e = cudaGraphLaunch(c->graph, st);
    if (e != cudaSuccess) {
        set_error("tick launch failed: %s", cudaGetErrorString(e));
        return KUN_CUDA_ERROR;
    }
    const KunGpuModuleDesc *m = c->m;
    for (int b = 0; b < m->num_buffers; b++)
        if (m->buffers[b].kind != KUN_BUF_INPUT) c->last_row[b] = (int)(c->tick % win_of(m, b));
    c->tick++;
    if (sync) {
        e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) {
            set_error("CUDA error: %s", cudaGetErrorString(e));
            return KUN_CUDA_ERROR;
        }
    }
    return KUN_SUCCESS;
}

static bool valid_handle(StreamCtx *c, size_t h) {
    if (!c || h >= (size_t)c->m->num_buffers) {
        set_error("Bad buffer handle");
        return false;
    }
    return true;
}

}  // namespace kungpu

using namespace kungpu;

static StreamCtx *C(KunStreamContextHandle h) { return (StreamCtx *)h; }

KUN_EXPORT KunStreamContextHandle kunCreateStream(KunExecutorHandle exec, KunModuleHandle m, size_t num_stocks) {
    clear_error();
    KunStatus rc;
    return create_ctx((Executor *)exec, (const KunGpuModuleDesc *)m, (long long)num_stocks, nullptr, rc);
}

KUN_EXPORT KunStatus kunCreateStreamEx(KunExecutorHandle exec, KunModuleHandle m, size_t num_stocks,
                                       const KunStreamExtraArgs *extra, KunStreamContextHandle *out) {
    clear_error();
    if (out) *out = nullptr;
    if (!out) return KUN_INVALID_ARGUMENT;
    std::unique_ptr<Reader> reader;
    if (extra) {
        if (extra->version != KUN_API_VERSION) return KUN_INVALID_ARGUMENT;
        if (extra->init_kind == KUN_INIT_FILE) {
            if (!extra->init.path) return KUN_INVALID_ARGUMENT;
            reader.reset(new FileReader(extra->init.path));
        } else if (extra->init_kind == KUN_INIT_MEMORY) {
            if (!extra->init.memory.buffer) return KUN_INVALID_ARGUMENT;
            reader.reset(new MemReader(extra->init.memory.buffer, extra->init.memory.size));
        } else if (extra->init_kind != KUN_INIT_NONE) {
            return KUN_INVALID_ARGUMENT;
        }
    }
    KunStatus rc;
    StreamCtx *c = create_ctx((Executor *)exec, (const KunGpuModuleDesc *)m, (long long)num_stocks, reader.get(), rc);
    if (!c) return rc == KUN_SUCCESS ? KUN_INIT_ERROR : rc;
    *out = c;
    return KUN_SUCCESS;
}

KUN_EXPORT KunStatus kunStreamSerializeStates(KunStreamContextHandle context, KunStateBufferKind kind,
                                              char *path_or_buffer, size_t *size) {
    StreamCtx *c = C(context);
    if (!c) return KUN_INVALID_ARGUMENT;
    cudaStream_t st = c->stream();
    cudaStreamSynchronize(st);
    if (kind == KUN_INIT_FILE) {
        if (!path_or_buffer) return KUN_INVALID_ARGUMENT;
        FileWriter w(path_or_buffer);
        return serialize_range(c->store, 0, c->S, c->tick, c->last_row, w, st) ? KUN_SUCCESS : KUN_INIT_ERROR;
    }
    if (kind == KUN_INIT_MEMORY) {
        // two-phase size query as the reference (cpp/Kun/CApi.cpp:139-164)
        if (!size || (*size != 0 && !path_or_buffer)) return KUN_INVALID_ARGUMENT;
        size_t in = *size;
        MemWriter w(in ? path_or_buffer : nullptr, in);
        if (!serialize_range(c->store, 0, c->S, c->tick, c->last_row, w, st)) return KUN_INVALID_ARGUMENT;
        *size = w.pos;
        return w.pos > in ? KUN_INIT_ERROR : KUN_SUCCESS;
    }
    return KUN_INVALID_ARGUMENT;
}

KUN_EXPORT size_t kunQueryBufferHandle(KunStreamContextHandle context, const char *name) {
    StreamCtx *c = C(context);
    if (!c || !name) return (size_t)-1;
    for (int b = 0; b < c->m->num_buffers; b++)
        if (!strcmp(c->m->buffers[b].name, name)) return (size_t)b;
    set_error("Cannot find the buffer name");
    return (size_t)-1;
}

KUN_EXPORT const void *kunStreamGetCurrentBufferDevice(KunStreamContextHandle context, size_t h) {
    StreamCtx *c = C(context);
    if (!valid_handle(c, h)) return nullptr;
    size_t elem = elem_of(c->m);
    return (const char *)c->store.rings[h] + (size_t)c->last_row[h] * c->S * elem;
}

KUN_EXPORT const float *kunStreamGetCurrentBuffer(KunStreamContextHandle context, size_t h) {
    StreamCtx *c = C(context);
    if (!valid_handle(c, h)) return nullptr;
    size_t elem = elem_of(c->m);
    auto &mir = c->mirror[h];
    mir.resize((size_t)c->S * elem);
    cudaMemcpyAsync(mir.data(), kunStreamGetCurrentBufferDevice(context, h), mir.size(), cudaMemcpyDeviceToHost,
                    c->stream());
    if (cudaStreamSynchronize(c->stream()) != cudaSuccess) {
        set_error("CUDA error reading a stream buffer");
        return nullptr;
    }
    return (const float *)mir.data();
}

static KunStatus push(StreamCtx *c, size_t h, const void *src, cudaMemcpyKind kind) {
    if (!valid_handle(c, h) || !src) return KUN_INVALID_ARGUMENT;
    size_t elem = elem_of(c->m);
    int row = (int)(c->tick % win_of(c->m, (int)h));
    cudaError_t e = cudaMemcpyAsync((char *)c->store.rings[h] + (size_t)row * c->S * elem, src, (size_t)c->S * elem,
                                    kind, c->stream());
    if (e != cudaSuccess) {
        set_error("push failed: %s", cudaGetErrorString(e));
        return KUN_CUDA_ERROR;
    }
    c->last_row[h] = row;
    return KUN_SUCCESS;
}

KUN_EXPORT void kunStreamPushData(KunStreamContextHandle context, size_t h, const float *buffer) {
    push(C(context), h, buffer, cudaMemcpyDefault);
}

KUN_EXPORT KunStatus kunStreamPushDataDevice(KunStreamContextHandle context, size_t h, const void *device_buffer) {
    return push(C(context), h, device_buffer, cudaMemcpyDeviceToDevice);
}

KUN_EXPORT void kunStreamRun(KunStreamContextHandle context) {
    if (C(context)) ctx_run(C(context), true);
}

KUN_EXPORT KunStatus kunStreamRunEx(KunStreamContextHandle context, int synchronize) {
    if (!C(context)) return KUN_INVALID_ARGUMENT;
    return ctx_run(C(context), synchronize != 0);
}

KUN_EXPORT void kunDestoryStream(KunStreamContextHandle context) {
    StreamCtx *c = C(context);
    if (!c) return;
    cudaStreamSynchronize(c->stream());
    delete c;
}

// GPU extension: the number of ticks the stream has run.
KUN_EXPORT int64_t kunStreamTick(KunStreamContextHandle context) { return C(context) ? C(context)->tick : -1; }

// GPU extension: device bytes one stock of this stream module occupies.
KUN_EXPORT int64_t kunStreamBytesPerStock(KunModuleHandle m) {
    StreamStore s;
    s.m = (const KunGpuModuleDesc *)m;
    return (int64_t)s.bytes_per_stock();
}

// GPU extension: copy the current row of a buffer to device memory `dst`
// (num_stocks values), ordered after the stream's queued ticks.
KUN_EXPORT KunStatus kunStreamCopyCurrentDevice(KunStreamContextHandle context, size_t h, void *dst) {
    StreamCtx *c = C(context);
    if (!valid_handle(c, h) || !dst) return KUN_INVALID_ARGUMENT;
    size_t elem = elem_of(c->m);
    cudaError_t e = cudaMemcpyAsync(dst, kunStreamGetCurrentBufferDevice(context, h), (size_t)c->S * elem,
                                    cudaMemcpyDeviceToDevice, c->stream());
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream());
    if (e != cudaSuccess) {
        set_error("CUDA error: %s", cudaGetErrorString(e));
        return KUN_CUDA_ERROR;
    }
    return KUN_SUCCESS;
}
