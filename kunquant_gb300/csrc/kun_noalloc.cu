// kunRunGraphNoAlloc: a batch run that allocates no device memory.
//
// The stage kernels of a batch module need device scratch: the temporaries
// between stages and the per-stage [length][num_stocks] materialisation
// buffers.  kunRunGraphEx takes them from an executor-owned arena grown with
// cudaMalloc.  Here they come from one file-scope __device__ array of
// KUN_NOALLOC_SCRATCH_BYTES, so the call makes no cudaMalloc/cudaFree and no
// call into an allocating library; it needs no executor either (creating one
// allocates).  Inputs and outputs must be device memory.
//
// Set-up: the first call on each device (with that device current) looks up
// the array's device address with cudaGetSymbolAddress; make that first call
// before any stream capture on the device.
//
// Concurrency: all calls on a device share the one array.  Calls whose GPU
// work overlaps (on different streams, or from several host threads without
// ordering) race on it and corrupt each other's results; order them on one
// stream or with events.
#include <cuda_runtime.h>

#include <cstring>
#include <map>
#include <mutex>
#include <tuple>

#include "kun_runtime_internal.h"

namespace kungpu {

// The temporaries and scratch slots of one run, slot after slot.
static __device__ __align__(256) unsigned char g_noalloc_scratch[KUN_NOALLOC_SCRATCH_BYTES];

static constexpr int kMaxDevices = 64;

// A cached plan, with the descriptor fields it was made from: a plan is
// reused only for the same module contents, and every plan is dropped when
// a library is unloaded (another one can then load at the same address).
struct CachedPlan {
    Plan plan;
    int num_buffers, num_stages, dtype;
    const void *stages, *buffers;
};

static std::mutex g_mu;
static void *g_base[kMaxDevices];
static std::map<std::tuple<const void *, long long, long long>, CachedPlan> g_plans;
static uint64_t g_plans_epoch = 0;

static bool on_device(const void *p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

static KunStatus no_alloc_run(const KunGpuModuleDesc *m, const NameMap &names, long long S, long long total_time,
                              long long cur_time, long long length, cudaStream_t st) {
    clear_error();
    if (!m) {
        set_error("null module");
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
        set_error("Bad shape: num_stocks %lld is not a multiple of %d", S, m->blocking_len);
        return KUN_INVALID_ARGUMENT;
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        cudaGetLastError();
        set_error("kunRunGraphNoAlloc: no usable current CUDA device");
        return KUN_CUDA_ERROR;
    }
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_base[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            set_error("kunRunGraphNoAlloc: cannot find the static scratch on device %d: %s", dev,
                      cudaGetErrorString(e));
            return KUN_CUDA_ERROR;
        }
        g_base[dev] = p;
    }
    char *base = (char *)g_base[dev];
    if (g_plans_epoch != library_epoch()) {
        g_plans.clear();
        g_plans_epoch = library_epoch();
    }
    auto key = std::make_tuple((const void *)m, S, length);
    auto it = g_plans.find(key);
    if (it != g_plans.end() &&
        (it->second.num_buffers != m->num_buffers || it->second.num_stages != m->num_stages ||
         it->second.dtype != m->dtype || it->second.stages != (const void *)m->stages ||
         it->second.buffers != (const void *)m->buffers)) {
        g_plans.erase(it);
        it = g_plans.end();
    }
    if (it == g_plans.end()) {
        CachedPlan c;
        if (!make_plan(m, S, length, 1, c.plan)) return KUN_INVALID_ARGUMENT;
        c.num_buffers = m->num_buffers;
        c.num_stages = m->num_stages;
        c.dtype = m->dtype;
        c.stages = m->stages;
        c.buffers = m->buffers;
        it = g_plans.emplace(key, std::move(c)).first;
    }
    const Plan &plan = it->second.plan;
    size_t need = plan.slot_bytes * (size_t)plan.num_slots;
    if (need > (size_t)KUN_NOALLOC_SCRATCH_BYTES) {
        set_error("kunRunGraphNoAlloc: module %s with %lld stocks x %lld time steps needs %zu bytes of scratch "
                  "(%d slots of %zu bytes); the static scratch holds %zu bytes. Use kunRunGraphEx, or fewer "
                  "stocks or time steps per call",
                  m->name, S, length, need, plan.num_slots, plan.slot_bytes, (size_t)KUN_NOALLOC_SCRATCH_BYTES);
        return KUN_OUT_OF_MEMORY;
    }
    std::vector<void *> ptrs(m->num_buffers, nullptr);
    for (int b = 0; b < m->num_buffers; b++) {
        const KunGpuBufferDesc &bd = m->buffers[b];
        if (bd.kind == KUN_BUF_TEMP) {
            if (plan.temp_slot[b] >= 0) ptrs[b] = base + plan.slot_bytes * (size_t)plan.temp_slot[b];
            continue;
        }
        auto f = names.find(bd.name);
        if (f == names.end() || !f->second) {
            set_error("Buffer name not found: %s", bd.name);
            return KUN_INVALID_ARGUMENT;
        }
        if (!on_device(f->second)) {
            set_error("kunRunGraphNoAlloc: buffer %s is not device memory", bd.name);
            return KUN_INVALID_ARGUMENT;
        }
        ptrs[b] = f->second;
    }
    // Nothing has to start at zero: every temporary and scratch slot is
    // written by its producer before any kernel reads it, so the contents a
    // previous call left behind are never seen.
    std::vector<void *> scratch;
    for (int si : plan.order) {
        const KunGpuStageDesc &s = m->stages[si];
        scratch.clear();
        for (int sl : plan.scratch[si]) scratch.push_back(base + plan.slot_bytes * (size_t)sl);
        KunGpuStageArgs a;
        memset(&a, 0, sizeof a);
        a.buffers = ptrs.data();
        a.scratch = scratch.data();
        a.num_stocks = S;
        a.total_time = total_time;
        a.start = cur_time;
        a.length = length;
        int rc = s.launch(&a, (void *)st);
        if (rc != 0) {
            set_error("stage %d (%s) launch failed: %s", si, s.name, cudaGetErrorString((cudaError_t)rc));
            return KUN_CUDA_ERROR;
        }
    }
    return KUN_SUCCESS;
}

}  // namespace kungpu

using namespace kungpu;

KUN_EXPORT KunStatus kunRunGraphNoAlloc(KunModuleHandle m, KunBufferNameMapHandle buffers, size_t num_stocks,
                                        size_t total_time, size_t cur_time, size_t length, void *cuda_stream) {
    if (!buffers) {
        set_error("null buffer map");
        return KUN_INVALID_ARGUMENT;
    }
    return no_alloc_run((const KunGpuModuleDesc *)m, *(const NameMap *)buffers, (long long)num_stocks,
                        (long long)total_time, (long long)cur_time, (long long)length, (cudaStream_t)cuda_stream);
}
