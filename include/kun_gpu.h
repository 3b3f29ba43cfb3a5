/*
 * kun_gpu.h -- C ABI of the GB300 backend of KunQuant.
 *
 * Drop-in for the reference C API (cpp/Kun/CApi.h): the same handles, the same
 * function names and argument meanings, so a C/Go/Rust/ctypes binding written
 * for KunQuant links against libkungpu.so unchanged.  Differences:
 *   - an "executor" is a CUDA execution context on the current device (one or
 *     more CUDA streams) instead of a CPU thread pool;
 *   - a "library" is a module library produced by the GPU code generator
 *     (kunquant_gb300.build.build_module_library, or the prebuilt
 *     Alpha101/Alpha158 ones);
 *   - buffers given to kunSetBufferNameMap may be host or device pointers;
 *     host buffers are copied to the device and back inside kunRunGraph;
 *   - every call reports errors through its return status and
 *     kunGetLastError() instead of C++ exceptions.
 * Functions below marked "GPU extension" have no counterpart in CApi.h.
 */
#ifndef KUN_GPU_H
#define KUN_GPU_H
#include <stddef.h>
#include <stdint.h>

typedef void *KunExecutorHandle;
typedef void *KunLibraryHandle;
typedef void *KunModuleHandle;
typedef void *KunBufferNameMapHandle;
typedef void *KunStreamContextHandle;
typedef void *KunServePoolHandle;

#ifdef __cplusplus
extern "C" {
#endif

#define KUN_API_VERSION 1

/* cpp/Kun/CApi.h:17-21 */
typedef enum {
    KUN_INIT_NONE = 0,
    KUN_INIT_FILE,
    KUN_INIT_MEMORY,
} KunStateBufferKind;

/* cpp/Kun/CApi.h:23-27, extended with GPU failure codes */
typedef enum {
    KUN_SUCCESS = 0,
    KUN_INIT_ERROR,
    KUN_INVALID_ARGUMENT,
    KUN_CUDA_ERROR,
    KUN_OUT_OF_MEMORY,
    KUN_TIMEOUT,
} KunStatus;

/* cpp/Kun/CApi.h:29-40 */
typedef struct {
    size_t version;
    KunStateBufferKind init_kind;
    union {
        const char *path;
        struct {
            const char *buffer;
            size_t size;
        } memory;
    } init;
} KunStreamExtraArgs;

/* Replaces kunCreateSingleThreadExecutor (cpp/Kun/CApi.h:48): a GPU executor
 * on the current CUDA device with one stream. */
KunExecutorHandle kunCreateSingleThreadExecutor(void);
/* Replaces kunCreateMultiThreadExecutor (cpp/Kun/CApi.h:57): `numthreads` is
 * the number of CUDA streams used to run independent stages concurrently. */
KunExecutorHandle kunCreateMultiThreadExecutor(int numthreads);
/* cpp/Kun/CApi.h:65 (sic: "Destory" as in the reference) */
void kunDestoryExecutor(KunExecutorHandle ptr);

/* cpp/Kun/CApi.h:73: load a GPU module library (.so) */
KunLibraryHandle kunLoadLibrary(const char *path_or_name);
/* cpp/Kun/CApi.h:82: borrowed handle, never freed */
KunModuleHandle kunGetModuleFromLibrary(KunLibraryHandle lib, const char *name);
/* cpp/Kun/CApi.h:90 */
void kunUnloadLibrary(KunLibraryHandle ptr);

/* cpp/Kun/CApi.h:98-125 */
KunBufferNameMapHandle kunCreateBufferNameMap(void);
void kunDestoryBufferNameMap(KunBufferNameMapHandle ptr);
void kunSetBufferNameMap(KunBufferNameMapHandle ptr, const char *name, float *buffer);
void kunEraseBufferNameMap(KunBufferNameMapHandle ptr, const char *name);

/* cpp/Kun/CApi.h:144: run the batch graph and wait for it.  Inputs are
 * [total_time][num_stocks] (TS) or [num_stocks/blocking][total_time][blocking]
 * (STs); outputs have `length` rows starting at `cur_time`.  Errors are
 * reported through kunGetLastError(). */
void kunRunGraph(KunExecutorHandle exec, KunModuleHandle m, KunBufferNameMapHandle buffers,
                 size_t num_stocks, size_t total_time, size_t cur_time, size_t length);

/* cpp/Kun/CApi.h:153-170 */
KunStreamContextHandle kunCreateStream(KunExecutorHandle exec, KunModuleHandle m, size_t num_stocks);
KunStatus kunCreateStreamEx(KunExecutorHandle exec, KunModuleHandle m, size_t num_stocks,
                            const KunStreamExtraArgs *extra_args, KunStreamContextHandle *out_handle);
/* cpp/Kun/CApi.h:190: two-phase size query as in the reference */
KunStatus kunStreamSerializeStates(KunStreamContextHandle context, KunStateBufferKind dump_kind,
                                   char *path_or_buffer, size_t *size);
/* cpp/Kun/CApi.h:205 */
size_t kunQueryBufferHandle(KunStreamContextHandle context, const char *name);
/* cpp/Kun/CApi.h:216: host copy of the buffer's current row, valid until the
 * next kunStreamPushData / kunStreamRun */
const float *kunStreamGetCurrentBuffer(KunStreamContextHandle context, size_t handle);
/* cpp/Kun/CApi.h:227: host data, num_stocks values */
void kunStreamPushData(KunStreamContextHandle context, size_t handle, const float *buffer);
/* cpp/Kun/CApi.h:235 */
void kunStreamRun(KunStreamContextHandle context);
/* cpp/Kun/CApi.h:241 */
void kunDestoryStream(KunStreamContextHandle context);

/* ---------------- GPU extensions ---------------- */

/* Status-returning kunRunGraph.  With `synchronize` = 0 and device buffers the
 * call only enqueues work on the executor's stream (and may be captured into
 * a CUDA graph). */
KunStatus kunRunGraphEx(KunExecutorHandle exec, KunModuleHandle m, KunBufferNameMapHandle buffers,
                        size_t num_stocks, size_t total_time, size_t cur_time, size_t length,
                        int synchronize);
/* Order the executor's work after and before the caller's CUDA stream
 * (cudaStream_t; 0 is the legacy default stream): runs start when the work
 * already queued on that stream is done, and later work on that stream waits
 * for the run.  The executor still computes on its own streams. */
KunStatus kunExecutorSetStream(KunExecutorHandle exec, void *cuda_stream);
/* Stop ordering with the caller's stream. */
KunStatus kunExecutorClearStream(KunExecutorHandle exec);
KunStatus kunExecutorSynchronize(KunExecutorHandle exec);
/* Record a CUDA event after every stage launch of the following runs (1) or
 * stop (0); kunExecutorStageTimes returns the per-stage milliseconds of the
 * last run (stage ids in launch order), or -1 when profiling is off. */
KunStatus kunExecutorSetProfiling(KunExecutorHandle exec, int enable);
int kunExecutorStageTimes(KunExecutorHandle exec, int32_t *stage_ids, float *ms, int cap);
/* Replay repeated runs (same module, shape and buffers) from a captured CUDA
 * graph (1, the default) or always enqueue kernel by kernel (0). */
KunStatus kunExecutorSetGraphs(KunExecutorHandle exec, int enable);
/* Count of kernel launches of the last run (for instrumentation). */
int64_t kunExecutorLastLaunchCount(KunExecutorHandle exec);
/* Text of the last error of the calling thread ("" if none). */
const char *kunGetLastError(void);

/* Module metadata (cpp/Python/PyBinding.cpp:182-221 exposes the same). */
int kunModuleNumBuffers(KunModuleHandle m);
const char *kunModuleBufferName(KunModuleHandle m, int idx);
int kunModuleBufferKind(KunModuleHandle m, int idx);        /* 0 input, 1 output, 2 temp */
int kunModuleBufferUnreliableCount(KunModuleHandle m, int idx);
int kunModuleBufferWindow(KunModuleHandle m, int idx);
int kunModuleInputLayout(KunModuleHandle m);                /* 0 STs, 1 TS, 2 STREAM */
int kunModuleOutputLayout(KunModuleHandle m);
int kunModuleBlockingLen(KunModuleHandle m);
int kunModuleDtype(KunModuleHandle m);                      /* 0 float, 1 double */
int kunModuleNumStages(KunModuleHandle m);

/* Stream sessions on device buffers (GPU extension of the stream API):
 * push a device row / read the device pointer of the current row. */
KunStatus kunStreamPushDataDevice(KunStreamContextHandle context, size_t handle, const void *device_buffer);
const void *kunStreamGetCurrentBufferDevice(KunStreamContextHandle context, size_t handle);
KunStatus kunStreamRunEx(KunStreamContextHandle context, int synchronize);
/* Many universes in one run (GPU extension; the reference runs one runGraph
 * per universe): `njobs` jobs of module m, each with its own buffer map (device
 * memory), stock count and time range.  Time-series stages run each kernel
 * once over the tiles of all jobs; the others run job by job.  Waits for the
 * work before returning. */
KunStatus kunRunGraphBatch(KunExecutorHandle exec, KunModuleHandle m, int njobs,
                           const KunBufferNameMapHandle *buffers, const size_t *num_stocks,
                           const size_t *total_time, const size_t *cur_time, const size_t *length,
                           int synchronize);
/* Autotuner (GPU extension): time candidate launch shapes (time tile x
 * threads per block, and per time-parallel kernel its instance compiled for
 * 64 registers a thread) of every time-series stage on these jobs and keep
 * the fastest per stage; the executor then uses them for this module in
 * kunRunGraphBatch and kunRunGraphEx.  Computes the jobs' outputs on the way.
 * Returns the number of stages tuned, -1 on error. */
int kunExecutorTune(KunExecutorHandle exec, KunModuleHandle m, int njobs, const KunBufferNameMapHandle *buffers,
                    const size_t *num_stocks, const size_t *total_time, const size_t *cur_time,
                    const size_t *length, int reps);
/* Tuned shape of one stage (kernel count, 0 if untuned) and clearing it.
 * A block entry or'd with KUN_BLOCK_REGCAP names the 64-register instance. */
#define KUN_BLOCK_REGCAP 0x10000
int kunExecutorTunedShape(KunExecutorHandle exec, KunModuleHandle m, int stage, int32_t *tile, int32_t *block,
                          int cap);
KunStatus kunExecutorClearTuning(KunExecutorHandle exec);

/* corrWith / RankCorrWith (GPU extension; the reference has them in C++ and
 * Python, cpp/Kun/CorrWith.hpp): for each of n inputs, out[k][t] = the
 * correlation across stocks of inputs[k] row t with corr_with row t (with
 * rank_inputs, of the input's cross-sectional rank).  Device memory; layout
 * 1 = TS [T][S], 0 = STs [S/8][T][8] (TS only with rank_inputs). */
KunStatus kunCorrWith(KunExecutorHandle exec, int n, const float *const *inputs, const float *corr_with,
                      float *const *outs, size_t num_stocks, size_t num_time, int layout, int rank_inputs);
/* aggregrate (GPU extension, cpp/Kun/Aggregration.cpp; the reference's
 * spelling): per stock, reductions over runs of equal consecutive labels.
 * outs[k*7 + kind], kind = sum, min, max, first, last, count, mean (NULL to
 * skip), each [groups][S]; dtype 0 float, 1 double; device memory. */
KunStatus kunAggregrate(KunExecutorHandle exec, int n, const void *const *inputs, const void *const *labels,
                        void *const *outs, size_t num_stocks, size_t length, int dtype);

/* Batch run that allocates no device memory; no counterpart in the reference.
 * For callers that cannot call cudaMalloc (an allocator-owning host process,
 * code between allocator checkpoints): temporaries and scratch come from a
 * static device array of KUN_NOALLOC_SCRATCH_BYTES inside libkungpu.so, and
 * no executor is needed.  Every buffer in the map must be device memory.  The
 * work is enqueued on `cuda_stream` (0 = legacy default stream) and the call
 * returns without waiting.  A run whose scratch would not fit is rejected
 * with KUN_OUT_OF_MEMORY and a message giving the bytes it needs.  The first
 * call on each device does a one-time set-up (address lookup of the static
 * array) and should come before any stream capture on that device.  All calls
 * on a device share the array: calls whose GPU work overlaps race and must be
 * ordered by the caller (one stream, or events).
 * Fixed cost: the array is device memory of the translation unit that holds
 * it.  With CUDA's default lazy module loading it is reserved on a device at
 * the first kunRunGraphNoAlloc call there; with CUDA_MODULE_LOADING=EAGER,
 * every process that loads libkungpu.so holds it on every device it uses,
 * until exit, whether it calls this function or not.  Memory budgets (the
 * serving pool's hbm budget, for one) should be measured after that. */
#define KUN_NOALLOC_SCRATCH_BYTES (64u << 20)
KunStatus kunRunGraphNoAlloc(KunModuleHandle m, KunBufferNameMapHandle buffers, size_t num_stocks,
                             size_t total_time, size_t cur_time, size_t length, void *cuda_stream);
/* Copy the current row of a buffer (num_stocks values) to device memory. */
KunStatus kunStreamCopyCurrentDevice(KunStreamContextHandle context, size_t handle, void *device_dst);
/* Ticks the stream has run (the time index of the next pushed row). */
int64_t kunStreamTick(KunStreamContextHandle context);
/* Device bytes one stock of a stream module holds (rings and op states). */
int64_t kunStreamBytesPerStock(KunModuleHandle m);

/* Serving pool (GPU extension; the reference runs one StreamContext per
 * session).  Sessions of one stream module share one device store of
 * `capacity_stocks` columns; a session keeps a contiguous column range, with
 * its rings and op states resident, until it is closed.  A step advances any
 * set of sessions by one tick each in one graph launch.
 *
 * Step data is laid out by column: inputs [num_inputs][capacity_stocks] and
 * outputs [num_outputs][capacity_stocks] (buffers in module order); session
 * s reads and writes columns [kunServeSessionColumn(s), + its stocks).  With
 * `device_inputs` / `device_outputs` NULL the pool's pinned host tables
 * (kunServeHostInputs/Outputs) are used, otherwise they are device tables of
 * the same layout.  Only the column span of the step's sessions is copied. */
KunStatus kunCreateServePool(KunExecutorHandle exec, KunModuleHandle m, size_t capacity_stocks, int max_sessions,
                             int max_session_stocks, KunServePoolHandle *out);
void kunDestroyServePool(KunServePoolHandle pool);
/* KUN_OUT_OF_MEMORY when no slot or no free column range fits: retry after a close */
KunStatus kunServeOpen(KunServePoolHandle pool, size_t num_stocks, int64_t *session_id);
KunStatus kunServeClose(KunServePoolHandle pool, int64_t session_id);
KunStatus kunServeStep(KunServePoolHandle pool, int num_sessions, const int64_t *session_ids,
                       const void *device_inputs, void *device_outputs);
/* Request loop (continuous batching): after kunServeStart, clients write a
 * session's input columns, kunServeSubmit it and kunServeWait for its tick;
 * each step takes every session submitted so far (after `batch_window_us`),
 * so ticks that arrive while a step is on the GPU go into the next one.  A
 * session has at most one tick in flight.  kunServeStep is for use without
 * the loop. */
KunStatus kunServeStart(KunServePoolHandle pool, int batch_window_us);
KunStatus kunServeStop(KunServePoolHandle pool);
KunStatus kunServeSubmit(KunServePoolHandle pool, int num_sessions, const int64_t *session_ids);
KunStatus kunServeWait(KunServePoolHandle pool, int64_t session_id, int64_t min_tick, int timeout_ms);
int kunServeTakeLatencies(KunServePoolHandle pool, float *latency_us, int cap, int32_t *step_sizes, int step_cap,
                          int *num_steps);
void *kunServeHostInputs(KunServePoolHandle pool);
void *kunServeHostOutputs(KunServePoolHandle pool);
int64_t kunServeSessionTick(KunServePoolHandle pool, int64_t session_id);
int64_t kunServeSessionStocks(KunServePoolHandle pool, int64_t session_id);
int64_t kunServeSessionColumn(KunServePoolHandle pool, int64_t session_id);
KunStatus kunServeFreeStocks(KunServePoolHandle pool, int64_t *total, int64_t *largest);
/* device bytes of a pool of `capacity_stocks` columns (store + packed rows) */
int64_t kunServePoolBytes(KunModuleHandle m, size_t capacity_stocks);

#ifdef __cplusplus
}
#endif
#endif
