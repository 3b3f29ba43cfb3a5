// ABI between the runtime (libkungpu.so) and the module libraries the code
// generator emits.  A module library exports one `KunGpuModuleDesc` per
// module, named `kun_module_<module name>`; this mirrors the reference's
// `Module` table (cpp/Kun/Module.hpp:16-28, cpp/Kun/Stage.hpp:26-66), with CUDA
// launch functions in place of the CPU stage functions.
#pragma once
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define KUN_GPU_MODULE_ABI 0x6b470009ull
#define KUN_BLOCK_REGCAP 0x10000

typedef enum { KUN_LAYOUT_STS = 0, KUN_LAYOUT_TS = 1, KUN_LAYOUT_STREAM = 2 } KunGpuLayout;
typedef enum { KUN_BUF_INPUT = 0, KUN_BUF_OUTPUT = 1, KUN_BUF_TEMP = 2 } KunGpuBufferKind;
typedef enum { KUN_STAGE_TS = 0, KUN_STAGE_RANK = 1, KUN_STAGE_SCALE = 2, KUN_STAGE_XSEC = 3 } KunGpuStageKind;

typedef struct {
    int32_t id;
    const char *name;
    int32_t kind;              /* KunGpuBufferKind */
    int32_t num_users;
    int32_t unreliable_count;  /* rows at the start of a run that are not reliable */
    int32_t window;            /* ring depth in stream mode */
} KunGpuBufferDesc;

/* Arguments of one stage launch.  `buffers` is indexed by module buffer id and
 * holds device pointers; `scratch` holds the stage's private [length][S]
 * device buffers (one per in-stage windowed temporary).  In stream mode
 * `buffers[b]` points at buffer b's ring ([window][S]) and `ring_pos` at the
 * per-buffer write positions. */
typedef struct {
    void *const *buffers;
    void *const *scratch;
    int64_t num_stocks;
    int64_t total_time;
    int64_t start;
    int64_t length;
    const int32_t *ring_pos;   /* unused */
    void *state;               /* stream mode: the stage's float/double state arrays */
    /* device word a kernel sets (to 1) when one of its bounded waits for a
     * bulk copy runs out, instead of hanging; the runtime reads it after a
     * run (NULL: not reported) */
    int32_t *error_flag;
    /* stream mode: stocks live in rings of num_stocks (capacity) columns; a
     * launch covers `nseg` segments (sessions): segment k holds stocks
     * [seg_stock0[k], seg_stock0[k] + seg_off[k+1] - seg_off[k]) and is at
     * tick seg_tick[k]; all three arrays are device memory */
    void *state_i;             /* stream mode: the stage's int32 state arrays */
    const int32_t *seg_off;
    const int32_t *seg_stock0;
    const int64_t *seg_tick;
    int32_t nseg;
    int64_t n_active;          /* seg_off[nseg] */
    int32_t max_seg_len;       /* longest segment (cross-sectional stages) */
    /* stream mode, optional: device int32[3] = {nseg, n_active, max_seg_len}.
     * When set, the kernels take the counts from here and the three host
     * fields above are upper bounds that size the grids, so one captured
     * graph serves any batch of segments within those bounds. */
    const int32_t *seg_count;
    /* optional per-kernel launch shape of a time-series stage (num_kernels
     * entries, 0 = default): time tile in rows (a multiple of 4) and threads
     * per block (at most 128), or'd with KUN_BLOCK_REGCAP to launch the
     * time-parallel kernel's instance compiled for 64 registers a thread */
    const int32_t *tune_tile;
    const int32_t *tune_block;
} KunGpuStageArgs;

typedef int (*KunGpuLaunchFn)(const KunGpuStageArgs *args, void *cuda_stream);
/* grouped launches over `njobs` jobs (args[0..njobs)): prepare() writes the
 * jobs' parameter blocks to `host` (when not NULL) and returns their size;
 * launch_group() runs every kernel of the stage once over all jobs, reading
 * the blocks from device memory `dev` */
typedef size_t (*KunGpuPrepareFn)(const KunGpuStageArgs *args, int32_t njobs, void *host);
typedef int (*KunGpuGroupLaunchFn)(const KunGpuStageArgs *args, int32_t njobs, const void *dev, void *cuda_stream);

typedef struct {
    const char *name;
    int32_t kind;              /* KunGpuStageKind */
    int32_t num_in;
    const int32_t *in_bufs;
    int32_t num_out;
    const int32_t *out_bufs;
    int32_t num_deps;          /* stages that depend on this one */
    const int32_t *deps;
    int32_t pending;           /* number of stages this one waits for */
    int32_t num_scratch;       /* private [length][S] buffers needed */
    int64_t state_bytes_per_stock; /* stream mode persistent state */
    KunGpuLaunchFn launch;
    int32_t num_kernels;       /* CUDA kernels one launch enqueues */
    /* stream mode: persistent state per stock and its initialiser, which
     * resets stocks [seg_stock0[0], seg_stock0[0] + n_active) */
    int32_t state_t_vars;      /* float/double arrays of num_stocks */
    int32_t state_i_vars;      /* int32 arrays of num_stocks */
    KunGpuLaunchFn init;
    /* per int32 state array: the largest value a restored state may hold
     * (valid values are 0..max), or -1 where any value is safe (tick
     * indices); the runtime checks restored dumps against it before any
     * kernel reads them.  NULL when state_i_vars is 0. */
    const int32_t *state_i_max;
    /* time-series stages with grouped launches: per kernel, default time
     * tile << 1 (or number of scan roles << 1) | 1 for a scan kernel */
    const int32_t *kernel_info;
    KunGpuPrepareFn prepare;
    KunGpuGroupLaunchFn launch_group;
} KunGpuStageDesc;

typedef struct {
    uint64_t abi;              /* KUN_GPU_MODULE_ABI */
    const char *name;
    int32_t num_stages;
    const KunGpuStageDesc *stages;
    int32_t num_buffers;
    const KunGpuBufferDesc *buffers;
    int32_t input_layout;      /* KunGpuLayout */
    int32_t output_layout;
    int32_t blocking_len;
    int32_t dtype;             /* 0 = float, 1 = double */
    int32_t aligned;
} KunGpuModuleDesc;

#ifdef __cplusplus
}
#endif
