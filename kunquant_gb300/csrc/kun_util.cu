// Utilities after the factor computation: corrWith / RankCorrWith (the
// cross-sectional correlation of every factor row with a label row, the IC)
// and aggregrate (per-stock group reductions over runs of equal labels).
// Reference: cpp/Kun/CorrWith.hpp:12-121, cpp/Kun/Aggregration.cpp:12-106,
// bound in Python at cpp/Python/PyBinding.cpp:396-506.
//
// corrWith: one block per (time row, input); the five moments are summed per
// thread over a strided share of the stocks in two-float compensated fp32,
// then tree-reduced.  The reference adds in stock order in plain fp32, so the
// results agree to rounding (its own tests hold 1e-4 relative to pandas).
// RankCorrWith first ranks each input row exactly as Rank does.
//
// aggregrate: one thread per (stock, input) walks the rows in order, with
// the reference's reductions (Kahan sum, NaN-sticky min/max), so the outputs
// are the reference's bits.
#include <cuda_runtime.h>

#include <cstring>
#include <vector>

#include "kun_runtime_internal.h"
#include "kun_xsec.cuh"

namespace kungpu {

constexpr int kCorrThreads = 256;

// element (t, s) of a [T][S] (layout 1) or [S/L][T][L] (layout 0) buffer
__device__ __forceinline__ long long util_index(int layout, long long s, long long t, long long S, long long T,
                                                int L) {
    return layout == 1 ? t * S + s : (s / L) * T * L + t * L + s % L;
}

__device__ __forceinline__ kun::DFloat warp_sum_df(kun::DFloat v) {
    for (int o = 16; o > 0; o >>= 1) {
        kun::DFloat w(__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o));
        v = kun::kadd(v, w);
    }
    return v;
}

// in[k] rows, y row source; out[k][t]
__global__ void __launch_bounds__(kCorrThreads) corr_rows(const float *const *in, const float *y, float *const *out,
                                                          long long S, long long T, int layout, int L) {
    const long long t = blockIdx.x;
    const int k = blockIdx.y;
    const float *x = in[k];
    kun::DFloat X, Y, X2, Y2, XY;
    for (long long s = threadIdx.x; s < S; s += blockDim.x) {
        const long long ix = util_index(layout, s, t, S, T, L);
        const float a = x[ix], b = y[ix];
        X = kun::df_add_f(X, a);
        Y = kun::df_add_f(Y, b);
        X2 = kun::df_add_prod(X2, a, a);
        Y2 = kun::df_add_prod(Y2, b, b);
        XY = kun::df_add_prod(XY, a, b);
    }
    __shared__ float sh[5][2][kCorrThreads / 32];
    kun::DFloat v[5] = {X, Y, X2, Y2, XY};
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < 5; q++) {
        v[q] = warp_sum_df(v[q]);
        if (lane == 0) {
            sh[q][0][w] = v[q].hi;
            sh[q][1][w] = v[q].lo;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        kun::DFloat r[5];
        for (int q = 0; q < 5; q++)
            for (int i = 0; i < kCorrThreads / 32; i++) r[q] = kun::kadd(r[q], kun::DFloat(sh[q][0][i], sh[q][1][i]));
        // moments in double from the two-float sums: x / S, then the
        // correlation (XY - X*Y) / (sqrt(X2 - X*X) * sqrt(Y2 - Y*Y))
        const double n = (double)S;
        const double mx = ((double)r[0].hi + r[0].lo) / n, my = ((double)r[1].hi + r[1].lo) / n;
        const double mx2 = ((double)r[2].hi + r[2].lo) / n, my2 = ((double)r[3].hi + r[3].lo) / n;
        const double mxy = ((double)r[4].hi + r[4].lo) / n;
        out[k][t] = (float)((mxy - mx * my) / (sqrt(mx2 - mx * mx) * sqrt(my2 - my * my)));
    }
}

template <typename T>
__global__ void aggregate_stocks(const T *__restrict__ in, const T *__restrict__ labels, T *const *outs,
                                 long long S, long long length) {
    const long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= S) return;
    T *sum = outs[0], *mn = outs[1], *mx = outs[2], *first = outs[3], *last = outs[4], *cnt = outs[5],
      *mean = outs[6];
    kun::RAdd<T> radd;
    kun::RMin<T> rmin;
    kun::RMax<T> rmax;
    T f = in[s], l = T(0), c = T(0);
    T last_label = labels[0];
    long long g = 0;
    auto store = [&]() {
        if (sum) sum[g * S + s] = radd.value();
        if (mn) mn[g * S + s] = rmin.value();
        if (mx) mx[g * S + s] = rmax.value();
        if (first) first[g * S + s] = f;
        if (last) last[g * S + s] = l;
        if (cnt) cnt[g * S + s] = c;
        if (mean) mean[g * S + s] = kun::kdiv(radd.value(), c);
    };
    for (long long i = 0; i < length; i++) {
        const T label = labels[i];
        const T cur = in[i * S + s];
        if (label != last_label) {
            store();
            g++;
            f = cur;
            radd = kun::RAdd<T>();
            rmin = kun::RMin<T>();
            rmax = kun::RMax<T>();
            c = T(0);
        }
        c = kun::kadd(c, T(1));
        l = cur;
        last_label = label;
        rmax.step(cur);
        rmin.step(cur);
        radd.step(cur);
    }
    store();
}

static KunStatus util_sync(Executor *ex, cudaStream_t st) {
    if (ex->has_user_stream) {
        cudaEventRecord(ex->bridge_out, st);
        cudaStreamWaitEvent(ex->user_stream, ex->bridge_out, 0);
    }
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        set_error("CUDA error: %s", cudaGetErrorString(e));
        return KUN_CUDA_ERROR;
    }
    return KUN_SUCCESS;
}

}  // namespace kungpu

using namespace kungpu;

// corrWith / RankCorrWith (GPU extension of the C API; the reference has it
// in C++ and Python).  inputs[n], corr_with and the n outputs (num_time
// floats each) are device memory; layout 1 = TS [T][S], 0 = STs [S/8][T][8].
KUN_EXPORT KunStatus kunCorrWith(KunExecutorHandle exec, int n, const float *const *inputs, const float *corr_with,
                                 float *const *outs, size_t num_stocks, size_t num_time, int layout,
                                 int rank_inputs) {
    clear_error();
    auto *ex = (Executor *)exec;
    if (!ex || n < 0 || (n > 0 && (!inputs || !outs)) || !corr_with) {
        set_error("corrWith: bad arguments");
        return KUN_INVALID_ARGUMENT;
    }
    if (n == 0) return KUN_SUCCESS;
    if (layout != 0 && layout != 1) {
        set_error("Unknown layout");
        return KUN_INVALID_ARGUMENT;
    }
    if (rank_inputs && layout != 1) {
        set_error("corrWith: rank_inputs needs the TS layout");
        return KUN_INVALID_ARGUMENT;
    }
    if (num_stocks == 0 || num_time == 0 || num_time > 0x7fffffff || n > 65535) {
        set_error("corrWith: bad shape");
        return KUN_INVALID_ARGUMENT;
    }
    std::lock_guard<std::mutex> lk(ex->mu);
    cudaSetDevice(ex->device);
    cudaStream_t st = ex->stream();
    if (ex->has_user_stream) {
        cudaEventRecord(ex->bridge_in, ex->user_stream);
        cudaStreamWaitEvent(st, ex->bridge_in, 0);
    }
    const size_t plane = num_stocks * num_time * sizeof(float);
    // device copies of the pointer arrays (and the ranked planes) in the arena
    size_t need = 2 * 256 + 2 * (size_t)n * sizeof(void *);
    if (rank_inputs) need += (size_t)n * ((plane + 255) / 256 * 256);
    if (!ex->arena.ensure(need)) {
        set_error("out of device memory for corrWith");
        return KUN_OUT_OF_MEMORY;
    }
    char *base = (char *)ex->arena.ptr;
    const float **d_in = (const float **)base;
    float **d_out = (float **)(base + (((size_t)n * sizeof(void *) + 255) / 256 * 256));
    char *ranked = base + 2 * (((size_t)n * sizeof(void *) + 255) / 256 * 256);
    std::vector<const float *> src(inputs, inputs + n);
    if (rank_inputs) {
        for (int k = 0; k < n; k++) {
            float *r = (float *)(ranked + (size_t)k * ((plane + 255) / 256 * 256));
            int rc = kun::launch_rank<float>(inputs[k], r, (long long)num_stocks, (long long)num_time, st);
            if (rc) {
                set_error("corrWith: rank failed: %s", cudaGetErrorString((cudaError_t)rc));
                return KUN_CUDA_ERROR;
            }
            src[k] = r;
        }
    }
    cudaMemcpyAsync(d_in, src.data(), (size_t)n * sizeof(void *), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(d_out, outs, (size_t)n * sizeof(void *), cudaMemcpyHostToDevice, st);
    corr_rows<<<dim3((unsigned)num_time, (unsigned)n), kCorrThreads, 0, st>>>(
        d_in, corr_with, d_out, (long long)num_stocks, (long long)num_time, layout, 8);
    if (cudaError_t e = cudaGetLastError()) {
        set_error("corrWith: %s", cudaGetErrorString(e));
        return KUN_CUDA_ERROR;
    }
    return util_sync(ex, st);
}

// aggregrate (GPU extension; PyBinding.cpp:449-506): for each of n inputs
// ([length][S], TS), labels[k] (length values) and outs[k*7 + kind] (kind =
// sum, min, max, first, last, count, mean; NULL to skip; [groups][S]).
// dtype 0 = float, 1 = double.  All pointers are device memory.
KUN_EXPORT KunStatus kunAggregrate(KunExecutorHandle exec, int n, const void *const *inputs,
                                   const void *const *labels, void *const *outs, size_t num_stocks, size_t length,
                                   int dtype) {
    clear_error();
    auto *ex = (Executor *)exec;
    if (!ex || n < 0 || (n > 0 && (!inputs || !labels || !outs)) || (dtype != 0 && dtype != 1)) {
        set_error("aggregrate: bad arguments");
        return KUN_INVALID_ARGUMENT;
    }
    if (n == 0) return KUN_SUCCESS;
    if (num_stocks == 0 || length == 0) {
        set_error("aggregrate: bad shape");
        return KUN_INVALID_ARGUMENT;
    }
    std::lock_guard<std::mutex> lk(ex->mu);
    cudaSetDevice(ex->device);
    cudaStream_t st = ex->stream();
    if (ex->has_user_stream) {
        cudaEventRecord(ex->bridge_in, ex->user_stream);
        cudaStreamWaitEvent(st, ex->bridge_in, 0);
    }
    if (!ex->arena.ensure((size_t)n * 7 * sizeof(void *) + 256)) {
        set_error("out of device memory for aggregrate");
        return KUN_OUT_OF_MEMORY;
    }
    void **d_outs = (void **)ex->arena.ptr;
    cudaMemcpyAsync(d_outs, outs, (size_t)n * 7 * sizeof(void *), cudaMemcpyHostToDevice, st);
    const unsigned grid = (unsigned)((num_stocks + 127) / 128);
    for (int k = 0; k < n; k++) {
        if (dtype == 0)
            aggregate_stocks<float><<<grid, 128, 0, st>>>((const float *)inputs[k], (const float *)labels[k],
                                                          (float *const *)(d_outs + 7 * k), (long long)num_stocks,
                                                          (long long)length);
        else
            aggregate_stocks<double><<<grid, 128, 0, st>>>((const double *)inputs[k], (const double *)labels[k],
                                                           (double *const *)(d_outs + 7 * k), (long long)num_stocks,
                                                           (long long)length);
    }
    if (cudaError_t e = cudaGetLastError()) {
        set_error("aggregrate: %s", cudaGetErrorString(e));
        return KUN_CUDA_ERROR;
    }
    return util_sync(ex, st);
}
