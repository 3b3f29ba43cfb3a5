/*
 * CPU restatement of KunQuant's factor-graph executor -- TEST INFRASTRUCTURE.
 * See kunoracle.h.  Built by oracle/oracle.py with
 *   gcc -O2 -fopenmp -ffp-contract=off -fno-fast-math -shared -fPIC
 * (no contraction: the reference is built -std=c++11, i.e. ISO mode, where
 * GCC does not fuse a*b+c; explicit FMAs are written as fma()).
 */
#include "kunoracle.h"
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static __thread char g_err[256];
static void set_err(const char *m) { snprintf(g_err, sizeof g_err, "%s", m); }
const char *ko_last_error(void) { return g_err; }

#define T float
#define UT uint32_t
#define ST int32_t
#define SFX(n) n##_f32
#define MANT_BITS 23
#define EXP_BITS 8
#define FMA(a, b, c) fmaf(a, b, c)
#define SQRT(a) sqrtf(a)
#define FLOOR(a) floorf(a)
#define LOG(a) logf(a)
#define KO_IS_FLOAT 1
#include "kunoracle_impl.h"
#undef T
#undef UT
#undef ST
#undef SFX
#undef MANT_BITS
#undef EXP_BITS
#undef FMA
#undef SQRT
#undef FLOOR
#undef LOG
#undef KO_IS_FLOAT

#define T double
#define UT uint64_t
#define ST int64_t
#define SFX(n) n##_f64
#define MANT_BITS 52
#define EXP_BITS 11
#define FMA(a, b, c) fma(a, b, c)
#define SQRT(a) sqrt(a)
#define FLOOR(a) floor(a)
#define LOG(a) log(a)
#include "kunoracle_impl.h"

int ko_run_f32(const KOStage *stages, int nstages, float **buffers, const int32_t *is_in,
               int64_t S, int64_t total_time, int64_t cur_time, int64_t length, int nthreads) {
    return run_all_f32(stages, nstages, buffers, is_in, S, total_time, cur_time, length, nthreads);
}
int ko_run_f64(const KOStage *stages, int nstages, double **buffers, const int32_t *is_in,
               int64_t S, int64_t total_time, int64_t cur_time, int64_t length, int nthreads) {
    return run_all_f64(stages, nstages, buffers, is_in, S, total_time, cur_time, length, nthreads);
}
void ko_logfast_f32(const float *x, float *y, int64_t n) { logfast_arr_f32(x, y, n); }
void ko_exp_f32(const float *x, float *y, int64_t n) { exp_arr_f32(x, y, n); }
void ko_logfast_f64(const double *x, double *y, int64_t n) { logfast_arr_f64(x, y, n); }
void ko_exp_f64(const double *x, double *y, int64_t n) { exp_arr_f64(x, y, n); }
