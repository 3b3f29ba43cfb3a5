/*
 * CPU restatement of KunQuant's factor-graph executor -- TEST INFRASTRUCTURE.
 *
 * This library is the parity checker for the GPU backend.  It is never part of
 * the product path: only tests/, the smoke check and the CPU-baseline leg of
 * bench.py load it.
 *
 * It interprets the post-partition stage graphs ("module specs") with the
 * semantics of the reference C++ templates, one scalar lane at a time:
 *   - batch executor: kun::runGraph (cpp/Kun/Runtime.cpp:311-352), per-stage
 *     loop nest of KunQuant/passes/CodegenCpp.py:140-307;
 *   - op templates: cpp/Kun/Ops.hpp, cpp/Kun/Ops/Quantile.hpp,
 *     cpp/Kun/SkipList.cpp, cpp/Kun/Rank.hpp, cpp/Kun/Scale.hpp;
 *   - SIMD semantics: cpp/KunSIMD/cpu/x86/f32x8.hpp (ordered compares,
 *     blend-by-sign-bit select, max/min as a>b?a:b), log/exp of
 *     cpp/KunSIMD/cpu/Math.hpp.
 * Parity is pinned against outputs of the reference itself (oracle/_ref, see
 * tests/golden/make_golden.py).
 */
#ifndef KUNORACLE_H
#define KUNORACLE_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* opcodes; kept in sync with oracle/oracle.py */
enum {
    KO_INPUT = 1, KO_OUTPUT, KO_WTEMP, KO_CONST,
    KO_ADD, KO_SUB, KO_MUL, KO_DIV, KO_MAX, KO_MIN, KO_OR, KO_AND,
    KO_GT, KO_GE, KO_LT, KO_LE, KO_EQ,
    KO_ADDC, KO_SUBC, KO_MULC, KO_DIVC, KO_GTC, KO_LTC,
    KO_SQRT, KO_LOG, KO_ABS, KO_SIGN, KO_NOT, KO_EXP, KO_SETINFNAN,
    KO_SELECT, KO_LOOP, KO_ITER, KO_LOOPIDX,
    KO_RADD, KO_RMUL, KO_RMIN, KO_RMAX, KO_RARGMAX, KO_RARGMIN, KO_RRANK, KO_RDECAY,
    KO_BACKREF, KO_FWSUM, KO_EMA, KO_LINREG, KO_LR_RSQ, KO_LR_SLOPE, KO_LR_RESI,
    KO_SKIPLIST, KO_SL_QUANTILE, KO_SL_RANK, KO_SL_MIN, KO_SL_MAX, KO_SL_ARGMIN,
    KO_ACC, KO_SETACC, KO_RETFIRST,
    KO_RANK, KO_SCALE, KO_DIFFWSUM,
    KO_NUM_OPS
};

typedef struct {
    int32_t kind;
    int32_t nin;
    int32_t in[3];
    int32_t parent;       /* loop op index within the stage, or -1 */
    int32_t window;
    int32_t seg_end;
    int32_t copy_prev;
    int32_t buf;          /* buffer id for Input/Output ops, -1 otherwise */
    int32_t single_value;
    int32_t swap;
    int32_t loop_window;  /* window used by WindowLoopIndex */
    int32_t fast_log;
    /* multiply-add contraction of the reference build: input `fma_pos` of
     * this op is a product fma_a * fma_b (fma_b < 0: times the constant
     * fma_c) evaluated with a single rounding */
    int32_t fma_pos;
    int32_t fma_a;
    int32_t fma_b;
    int32_t unrolled;     /* reduction whose own loop the reference build fully unrolls */
    int32_t first_iter;   /* first iteration index of that reduction */
    int32_t shared_sq;    /* regression whose input feeds another regression of the stage */
    char fma_c[40];
    char cval[40];        /* decimal text of the constant ("value" attr) */
    char qval[40];        /* decimal text of "q" */
} KOOp;

typedef struct {
    int32_t kind;   /* 0 = time series, 1 = rank, 2 = scale, 3 = diff-with-weighted-sum */
    int32_t nops;
    const KOOp *ops;
} KOStage;

/* buffers[b] points at buffer b: user inputs have total_time rows (and are
 * read from row cur_time on), outputs and temps have `length` rows; rows are
 * num_stocks wide ([T][S]).  single_value inputs are one row.  Returns 0 on
 * success, a negative code on an unsupported graph. */
int ko_run_f32(const KOStage *stages, int nstages, float **buffers, const int32_t *buf_is_input,
               int64_t num_stocks, int64_t total_time, int64_t cur_time, int64_t length,
               int nthreads);
int ko_run_f64(const KOStage *stages, int nstages, double **buffers, const int32_t *buf_is_input,
               int64_t num_stocks, int64_t total_time, int64_t cur_time, int64_t length,
               int nthreads);

/* element-wise helpers exposed for unit tests of the restated math */
void ko_logfast_f32(const float *x, float *y, int64_t n);
void ko_exp_f32(const float *x, float *y, int64_t n);
void ko_logfast_f64(const double *x, double *y, int64_t n);
void ko_exp_f64(const double *x, double *y, int64_t n);
const char *ko_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
