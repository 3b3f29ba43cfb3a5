/*
 * Type-generic body of the oracle interpreter.  Included twice by
 * kunoracle.c, with T = float and T = double.  TEST INFRASTRUCTURE ONLY.
 *
 * Required macros: T, UT (same-width unsigned int), ST (same-width signed
 * int), SFX(name), MANT_BITS, EXP_BITS, FMA(a,b,c), SQRT, FLOOR, LOG.
 */

static inline UT SFX(bits)(T x) { UT u; memcpy(&u, &x, sizeof u); return u; }
static inline T SFX(from_bits)(UT u) { T x; memcpy(&x, &u, sizeof x); return x; }
static inline T SFX(mask)(int b) { return b ? SFX(from_bits)((UT)~(UT)0) : (T)0; }
static inline int SFX(sel)(T c) { return (int)(SFX(bits)(c) >> (sizeof(UT) * 8 - 1)); }

static T SFX(r_table)[32];
static T SFX(logr_table)[32];

/* Reciprocal table of the table-driven log (cpp/KunSIMD/cpu/Math.hpp:20-93,
 * tables in cpp/KunSIMD/cpu/tables.cpp): entry i approximates 1/M for the
 * mantissa bin selected by the top 5 mantissa bits.  Bins 0-15 hold
 * M in [1, 1.5) and are rounded to a 1/32 grid; bins 16-31 hold M in
 * [0.75, 1) (exponent lowered by one) and are rounded to a 1/16 grid.
 * logr = -log(R) - bias*ln2 with bias 127 / 1023 folds the exponent bias. */
static void SFX(init_tables)(void) {
    int bias = (1 << (EXP_BITS - 1)) - 1;
    for (int i = 0; i < 32; i++) {
        double m, g;
        if (i < 16) { m = 1.0 + (i + 0.5) / 32.0; g = 32.0; }
        else { m = 0.5 * (1.0 + (i + 0.5) / 32.0); g = 16.0; }
        double r = floor(g / m + 0.5) / g;
        SFX(r_table)[i] = (T)r;
        double shift = -log(2.0) * bias;
        SFX(logr_table)[i] = (T)(-log(r) + shift);
    }
}

/* kun_simd::log, cpp/KunSIMD/cpu/Math.hpp:20-93 */
static T SFX(logfast)(T x) {
    const int mb = MANT_BITS, eb = EXP_BITS;
    UT xi = SFX(bits)(x);
    UT high5 = (xi >> (mb - 5)) & (UT)31;
    UT high1 = high5 >> 4;
    UT e1 = (high1 ^ (((UT)1 << (eb - 1)) - 1)) << mb;
    UT m = (xi & ((((UT)1) << mb) - 1)) | e1;
    T ri = SFX(r_table)[high5];
    /* the reference build contracts `Ri * M - 1` and both uses of
     * `poly * Z` into FMAs (GCC fuses a product whose only uses are
     * additions/subtractions in the same basic block) */
    T z = FMA(ri, SFX(from_bits)(m), (T)-1.0);
    T poly = (T)(1 / 5.0);
    poly = FMA(poly, z, (T)(-1 / 4.0));
    poly = FMA(poly, z, (T)(1 / 3.0));
    poly = FMA(poly, z, (T)(-1 / 2.0));
    poly = FMA(poly, z, (T)1.0);
    T mlog = SFX(logr_table)[high5];
    UT er = (xi >> mb) + high1;
    T ep = (T)(ST)er;
    T v2 = FMA(ep, (T)0.6931471805599453, mlog);
    T hi = FMA(poly, z, v2);
    T lo = hi - v2;
    lo = FMA(-poly, z, lo);
    hi = hi + lo;
    if (x == (T)0) hi = -(T)INFINITY;
    if (x < (T)0) hi = (T)NAN;
    if (x == (T)INFINITY) hi = (T)INFINITY;
    if (x != x) hi = (T)NAN;
    if (x == (T)1.0) hi = (T)0;
    return hi;
}

/* kun_simd::exp, cpp/KunSIMD/cpu/Math.hpp:96-140 (float thresholds for both
 * types, as in the reference) */
static T SFX(expk)(T x) {
    T k = FLOOR(FMA(x, (T)1.4426950408889634, (T)0.5));
    ST ki;
    if (k != k || k > (T)1e9 || k < (T)-1e9) ki = 0; else ki = (ST)k;
    T r = FMA(-k, (T)0.6931471805599453, x);
    T tn = FMA(r, (T)0.16666666666666666, (T)1.0);
    tn = FMA(tn, r * (T)0.2, (T)1.0);
    tn = FMA(tn, r * (T)0.25, (T)1.0);
    tn = FMA(tn, r * (T)0.3333333333333333, (T)1.0);
    tn = FMA(tn, r * (T)0.5, (T)1.0);
    tn = FMA(tn, r, (T)1.0);
    UT p = ((UT)ki) << MANT_BITS;
    T res = SFX(from_bits)(p + SFX(bits)(tn));
    if (x > (T)88.72283935) res = (T)INFINITY;
    if (x < (T)-87.33654785) res = (T)0;
    return res;
}

/* ---------- skip-list state (cpp/Kun/Ops/Quantile.hpp:16-45,
 * cpp/Kun/SkipList.cpp:125-273), restated as a sorted array per lane.
 * Equal values keep insertion order: insert goes after equals, remove takes
 * the first equal. ---------- */
typedef struct {
    double *v;
    int64_t *idx;
    int size;
    int last_rank;
} SFX(SkipLane);

static int SFX(sl_insert)(SFX(SkipLane) *s, double value, int64_t index) {
    int p = 0;
    while (p < s->size && s->v[p] <= value) p++;
    for (int j = s->size; j > p; j--) { s->v[j] = s->v[j - 1]; s->idx[j] = s->idx[j - 1]; }
    s->v[p] = value;
    s->idx[p] = index;
    s->size++;
    return p;
}
static void SFX(sl_remove)(SFX(SkipLane) *s, double value) {
    int p = 0;
    while (p < s->size && s->v[p] < value) p++;
    if (p >= s->size || s->v[p] != value) return;
    for (int j = p; j < s->size - 1; j++) { s->v[j] = s->v[j + 1]; s->idx[j] = s->idx[j + 1]; }
    s->size--;
}
static int SFX(sl_minrank)(const SFX(SkipLane) *s, double value) {
    int p = 0;
    while (p < s->size && s->v[p] < value) p++;
    return p;
}

/* per-op runtime storage of one stock block */
typedef struct {
    T *val;          /* [nops][L] current values */
    T **st;          /* per-op float state arrays */
    int32_t **sti;   /* per-op int state arrays */
    SFX(SkipLane) **sl;
} SFX(Block);

typedef struct {
    const KOStage *stage;
    int *is_top;
    int **loop_body;     /* loop op -> list of ops to evaluate per iteration */
    int *loop_body_n;
    int **loop_red;      /* loop op -> list of reductions stepped per iteration */
    int *loop_red_n;
    int **loop_own_red;  /* loop op -> reductions initialised before it */
    int *loop_own_red_n;
    T *cst;              /* parsed "value" attr per op */
    T *qv;               /* parsed "q" attr per op */
    T *fc;               /* parsed fma_c per op */
} SFX(StagePlan);

#define NST 8

static T SFX(window_get)(const KOOp *ops, int src, T **buffers, const int32_t *is_in,
                         SFX(Block) *B, int64_t S, int64_t s0, int L, int lane, int64_t t,
                         int64_t off, int64_t cur_time) {
    const KOOp *o = &ops[src];
    if (o->kind == KO_WTEMP) {
        /* ring of `window` rows, NaN before the run start (Ops.hpp:176-210) */
        if (t < off) return (T)NAN;
        int w = o->window;
        int64_t row = (t - off) % w;
        return B->st[src][row * L + lane];
    }
    if (t < off) return (T)NAN;
    int b = o->buf;
    int64_t base = (is_in[b] && !o->single_value) ? cur_time : 0;
    return buffers[b][(base + t - off) * S + s0 + lane];
}

static int SFX(red_loop)(const KOOp *ops, int r) {
    int in0 = ops[r].in[0];
    if (ops[in0].kind == KO_LOOP) return in0;
    return ops[in0].parent;
}

static T SFX(parse)(const char *s);

static int SFX(plan)(const KOStage *stg, SFX(StagePlan) *P) {
    int n = stg->nops;
    const KOOp *ops = stg->ops;
    P->stage = stg;
    P->cst = calloc(n, sizeof(T));
    P->qv = calloc(n, sizeof(T));
    P->fc = calloc(n, sizeof(T));
    for (int i = 0; i < n; i++) {
        if (ops[i].cval[0]) P->cst[i] = SFX(parse)(ops[i].cval);
        if (ops[i].qval[0]) P->qv[i] = SFX(parse)(ops[i].qval);
        if (ops[i].fma_c[0]) P->fc[i] = SFX(parse)(ops[i].fma_c);
    }
    P->is_top = calloc(n, sizeof(int));
    P->loop_body = calloc(n, sizeof(int *));
    P->loop_body_n = calloc(n, sizeof(int));
    P->loop_red = calloc(n, sizeof(int *));
    P->loop_red_n = calloc(n, sizeof(int));
    P->loop_own_red = calloc(n, sizeof(int *));
    P->loop_own_red_n = calloc(n, sizeof(int));
    int prev = -1;
    for (int i = 0; i < n; i++) {
        const KOOp *o = &ops[i];
        if (o->parent < 0) P->is_top[i] = 1;
        else if (ops[o->parent].parent >= 0) {
            set_err("nested loops are not supported");
            return -1;
        }
        if (o->kind != KO_LOOP) continue;
        int nb = 0, nr = 0, no = 0;
        int *body = malloc(sizeof(int) * (n + (prev >= 0 ? P->loop_body_n[prev] : 0)));
        int *red = malloc(sizeof(int) * (n + (prev >= 0 ? P->loop_red_n[prev] : 0)));
        int *own = malloc(sizeof(int) * n);
        if (o->copy_prev && prev >= 0) {
            for (int j = 0; j < P->loop_body_n[prev]; j++) body[nb++] = P->loop_body[prev][j];
            for (int j = 0; j < P->loop_red_n[prev]; j++) red[nr++] = P->loop_red[prev][j];
        }
        for (int j = 0; j < n; j++) {
            if (ops[j].parent == i) body[nb++] = j;
            if (ops[j].kind >= KO_RADD && ops[j].kind <= KO_RDECAY && SFX(red_loop)(ops, j) == i) {
                red[nr++] = j;
                own[no++] = j;
            }
        }
        P->loop_body[i] = body; P->loop_body_n[i] = nb;
        P->loop_red[i] = red; P->loop_red_n[i] = nr;
        P->loop_own_red[i] = own; P->loop_own_red_n[i] = no;
        prev = i;
    }
    return 0;
}

static void SFX(unplan)(SFX(StagePlan) *P) {
    int n = P->stage->nops;
    for (int i = 0; i < n; i++) {
        free(P->loop_body[i]); free(P->loop_red[i]); free(P->loop_own_red[i]);
    }
    free(P->is_top); free(P->loop_body); free(P->loop_body_n); free(P->loop_red);
    free(P->loop_red_n); free(P->loop_own_red); free(P->loop_own_red_n);
    free(P->cst); free(P->qv); free(P->fc);
}

static T SFX(parse)(const char *s) {
#if defined(KO_IS_FLOAT)
    return strtof(s, NULL);
#else
    return strtod(s, NULL);
#endif
}

/* element-wise ops shared by the top level and loop bodies; `iter` is the
 * loop iteration for ops inside a loop.  Returns 1 if handled. */
static int SFX(eval_simple)(const KOOp *ops, const T *cst, const T *fc, int i, SFX(Block) *B, int L, int64_t iter) {
    const KOOp *o = &ops[i];
    if (o->fma_pos >= 0) {
        /* contracted multiply-add: input fma_pos is the product fa * fb */
        T *out = B->val + (int64_t)i * L;
        const T *fa = B->val + (int64_t)o->fma_a * L;
        const T *fb = o->fma_b >= 0 ? B->val + (int64_t)o->fma_b * L : NULL;
        T fcv = fc[i];
        const T *other = (o->nin > 1) ? B->val + (int64_t)o->in[1 - o->fma_pos] * L : NULL;
        T c = cst[i];
        for (int l = 0; l < L; l++) {
            T A = fa[l], Bv = fb ? fb[l] : fcv;
            switch (o->kind) {
            case KO_ADD: out[l] = FMA(A, Bv, other[l]); break;
            case KO_SUB: out[l] = o->fma_pos == 0 ? FMA(A, Bv, -other[l]) : FMA(-A, Bv, other[l]); break;
            case KO_ADDC: out[l] = FMA(A, Bv, c); break;
            case KO_SUBC: out[l] = o->swap ? FMA(-A, Bv, c) : FMA(A, Bv, -c); break;
            default: return 0;
            }
        }
        return 1;
    }
    T *out = B->val + (int64_t)i * L;
    const T *a = o->nin > 0 ? B->val + (int64_t)o->in[0] * L : NULL;
    const T *b = o->nin > 1 ? B->val + (int64_t)o->in[1] * L : NULL;
    const T *c3 = o->nin > 2 ? B->val + (int64_t)o->in[2] * L : NULL;
    T c = (T)0;
    switch (o->kind) {
    case KO_CONST: c = cst[i]; for (int l = 0; l < L; l++) out[l] = c; return 1;
    case KO_ADD: for (int l = 0; l < L; l++) out[l] = a[l] + b[l]; return 1;
    case KO_SUB: for (int l = 0; l < L; l++) out[l] = a[l] - b[l]; return 1;
    case KO_MUL: for (int l = 0; l < L; l++) out[l] = a[l] * b[l]; return 1;
    case KO_DIV: for (int l = 0; l < L; l++) out[l] = a[l] / b[l]; return 1;
    case KO_MAX: for (int l = 0; l < L; l++) out[l] = a[l] > b[l] ? a[l] : b[l]; return 1;
    case KO_MIN: for (int l = 0; l < L; l++) out[l] = a[l] < b[l] ? a[l] : b[l]; return 1;
    case KO_OR: for (int l = 0; l < L; l++) out[l] = SFX(from_bits)(SFX(bits)(a[l]) | SFX(bits)(b[l])); return 1;
    case KO_AND: for (int l = 0; l < L; l++) out[l] = SFX(from_bits)(SFX(bits)(a[l]) & SFX(bits)(b[l])); return 1;
    case KO_NOT: for (int l = 0; l < L; l++) out[l] = SFX(from_bits)(~SFX(bits)(a[l])); return 1;
    case KO_GT: for (int l = 0; l < L; l++) out[l] = SFX(mask)(a[l] > b[l]); return 1;
    case KO_GE: for (int l = 0; l < L; l++) out[l] = SFX(mask)(a[l] >= b[l]); return 1;
    case KO_LT: for (int l = 0; l < L; l++) out[l] = SFX(mask)(a[l] < b[l]); return 1;
    case KO_LE: for (int l = 0; l < L; l++) out[l] = SFX(mask)(a[l] <= b[l]); return 1;
    case KO_EQ: for (int l = 0; l < L; l++) out[l] = SFX(mask)(a[l] == b[l]); return 1;
    case KO_ADDC: c = cst[i]; for (int l = 0; l < L; l++) out[l] = o->swap ? c + a[l] : a[l] + c; return 1;
    case KO_SUBC: c = cst[i]; for (int l = 0; l < L; l++) out[l] = o->swap ? c - a[l] : a[l] - c; return 1;
    case KO_MULC: c = cst[i]; for (int l = 0; l < L; l++) out[l] = o->swap ? c * a[l] : a[l] * c; return 1;
    case KO_DIVC: c = cst[i]; for (int l = 0; l < L; l++) out[l] = o->swap ? c / a[l] : a[l] / c; return 1;
    case KO_GTC: c = cst[i]; for (int l = 0; l < L; l++) out[l] = SFX(mask)(o->swap ? c > a[l] : a[l] > c); return 1;
    case KO_LTC: c = cst[i]; for (int l = 0; l < L; l++) out[l] = SFX(mask)(o->swap ? c < a[l] : a[l] < c); return 1;
    case KO_SQRT: for (int l = 0; l < L; l++) out[l] = SQRT(a[l]); return 1;
    case KO_LOG:
        if (o->fast_log) { for (int l = 0; l < L; l++) out[l] = SFX(logfast)(a[l]); }
        else { for (int l = 0; l < L; l++) out[l] = LOG(a[l]); }
        return 1;
    case KO_EXP: for (int l = 0; l < L; l++) out[l] = SFX(expk)(a[l]); return 1;
    case KO_ABS: for (int l = 0; l < L; l++) out[l] = SFX(from_bits)(SFX(bits)(a[l]) & (((UT)~(UT)0) >> 1)); return 1;
    case KO_SIGN:
        /* Ops.hpp:693-701 */
        for (int l = 0; l < L; l++) {
            T v = a[l];
            T r = (v != v) ? (T)NAN : (T)1.0;
            if (v < (T)0) r = (T)-1.0;
            if (v == (T)0) r = (T)0;
            out[l] = r;
        }
        return 1;
    case KO_SETINFNAN:
        /* Ops.hpp:716-720 */
        c = cst[i];
        for (int l = 0; l < L; l++) { T d = a[l] - a[l]; out[l] = (d != d) ? c : a[l]; }
        return 1;
    case KO_SELECT:
        for (int l = 0; l < L; l++) out[l] = SFX(sel)(a[l]) ? b[l] : c3[l];
        return 1;
    case KO_RETFIRST:
        for (int l = 0; l < L; l++) out[l] = a[l];
        return 1;
    case KO_LOOPIDX:
        for (int l = 0; l < L; l++) out[l] = (T)(o->loop_window - 1 - iter);
        return 1;
    default:
        return 0;
    }
}

/* reduction templates, cpp/Kun/Ops.hpp:468-616 */
static void SFX(red_init)(const KOOp *ops, int r, SFX(Block) *B, int L) {
    const KOOp *o = &ops[r];
    T *s = B->st[r];
    switch (o->kind) {
    case KO_RADD: for (int l = 0; l < L; l++) { s[l] = 0; s[L + l] = 0; } break;
    case KO_RMUL: for (int l = 0; l < L; l++) s[l] = (T)1.0; break;
    case KO_RMIN: for (int l = 0; l < L; l++) s[l] = (T)INFINITY; break;
    case KO_RMAX: for (int l = 0; l < L; l++) s[l] = -(T)INFINITY; break;
    case KO_RARGMAX: for (int l = 0; l < L; l++) { s[l] = -(T)INFINITY; s[L + l] = 0; } break;
    case KO_RARGMIN: for (int l = 0; l < L; l++) { s[l] = (T)INFINITY; s[L + l] = 0; } break;
    case KO_RRANK: {
        const T *cur = B->val + (int64_t)o->in[1] * L;
        for (int l = 0; l < L; l++) { s[l] = cur[l]; s[L + l] = 0; s[2 * L + l] = 0; }
        break;
    }
    case KO_RDECAY: {
        T step = (T)(1.0 / ((1.0 + o->window) * o->window / 2));
        for (int l = 0; l < L; l++) { s[l] = step; s[L + l] = 0; }
        break;
    }
    }
}

static void SFX(red_step)(const KOOp *ops, const T *fc, int r, SFX(Block) *B, int L, int64_t iter) {
    const KOOp *o = &ops[r];
    T *s = B->st[r];
    const T *x = B->val + (int64_t)o->in[0] * L;
    switch (o->kind) {
    case KO_RADD:
        if (o->fma_pos == 0) {
            /* Kahan step whose input is a contracted product: y = a*b - c */
            const T *fa = B->val + (int64_t)o->fma_a * L;
            const T *fb = o->fma_b >= 0 ? B->val + (int64_t)o->fma_b * L : NULL;
            if (o->unrolled && iter == o->first_iter) {
                /* first step of a fully unrolled loop: with s = c = 0 folded in,
                 * the product feeds both `0 + p` and `t - p` and is contracted
                 * into each */
                for (int l = 0; l < L; l++) {
                    T A = fa[l], Bv = fb ? fb[l] : fc[r];
                    T t = FMA(A, Bv, s[l]);
                    s[L + l] = FMA(-A, Bv, t - s[l]);
                    s[l] = t;
                }
                break;
            }
            for (int l = 0; l < L; l++) {
                T y = FMA(fa[l], fb ? fb[l] : fc[r], -s[L + l]);
                T t = s[l] + y;
                s[L + l] = t - s[l] - y;
                s[l] = t;
            }
            break;
        }
        for (int l = 0; l < L; l++) {
            T y = x[l] - s[L + l];
            T t = s[l] + y;
            s[L + l] = t - s[l] - y;
            s[l] = t;
        }
        break;
    case KO_RMUL: for (int l = 0; l < L; l++) s[l] = s[l] * x[l]; break;
    case KO_RMIN:
        for (int l = 0; l < L; l++) {
            T v = s[l], in = x[l];
            s[l] = (v != v || in != in) ? (T)NAN : (v < in ? v : in);
        }
        break;
    case KO_RMAX:
        for (int l = 0; l < L; l++) {
            T v = s[l], in = x[l];
            s[l] = (v != v || in != in) ? (T)NAN : (v > in ? v : in);
        }
        break;
    case KO_RARGMAX:
    case KO_RARGMIN:
        for (int l = 0; l < L; l++) {
            T v = s[l], in = x[l];
            int isn = (v != v) || (in != in);
            int cmp = o->kind == KO_RARGMAX ? (v < in) : (v > in);
            v = cmp ? in : v;
            v = isn ? (T)NAN : v;
            T id = cmp ? (T)iter : s[L + l];
            id = isn ? (T)NAN : id;
            s[l] = v;
            s[L + l] = id;
        }
        break;
    case KO_RRANK:
        for (int l = 0; l < L; l++) {
            T v = s[l], in = x[l];
            int isn = (v != v) || (in != in);
            T less = s[L + l], eq = s[2 * L + l];
            less = isn ? (T)NAN : less;
            less = (in < v) ? less + (T)1.0 : less;
            eq = (in == v) ? eq + (T)1.0 : eq;
            s[L + l] = less;
            s[2 * L + l] = eq;
        }
        break;
    case KO_RDECAY: {
        T step = (T)(1.0 / ((1.0 + o->window) * o->window / 2));
        for (int l = 0; l < L; l++) {
            s[L + l] = FMA(x[l], s[l], s[L + l]);
            s[l] = s[l] + step;
        }
        break;
    }
    }
}

static void SFX(red_final)(const KOOp *ops, int r, SFX(Block) *B, int L) {
    const KOOp *o = &ops[r];
    T *s = B->st[r];
    T *out = B->val + (int64_t)r * L;
    switch (o->kind) {
    case KO_RADD: case KO_RMUL: case KO_RMIN: case KO_RMAX:
        for (int l = 0; l < L; l++) out[l] = s[l];
        break;
    case KO_RARGMAX: case KO_RARGMIN: case KO_RDECAY:
        for (int l = 0; l < L; l++) out[l] = s[L + l];
        break;
    case KO_RRANK:
        for (int l = 0; l < L; l++) out[l] = s[L + l] + (s[2 * L + l] + (T)1.0) / (T)2.0;
        break;
    }
}

static void SFX(block_alloc)(const KOStage *stg, SFX(Block) *B, int L) {
    int n = stg->nops;
    B->val = calloc((size_t)n * L, sizeof(T));
    B->st = calloc(n, sizeof(T *));
    B->sti = calloc(n, sizeof(int32_t *));
    B->sl = calloc(n, sizeof(SFX(SkipLane) *));
    for (int i = 0; i < n; i++) {
        const KOOp *o = &stg->ops[i];
        switch (o->kind) {
        case KO_WTEMP: if (o->parent < 0) B->st[i] = malloc(sizeof(T) * (size_t)o->window * L); break;
        case KO_RADD: case KO_RARGMAX: case KO_RARGMIN: case KO_RDECAY: case KO_RRANK:
        case KO_RMUL: case KO_RMIN: case KO_RMAX:
            B->st[i] = malloc(sizeof(T) * 3 * L); break;
        case KO_FWSUM: B->st[i] = malloc(sizeof(T) * 3 * L); B->sti[i] = malloc(sizeof(int32_t) * L); break;
        case KO_LINREG: B->st[i] = malloc(sizeof(T) * 6 * L); B->sti[i] = malloc(sizeof(int32_t) * L); break;
        case KO_EMA: case KO_ACC: B->st[i] = malloc(sizeof(T) * L); break;
        case KO_SKIPLIST:
            B->sl[i] = calloc(L, sizeof(SFX(SkipLane)));
            for (int l = 0; l < L; l++) {
                B->sl[i][l].v = malloc(sizeof(double) * (o->window + 2));
                B->sl[i][l].idx = malloc(sizeof(int64_t) * (o->window + 2));
            }
            break;
        }
    }
}

static void SFX(block_free)(const KOStage *stg, SFX(Block) *B, int L) {
    int n = stg->nops;
    for (int i = 0; i < n; i++) {
        free(B->st[i]);
        free(B->sti[i]);
        if (B->sl[i]) {
            for (int l = 0; l < L; l++) { free(B->sl[i][l].v); free(B->sl[i][l].idx); }
            free(B->sl[i]);
        }
    }
    free(B->val); free(B->st); free(B->sti); free(B->sl);
}

/* reset the per-run state: cpp/Kun/Ops.hpp constructors */
static void SFX(block_reset)(const KOStage *stg, SFX(Block) *B, int L, T **buffers, int64_t S, int64_t s0) {
    int n = stg->nops;
    for (int i = 0; i < n; i++) {
        const KOOp *o = &stg->ops[i];
        switch (o->kind) {
        case KO_WTEMP:
            if (B->st[i]) for (int64_t j = 0; j < (int64_t)o->window * L; j++) B->st[i][j] = (T)NAN;
            break;
        case KO_FWSUM:
            for (int l = 0; l < 3 * L; l++) B->st[i][l] = 0;
            for (int l = 0; l < L; l++) B->sti[i][l] = o->window;
            break;
        case KO_LINREG:
            for (int l = 0; l < 6 * L; l++) B->st[i][l] = 0;
            for (int l = 0; l < L; l++) B->sti[i][l] = o->window;
            break;
        case KO_EMA:
            if (o->nin == 2) {
                /* init value: Input{single_value} read at row 0 (MiscOp.py:106-111) */
                int src = o->in[1];
                int b = stg->ops[src].buf;
                for (int l = 0; l < L; l++) B->st[i][l] = buffers[b][s0 + l];
            } else {
                for (int l = 0; l < L; l++) B->st[i][l] = (T)NAN;
            }
            break;
        case KO_ACC:
            for (int l = 0; l < L; l++) B->st[i][l] = 0;
            break;
        case KO_SKIPLIST:
            for (int l = 0; l < L; l++) { B->sl[i][l].size = 0; B->sl[i][l].last_rank = 0; }
            break;
        }
    }
    (void)S;
}

static int SFX(run_ts_block)(const SFX(StagePlan) *P, SFX(Block) *B, T **buffers, const int32_t *is_in,
                             int64_t S, int64_t s0, int L, int64_t cur_time, int64_t length) {
    const KOStage *stg = P->stage;
    const KOOp *ops = stg->ops;
    int n = stg->nops;
    SFX(block_reset)(stg, B, L, buffers, S, s0);
    for (int64_t t = 0; t < length; t++) {
        for (int i = 0; i < n; i++) {
            if (!P->is_top[i]) continue;
            const KOOp *o = &ops[i];
            T *out = B->val + (int64_t)i * L;
            const T *a = o->nin > 0 ? B->val + (int64_t)o->in[0] * L : NULL;
            switch (o->kind) {
            case KO_INPUT: {
                int b = o->buf;
                if (o->single_value) {
                    for (int l = 0; l < L; l++) out[l] = buffers[b][s0 + l];
                } else {
                    int64_t base = is_in[b] ? cur_time : 0;
                    const T *src = buffers[b] + (base + t) * S + s0;
                    for (int l = 0; l < L; l++) out[l] = src[l];
                }
                break;
            }
            case KO_OUTPUT: {
                T *dst = buffers[o->buf] + t * S + s0;
                for (int l = 0; l < L; l++) { dst[l] = a[l]; out[l] = a[l]; }
                break;
            }
            case KO_WTEMP: {
                T *ring = B->st[i] + (t % o->window) * L;
                for (int l = 0; l < L; l++) { ring[l] = a[l]; out[l] = a[l]; }
                break;
            }
            case KO_LOOP: {
                for (int j = 0; j < P->loop_own_red_n[i]; j++) SFX(red_init)(ops, P->loop_own_red[i][j], B, L);
                for (int64_t iter = o->window - 1; iter >= o->seg_end; iter--) {
                    for (int j = 0; j < P->loop_body_n[i]; j++) {
                        int bi = P->loop_body[i][j];
                        const KOOp *bo = &ops[bi];
                        if (bo->kind == KO_ITER) {
                            T *bout = B->val + (int64_t)bi * L;
                            for (int l = 0; l < L; l++)
                                bout[l] = SFX(window_get)(ops, bo->in[1], buffers, is_in, B, S, s0, L, l, t, iter, cur_time);
                        } else if (!SFX(eval_simple)(ops, P->cst, P->fc, bi, B, L, iter)) {
                            set_err("unsupported op inside a loop");
                            return -1;
                        }
                    }
                    for (int j = 0; j < P->loop_red_n[i]; j++) SFX(red_step)(ops, P->fc, P->loop_red[i][j], B, L, iter);
                }
                for (int j = 0; j < P->loop_red_n[i]; j++) SFX(red_final)(ops, P->loop_red[i][j], B, L);
                break;
            }
            case KO_RADD: case KO_RMUL: case KO_RMIN: case KO_RMAX: case KO_RARGMAX:
            case KO_RARGMIN: case KO_RRANK: case KO_RDECAY:
                break; /* value produced by its loop */
            case KO_BACKREF:
                /* windowedRef, Ops.hpp:528-535 */
                for (int l = 0; l < L; l++)
                    out[l] = (t >= o->window) ? SFX(window_get)(ops, o->in[0], buffers, is_in, B, S, s0, L, l, t, o->window, cur_time) : (T)NAN;
                break;
            case KO_FWSUM: {
                /* FastWindowedSum, Ops.hpp:324-356 */
                T *v = B->st[i], *cadd = B->st[i] + L, *csub = B->st[i] + 2 * L;
                int32_t *nn = B->sti[i];
                for (int l = 0; l < L; l++) {
                    T old = SFX(window_get)(ops, o->in[0], buffers, is_in, B, S, s0, L, l, t, o->window, cur_time);
                    T cur = a[l];
                    int on = old != old, cn = cur != cur;
                    if (!on) {
                        T small = (T)0 - old;
                        T y = small - csub[l];
                        T tt = v[l] + y;
                        csub[l] = tt - v[l] - y;
                        v[l] = tt;
                    }
                    if (!cn) {
                        T y = cur - cadd[l];
                        T tt = v[l] + y;
                        cadd[l] = tt - v[l] - y;
                        v[l] = tt;
                    }
                    nn[l] = nn[l] - on + cn;
                    out[l] = nn[l] == 0 ? v[l] : (T)NAN;
                }
                break;
            }
            case KO_EMA: {
                /* ExpMovingAvg, Ops.hpp:358-375 */
                T w = (T)2.0 / (o->window + 1);
                T *v = B->st[i];
                for (int l = 0; l < L; l++) {
                    T cur = a[l];
                    T nv = FMA(cur, w, v[l] * ((T)1 - w));
                    T r = (cur != cur) ? v[l] : nv;
                    r = (v[l] != v[l]) ? cur : r;
                    v[l] = r;
                    out[l] = r;
                }
                break;
            }
            case KO_LINREG: {
                /* WindowedLinearRegression, Ops.hpp:377-423 */
                T *isum = B->st[i], *xsum = isum + L, *x2sum = isum + 2 * L, *ysum = isum + 3 * L,
                  *y2sum = isum + 4 * L, *xysum = isum + 5 * L;
                int32_t *nn = B->sti[i];
                T W = (T)o->window;
                for (int l = 0; l < L; l++) {
                    xysum[l] = xysum[l] - ysum[l];
                    x2sum[l] = x2sum[l] + isum[l] - (T)2.0 * xsum[l];
                    xsum[l] = xsum[l] - isum[l];
                    T old = SFX(window_get)(ops, o->in[0], buffers, is_in, B, S, s0, L, l, t, o->window, cur_time);
                    T cur = a[l];
                    int on = old != old, cn = cur != cur;
                    /* products feeding a single add/sub are contracted by the reference build */
                    if (!on) { isum[l] = isum[l] - (T)1; ysum[l] = ysum[l] - old; y2sum[l] = FMA(-old, old, y2sum[l]); }
                    nn[l] = nn[l] - on + cn;
                    if (!cn) {
                        isum[l] = isum[l] + (T)1;
                        xsum[l] = xsum[l] + W;
                        x2sum[l] = x2sum[l] + (W * W);
                        ysum[l] = ysum[l] + cur;
                        /* cur*cur is shared by every regression on the same input
                         * of the stage; shared, its uses span several basic blocks
                         * and it is not contracted */
                        y2sum[l] = o->shared_sq ? y2sum[l] + cur * cur : FMA(cur, cur, y2sum[l]);
                        xysum[l] = FMA(W, cur, xysum[l]);
                    }
                }
                break;
            }
            case KO_LR_RSQ: case KO_LR_SLOPE: case KO_LR_RESI: {
                int src = o->in[0];
                T *isum = B->st[src], *xsum = isum + L, *x2sum = isum + 2 * L, *ysum = isum + 3 * L,
                  *y2sum = isum + 4 * L, *xysum = isum + 5 * L;
                int32_t *nn = B->sti[src];
                T W = (T)ops[src].window;
                const T *val = o->nin > 1 ? B->val + (int64_t)o->in[1] * L : NULL;
                for (int l = 0; l < L; l++) {
                    T N = (T)(int32_t)(ops[src].window - nn[l]);
                    /* `N*a - b*c`: the reference build evaluates operands right to left
                     * and contracts the product that is computed first (b*c) */
                    if (o->kind == KO_LR_RSQ) {
                        T r1 = FMA(-xsum[l], ysum[l], N * xysum[l]);
                        r1 = r1 * r1;
                        T r2 = FMA(-xsum[l], xsum[l], N * x2sum[l]) * FMA(-ysum[l], ysum[l], N * y2sum[l]);
                        out[l] = r1 / r2;
                    } else {
                        T slope = FMA(-xsum[l], ysum[l], N * xysum[l]) / FMA(-xsum[l], xsum[l], N * x2sum[l]);
                        if (o->kind == KO_LR_SLOPE) out[l] = slope;
                        else {
                            T xm = xsum[l] / N, ym = ysum[l] / N;
                            T interp = FMA(-slope, xm, ym);
                            out[l] = val[l] - FMA(slope, W, interp);
                        }
                    }
                }
                break;
            }
            case KO_SKIPLIST: {
                const T *oldv = a, *newv = B->val + (int64_t)o->in[1] * L;
                for (int l = 0; l < L; l++) {
                    SFX(SkipLane) *s = &B->sl[i][l];
                    if (oldv[l] == oldv[l]) SFX(sl_remove)(s, (double)oldv[l]);
                    if (newv[l] == newv[l]) s->last_rank = SFX(sl_insert)(s, (double)newv[l], t);
                }
                break;
            }
            case KO_SL_QUANTILE: case KO_SL_MIN: case KO_SL_MAX: case KO_SL_ARGMIN: case KO_SL_RANK: {
                /* cpp/Kun/Ops/Quantile.hpp:82-170 */
                int src = o->in[0];
                int W = stg->ops[src].window;
                T q = P->qv[i];
                const T *cur = o->nin > 1 ? B->val + (int64_t)o->in[1] * L : NULL;
                for (int l = 0; l < L; l++) {
                    SFX(SkipLane) *s = &B->sl[src][l];
                    int nobs = s->size;
                    if (nobs != W) { out[l] = (T)NAN; continue; }
                    if (o->kind == KO_SL_QUANTILE) {
                        T iwf = q * (T)(nobs - 1);
                        int id = (int)iwf;
                        if ((T)id == iwf) out[l] = (T)s->v[id];
                        else {
                            double lo = s->v[id], hi = s->v[id + 1];
                            T frac = iwf - (T)id;
                            out[l] = (T)fma(hi - lo, (double)frac, lo);
                        }
                    } else if (o->kind == KO_SL_MIN) out[l] = (T)s->v[0];
                    else if (o->kind == KO_SL_MAX) out[l] = (T)s->v[W - 1];
                    else if (o->kind == KO_SL_ARGMIN) out[l] = (T)(uint64_t)((uint64_t)s->idx[0] + (uint64_t)nobs - (uint64_t)t);
                    else {
                        double rank = s->last_rank + 1;
                        double rmin = SFX(sl_minrank)(s, (double)cur[l]) + 1;
                        rank = (((rank * (rank + 1) / 2) - ((rmin - 1) * rmin / 2)) / (rank - rmin + 1));
                        out[l] = (T)rank;
                    }
                }
                break;
            }
            case KO_ACC: {
                T *v = B->st[i];
                for (int l = 0; l < L; l++) out[l] = v[l];
                break;
            }
            case KO_SETACC: {
                /* SetAccumulator, Ops.hpp:315-322 */
                int acc = o->in[0];
                T *v = B->st[acc];
                const T *msk = B->val + (int64_t)o->in[1] * L, *nv = B->val + (int64_t)o->in[2] * L;
                for (int l = 0; l < L; l++) {
                    v[l] = SFX(sel)(msk[l]) ? nv[l] : a[l];
                    out[l] = v[l];
                }
                break;
            }
            default:
                if (!SFX(eval_simple)(ops, P->cst, P->fc, i, B, L, 0)) {
                    set_err("unsupported op at top level");
                    return -1;
                }
            }
        }
    }
    return 0;
}

static int SFX(cmp)(const void *x, const void *y) {
    T a = *(const T *)x, b = *(const T *)y;
    return a < b ? -1 : (a > b ? 1 : 0);
}

/* RankStocks, cpp/Kun/Rank.hpp:13-57 */
static void SFX(rank_row)(const T *in, T *out, int64_t S, T *scratch) {
    int64_t n = 0;
    for (int64_t i = 0; i < S; i++) if (in[i] == in[i]) scratch[n++] = in[i];
    qsort(scratch, n, sizeof(T), SFX(cmp));
    for (int64_t i = 0; i < S; i++) {
        T x = in[i];
        if (x != x) { out[i] = (T)NAN; continue; }
        int64_t lo = 0, hi = n;
        while (lo < hi) { int64_t m = (lo + hi) / 2; if (scratch[m] < x) lo = m + 1; else hi = m; }
        int64_t start = lo;
        hi = n;
        while (lo < hi) { int64_t m = (lo + hi) / 2; if (x < scratch[m]) hi = m; else lo = m + 1; }
        int64_t end = lo;
        int64_t sum = (start + end + 1) * (end - start) / 2;
        out[i] = (T)sum / (T)(end - start) / (T)n;
    }
}

/* ScaleStocks, cpp/Kun/Scale.hpp:14-46 */
static void SFX(scale_row)(const T *in, T *out, int64_t S) {
    T sum = 0;
    for (int64_t i = 0; i < S; i++) if (in[i] == in[i]) sum += SFX(from_bits)(SFX(bits)(in[i]) & (((UT)~(UT)0) >> 1));
    for (int64_t i = 0; i < S; i++) out[i] = (in[i] == 0 && sum == 0) ? (T)NAN : in[i] / sum;
}

/* DiffWithWeightedSum, KunQuant/ops/MiscOp.py:220-240 */
static void SFX(diffw_row)(const T *in0, const T *in1, T *out, int64_t S) {
    T sum = 0;
    for (int64_t i = 0; i < S; i++) sum += in0[i] * in1[i];
    for (int64_t i = 0; i < S; i++) out[i] = in0[i] - sum;
}

static int SFX(run_xsec)(const KOStage *stg, T **buffers, const int32_t *is_in, int64_t S,
                         int64_t cur_time, int64_t length, int nthreads) {
    const KOOp *ops = stg->ops;
    int inb[2] = {-1, -1}, nin = 0, outb = -1;
    for (int i = 0; i < stg->nops; i++) {
        if (ops[i].kind == KO_INPUT && nin < 2) inb[nin++] = ops[i].buf;
        if (ops[i].kind == KO_OUTPUT) outb = ops[i].buf;
    }
    /* the op order may list inputs in any order; take them in the cross-sectional op's order */
    for (int i = 0; i < stg->nops; i++) {
        if (ops[i].kind == KO_RANK || ops[i].kind == KO_SCALE || ops[i].kind == KO_DIFFWSUM) {
            for (int j = 0; j < ops[i].nin && j < 2; j++) inb[j] = ops[ops[i].in[j]].buf;
        }
    }
    if (inb[0] < 0 || outb < 0) { set_err("bad cross-sectional stage"); return -1; }
    int rc = 0;
#pragma omp parallel num_threads(nthreads)
    {
        T *scratch = malloc(sizeof(T) * (S + 1));
#pragma omp for schedule(static)
        for (int64_t t = 0; t < length; t++) {
            int64_t r0 = is_in[inb[0]] ? cur_time + t : t;
            const T *in0 = buffers[inb[0]] + r0 * S;
            T *out = buffers[outb] + t * S;
            if (stg->kind == 1) SFX(rank_row)(in0, out, S, scratch);
            else if (stg->kind == 2) SFX(scale_row)(in0, out, S);
            else {
                int64_t r1 = is_in[inb[1]] ? cur_time + t : t;
                SFX(diffw_row)(in0, buffers[inb[1]] + r1 * S, out, S);
            }
        }
        free(scratch);
    }
    return rc;
}

static int SFX(run_all)(const KOStage *stages, int nstages, T **buffers, const int32_t *is_in, int64_t S,
                int64_t total_time, int64_t cur_time, int64_t length, int nthreads) {
    (void)total_time;
    if (nthreads <= 0) nthreads = 1;
    static int inited = 0;
    if (!inited) { SFX(init_tables)(); inited = 1; }
    for (int si = 0; si < nstages; si++) {
        const KOStage *stg = &stages[si];
        if (stg->kind != 0) {
            if (SFX(run_xsec)(stg, buffers, is_in, S, cur_time, length, nthreads)) return -1;
            continue;
        }
        SFX(StagePlan) P;
        if (SFX(plan)(stg, &P)) return -1;
        const int LB = 16;
        int64_t nblocks = (S + LB - 1) / LB;
        int err = 0;
#pragma omp parallel num_threads(nthreads)
        {
            SFX(Block) B;
            SFX(block_alloc)(stg, &B, LB);
            SFX(Block) Btail;
            int tailL = (int)(S % LB);
            if (tailL) SFX(block_alloc)(stg, &Btail, tailL);
#pragma omp for schedule(dynamic, 1)
            for (int64_t bi = 0; bi < nblocks; bi++) {
                int64_t s0 = bi * LB;
                int L = (int)((S - s0) < LB ? (S - s0) : LB);
                int r = SFX(run_ts_block)(&P, L == LB ? &B : &Btail, buffers, is_in, S, s0, L, cur_time, length);
                if (r) {
#pragma omp atomic write
                    err = 1;
                }
            }
            SFX(block_free)(stg, &B, LB);
            if (tailL) SFX(block_free)(stg, &Btail, tailL);
        }
        SFX(unplan)(&P);
        if (err) return -1;
    }
    return 0;
}

static void SFX(logfast_arr)(const T *x, T *y, int64_t n) {
    SFX(init_tables)();
    for (int64_t i = 0; i < n; i++) y[i] = SFX(logfast)(x[i]);
}
static void SFX(exp_arr)(const T *x, T *y, int64_t n) {
    for (int64_t i = 0; i < n; i++) y[i] = SFX(expk)(x[i]);
}
