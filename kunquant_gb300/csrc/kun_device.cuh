// Device templates of the GPU backend: the arithmetic of KunQuant's op
// templates (cpp/Kun/Ops.hpp, cpp/Kun/Ops/Quantile.hpp, cpp/Kun/Rank.hpp,
// cpp/Kun/Scale.hpp, cpp/KunSIMD/cpu/Math.hpp) written for one stock per
// thread.  Every translation unit that includes this file is compiled with
// -fmad=false: a product is fused into an add only where a template below
// calls kfma(), which is exactly where the reference's GCC build forms an FMA.
#pragma once
#include <cstdlib>
#include <cstdint>
#include <cuda_runtime.h>

namespace kun {

template <typename T> struct FpBits;
template <> struct FpBits<float> {
    using U = uint32_t;
    using S = int32_t;
    static constexpr int mant = 23;
    static constexpr int expo = 8;
};
template <> struct FpBits<double> {
    using U = unsigned long long;
    using S = long long;
    static constexpr int mant = 52;
    static constexpr int expo = 11;
};

__device__ __forceinline__ uint32_t kbits(float x) { return __float_as_uint(x); }
__device__ __forceinline__ unsigned long long kbits(double x) {
    return (unsigned long long)__double_as_longlong(x);
}
__device__ __forceinline__ float kfrom(uint32_t u, float) { return __uint_as_float(u); }
__device__ __forceinline__ double kfrom(unsigned long long u, double) {
    return __longlong_as_double((long long)u);
}
template <typename T> __device__ __forceinline__ T knan() {
    return kfrom((typename FpBits<T>::U)(sizeof(T) == 4 ? 0x7fc00000ull : 0x7ff8000000000000ull), T());
}
template <typename T> __device__ __forceinline__ T kinf() {
    return kfrom((typename FpBits<T>::U)(sizeof(T) == 4 ? 0x7f800000ull : 0x7ff0000000000000ull), T());
}
// read of row `row` of a [T][S] series column (stride st): NaN outside
// [0, length) when EDGE; interior tiles, whose rows are all inside, skip the test
template <bool EDGE, typename T>
__device__ __forceinline__ T ldw(const T* __restrict__ p, long long st, long long row, long long length) {
    if (EDGE) return (unsigned long long)row < (unsigned long long)length ? p[row * st] : knan<T>();
    return p[row * st];
}
// ---------------- bulk async copies (TMA) into shared memory, on mbarriers
// One thread of a block issues cp.async.bulk copies of whole rows (16-byte
// aligned, sizes multiples of 16) into a shared-memory stage and tells the
// stage's mbarrier how many bytes to expect; every thread waits on the
// barrier's phase before reading the stage.  Waits are bounded.
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(unsigned long long *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
// makes the initialised barriers visible to the async proxy
__device__ __forceinline__ void mbar_init_fence() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// orders this thread's earlier generic-proxy shared-memory accesses before
// later async-proxy (bulk copy) writes
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_copy_g2s(void *dst, const void *src, uint32_t bytes, unsigned long long *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// waits for the barrier's phase `parity` to complete; false after `limit`
// polls (each try_wait itself suspends for a while)
__device__ __forceinline__ bool mbar_wait(unsigned long long *bar, uint32_t parity, int limit) {
    for (int i = 0; i < limit; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}
constexpr int kTmaWaitLimit = 1 << 20;
// the staged (bulk-copy) instance of an elementwise kernel is used when
// KUN_TMA is set to a value other than 0 (read once).  Off by default: the
// plain instances already stream at ~0.8 of the copy rate, and inside a
// multi-stream module run the staged ones' shared memory (up to 45 KB per
// 128-thread block) crowds out the kernels of the other streams (Alpha158
// 5000 x 2500: 14.9 ms per run staged against 14.5 plain).
inline bool tma_enabled() {
    static const bool on = [] {
        const char *v = std::getenv("KUN_TMA");
        return v != nullptr && v[0] != '\0' && !(v[0] == '0' && v[1] == '\0');
    }();
    return on;
}
inline bool aligned16(const void *p) { return ((unsigned long long)p & 15ull) == 0; }
constexpr int kTmaRows = 4;  // rows of every input series per stage

// ring row of the value `off` ticks back, given this tick's row nm (0 <= off < W)
__device__ __forceinline__ int ring_row(int nm, int off, int W) {
    const int r = nm - off;
    return r < 0 ? r + W : r;
}
// boolean results are all-ones / all-zeros bit masks, as SIMD compares produce
template <typename T> __device__ __forceinline__ T kmask(bool b) {
    using U = typename FpBits<T>::U;
    return kfrom(b ? (U)~(U)0 : (U)0, T());
}
// blend by the sign bit of the condition (_mm256_blendv_ps semantics)
template <typename T> __device__ __forceinline__ bool ksel(T c) {
    using U = typename FpBits<T>::U;
    return (kbits(c) >> (sizeof(U) * 8 - 1)) != 0;
}
template <typename T> __device__ __forceinline__ bool kisnan(T x) { return x != x; }

__device__ __forceinline__ float kfma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double kfma(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float kadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double kadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float ksub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double ksub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float kmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double kmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float kdiv(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ double kdiv(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ float ksqrt(float a) { return __fsqrt_rn(a); }
__device__ __forceinline__ double ksqrt(double a) { return __dsqrt_rn(a); }
__device__ __forceinline__ float kfloor(float a) { return floorf(a); }
__device__ __forceinline__ double kfloor(double a) { return floor(a); }

template <typename T> __device__ __forceinline__ T kmax(T a, T b) { return a > b ? a : b; }
template <typename T> __device__ __forceinline__ T kmin(T a, T b) { return a < b ? a : b; }
template <typename T> __device__ __forceinline__ T kabs(T a) {
    using U = typename FpBits<T>::U;
    return kfrom(kbits(a) & (((U)~(U)0) >> 1), T());
}
template <typename T> __device__ __forceinline__ T kor(T a, T b) { return kfrom(kbits(a) | kbits(b), T()); }
template <typename T> __device__ __forceinline__ T kand(T a, T b) { return kfrom(kbits(a) & kbits(b), T()); }
template <typename T> __device__ __forceinline__ T knot(T a) { return kfrom(~kbits(a), T()); }
template <typename T> __device__ __forceinline__ T kselect(T c, T a, T b) { return ksel(c) ? a : b; }

// Sign, cpp/Kun/Ops.hpp:692-701
template <typename T> __device__ __forceinline__ T ksign(T v) {
    T r = kisnan(v) ? knan<T>() : T(1);
    r = v < T(0) ? T(-1) : r;
    r = v == T(0) ? T(0) : r;
    return r;
}
// SetInfOrNanToValue, cpp/Kun/Ops.hpp:715-720
template <typename T> __device__ __forceinline__ T ksetinfnan(T a, T v) {
    T d = ksub(a, a);
    return kisnan(d) ? v : a;
}

// Table-driven log of cpp/KunSIMD/cpu/Math.hpp:20-93.  The reciprocal and
// log tables are supplied by the generated code (kLogR<T>, kLogLR<T>) as
// exact binary literals.
template <typename T> struct LogTables;

template <typename T> __device__ __forceinline__ T klogfast(T x) {
    using U = typename FpBits<T>::U;
    using S = typename FpBits<T>::S;
    constexpr int mb = FpBits<T>::mant, eb = FpBits<T>::expo;
    U xi = kbits(x);
    U high5 = (xi >> (mb - 5)) & (U)31;
    U high1 = high5 >> 4;
    U e1 = (high1 ^ (((U)1 << (eb - 1)) - 1)) << mb;
    U m = (xi & ((((U)1) << mb) - 1)) | e1;
    T ri = LogTables<T>::r(high5);
    // the reference build contracts `Ri * M - 1` and both uses of `poly * Z`
    T z = kfma(ri, kfrom(m, T()), T(-1.0));
    T poly = T(1 / 5.0);
    poly = kfma(poly, z, T(-1 / 4.0));
    poly = kfma(poly, z, T(1 / 3.0));
    poly = kfma(poly, z, T(-1 / 2.0));
    poly = kfma(poly, z, T(1.0));
    T mlog = LogTables<T>::lr(high5);
    U er = (xi >> mb) + high1;
    T ep = (T)(S)er;
    T v2 = kfma(ep, T(0.6931471805599453), mlog);
    T hi = kfma(poly, z, v2);
    T lo = ksub(hi, v2);
    lo = kfma(-poly, z, lo);
    hi = kadd(hi, lo);
    if (x == T(0)) hi = -kinf<T>();
    if (x < T(0)) hi = knan<T>();
    if (x == kinf<T>()) hi = kinf<T>();
    if (kisnan(x)) hi = knan<T>();
    if (x == T(1.0)) hi = T(0);
    return hi;
}

// exp of cpp/KunSIMD/cpu/Math.hpp:96-140 (float thresholds for both types)
template <typename T> __device__ __forceinline__ T kexpk(T x) {
    using U = typename FpBits<T>::U;
    using S = typename FpBits<T>::S;
    T k = kfloor(kfma(x, T(1.4426950408889634), T(0.5)));
    S ki = (kisnan(k) || k > T(1e9) || k < T(-1e9)) ? (S)0 : (S)k;
    T r = kfma(-k, T(0.6931471805599453), x);
    T tn = kfma(r, T(0.16666666666666666), T(1.0));
    tn = kfma(tn, kmul(r, T(0.2)), T(1.0));
    tn = kfma(tn, kmul(r, T(0.25)), T(1.0));
    tn = kfma(tn, kmul(r, T(0.3333333333333333)), T(1.0));
    tn = kfma(tn, kmul(r, T(0.5)), T(1.0));
    tn = kfma(tn, r, T(1.0));
    U p = ((U)ki) << FpBits<T>::mant;
    T res = kfrom(p + kbits(tn), T());
    if (x > T(88.72283935)) res = kinf<T>();
    if (x < T(-87.33654785)) res = T(0);
    return res;
}

// ---------------- grouped launches
// One launch of a stage kernel over several jobs (universes): flat block g
// belongs to job j when off[j] <= g < off[j+1].  Passed by value.
#ifndef KUN_MAX_GROUP
#define KUN_MAX_GROUP 256
#endif
struct TileTable {
    int njobs;
    int off[KUN_MAX_GROUP + 1];
};
__device__ __forceinline__ int tile_job(const TileTable &tt, int g) {
    int lo = 0, hi = tt.njobs - 1;
    while (lo < hi) {
        const int m = (lo + hi + 1) >> 1;
        if (tt.off[m] <= g) lo = m;
        else hi = m - 1;
    }
    return lo;
}

// ---------------- compensated fp32 ("double-float") running sums
// A value hi + lo of two floats (|lo| <= ulp(hi)/2) carries about 48 bits.
// Sums use Knuth's error-free TwoSum on both parts followed by two
// renormalisations (the accurate double-word addition of Joldes, Muller and
// Popescu, ACM TOMS 2017); products use the FMA-exact product error; all steps
// are single fp32 operations, so the accumulators run at fp32 rates.  Used as
// the accumulator type of the window sums, window reductions and regression
// sums in the compensated precision form.
struct DFloat {
    float hi, lo;
    __device__ __forceinline__ DFloat() : hi(0.f), lo(0.f) {}
    __device__ __forceinline__ DFloat(float h) : hi(h), lo(0.f) {}
    __device__ __forceinline__ DFloat(int i) : hi((float)i), lo(0.f) {}
    __device__ __forceinline__ DFloat(double d) : hi((float)d), lo((float)(d - (double)(float)d)) {}
    __device__ __forceinline__ DFloat(float h, float l) : hi(h), lo(l) {}
    __device__ __forceinline__ explicit operator float() const { return __fadd_rn(hi, lo); }
};
__device__ __forceinline__ DFloat df_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    return DFloat(s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb)));
}
__device__ __forceinline__ DFloat df_fast_two_sum(float a, float b) {  // |a| >= |b|
    const float s = __fadd_rn(a, b);
    return DFloat(s, __fsub_rn(b, __fsub_rn(s, a)));
}
__device__ __forceinline__ bool kisnan(DFloat x) { return x.hi != x.hi; }
__device__ __forceinline__ DFloat operator-(DFloat x) { return DFloat(-x.hi, -x.lo); }
__device__ __forceinline__ DFloat kadd(DFloat x, DFloat y) {
    const DFloat s = df_two_sum(x.hi, y.hi);
    if (!isfinite(s.hi)) return DFloat(s.hi, 0.f);
    const DFloat t = df_two_sum(x.lo, y.lo);
    const DFloat u = df_fast_two_sum(s.hi, __fadd_rn(s.lo, t.hi));
    return df_fast_two_sum(u.hi, __fadd_rn(u.lo, t.lo));
}
__device__ __forceinline__ DFloat ksub(DFloat x, DFloat y) { return kadd(x, -y); }
__device__ __forceinline__ DFloat kmul(DFloat x, DFloat y) {
    const float p = __fmul_rn(x.hi, y.hi);
    if (!isfinite(p)) return DFloat(p, 0.f);
    float e = __fmaf_rn(x.hi, y.hi, -p);
    e = __fmaf_rn(x.hi, y.lo, e);
    e = __fmaf_rn(x.lo, y.hi, e);
    return df_fast_two_sum(p, e);
}
__device__ __forceinline__ DFloat kdiv(DFloat x, DFloat y) {
    const float q1 = __fdiv_rn(x.hi, y.hi);
    if (!isfinite(q1)) return DFloat(q1, 0.f);
    const DFloat r = ksub(x, kmul(DFloat(q1), y));
    const float q2 = __fdiv_rn(r.hi, y.hi);
    const DFloat q = df_fast_two_sum(q1, q2);
    const DFloat r2 = ksub(x, kmul(q, y));
    return kadd(q, DFloat(__fdiv_rn(r2.hi, y.hi)));
}
__device__ __forceinline__ DFloat kfma(DFloat a, DFloat b, DFloat c) { return kadd(kmul(a, b), c); }
template <> __device__ __forceinline__ DFloat knan<DFloat>() { return DFloat(knan<float>(), 0.f); }
// x + y for a float y: one TwoSum and one renormalisation
__device__ __forceinline__ DFloat df_add_f(DFloat x, float y) {
    const DFloat s = df_two_sum(x.hi, y);
    if (!isfinite(s.hi)) return DFloat(s.hi, 0.f);
    return df_fast_two_sum(s.hi, __fadd_rn(s.lo, x.lo));
}
// Running window sums of the sliding-moment form: (hi, lo) with hi the
// float sum and lo the accumulated rounding errors of its additions (each
// found exactly by TwoSum), left unnormalised between rows; after n
// additions the pair holds the exact sum to about n * 2^-48 of the largest
// partial sum.  The polynomial of the window sums is evaluated the same way.
__device__ __forceinline__ void df_acc(DFloat &s, float x) {
    const float h = __fadd_rn(s.hi, x);
    const float bb = __fsub_rn(h, s.hi);
    const float err = __fadd_rn(__fsub_rn(s.hi, __fsub_rn(h, bb)), __fsub_rn(x, bb));
    s.hi = h;
    s.lo = __fadd_rn(s.lo, err);
}
// s += a*b with the product exact (Dekker's product by one FMA)
__device__ __forceinline__ void df_acc_prod(DFloat &s, float a, float b) {
    const float p = __fmul_rn(a, b);
    const float e = __fmaf_rn(a, b, -p);
    df_acc(s, p);
    s.lo = __fadd_rn(s.lo, e);
}
// s -= a*b
__device__ __forceinline__ void df_acc_prod_neg(DFloat &s, float a, float b) {
    const float p = __fmul_rn(a, b);
    const float e = __fmaf_rn(a, b, -p);
    df_acc(s, -p);
    s.lo = __fsub_rn(s.lo, e);
}
// (hi + lo) * b for an unnormalised pair, kept as a pair: hi*b exact plus
// lo*b rounded
__device__ __forceinline__ DFloat df_scale(DFloat a, float b) {
    const float p = __fmul_rn(a.hi, b);
    return DFloat(p, __fmaf_rn(a.lo, b, __fmaf_rn(a.hi, b, -p)));
}
// s += a for pairs (TwoSum of the high parts, low parts added)
__device__ __forceinline__ void df_acc_pair(DFloat &s, DFloat a) {
    df_acc(s, a.hi);
    s.lo = __fadd_rn(s.lo, a.lo);
}
// a*b exactly, as a two-float (Dekker's product by one FMA)
__device__ __forceinline__ DFloat df_prod(float a, float b) {
    const float p = __fmul_rn(a, b);
    if (!isfinite(p)) return DFloat(p, 0.f);
    return DFloat(p, __fmaf_rn(a, b, -p));
}
// x + a*b with the product taken exactly (a*b = p + e)
__device__ __forceinline__ DFloat df_add_prod(DFloat x, float a, float b) {
    const float p = __fmul_rn(a, b);
    if (!isfinite(p)) return DFloat(__fadd_rn(x.hi, p), 0.f);
    return kadd(x, DFloat(p, __fmaf_rn(a, b, -p)));
}

// ---------------- reductions of a back-window loop, cpp/Kun/Ops.hpp:468-616
template <typename T> struct RAdd {
    T v = 0, c = 0;
    __device__ __forceinline__ void step(T x) {
        T y = ksub(x, c);
        T t = kadd(v, y);
        c = ksub(ksub(t, v), y);
        v = t;
    }
    // input is a product a*b contracted into `y = a*b - c`
    __device__ __forceinline__ void step_fma(T a, T b) {
        T y = kfma(a, b, -c);
        T t = kadd(v, y);
        c = ksub(ksub(t, v), y);
        v = t;
    }
    // first step of a loop the reference build unrolls completely: with
    // v = c = 0 folded in, the product feeds both `0 + p` and `t - p`
    __device__ __forceinline__ void step_fma_first(T a, T b) {
        T t = kfma(a, b, v);
        c = kfma(-a, b, ksub(t, v));
        v = t;
    }
    __device__ __forceinline__ T value() const { return v; }
};
// compensated form: the two-float sum needs no Kahan term of its own
template <> struct RAdd<DFloat> {
    DFloat v;
    __device__ __forceinline__ void step(float x) { v = df_add_f(v, x); }
    __device__ __forceinline__ void step_fma(float a, float b) { v = df_add_prod(v, a, b); }
    __device__ __forceinline__ void step_fma_first(float a, float b) { v = df_add_prod(v, a, b); }
    __device__ __forceinline__ DFloat value() const { return v; }
};
template <typename T> struct RMul {
    T v = T(1.0);
    __device__ __forceinline__ void step(T x) { v = kmul(v, x); }
    __device__ __forceinline__ T value() const { return v; }
};
template <typename T> struct RMin {
    T v = kinf<T>();
    __device__ __forceinline__ void step(T x) { v = (kisnan(v) || kisnan(x)) ? knan<T>() : kmin(v, x); }
    __device__ __forceinline__ T value() const { return v; }
};
template <typename T> struct RMax {
    T v = -kinf<T>();
    __device__ __forceinline__ void step(T x) { v = (kisnan(v) || kisnan(x)) ? knan<T>() : kmax(v, x); }
    __device__ __forceinline__ T value() const { return v; }
};
template <typename T, bool IsMax> struct RArg {
    T v = IsMax ? -kinf<T>() : kinf<T>();
    T idx = 0;
    __device__ __forceinline__ void step(T x, int iter) {
        bool isn = kisnan(v) || kisnan(x);
        bool cmp = IsMax ? (v < x) : (v > x);
        v = cmp ? x : v;
        v = isn ? knan<T>() : v;
        idx = cmp ? T(iter) : idx;
        idx = isn ? knan<T>() : idx;
    }
    __device__ __forceinline__ T value() const { return idx; }
};
// The same Min/Max/ArgMin/ArgMax of a window taken in runs of positions, so
// that rows whose windows overlap share the run they have in common.  A state
// covers one run; then(b) continues it with a later run b and gives exactly
// the state that stepping through both runs in order gives: NaN in either run
// is NaN; Min/Max keep the later of equal values as kmin/kmax do; Arg keeps
// the earlier position of equal values, as only a strictly better value
// replaces it.  Positions are small integers relative to the row tile, held
// in T.
template <typename T, bool IsMax, bool IsArg> struct RExt {
    T v = IsMax ? -kinf<T>() : kinf<T>();
    T pos = 0;
    __device__ __forceinline__ void step(T x, T p) {
        const bool isn = kisnan(v) || kisnan(x);
        if (IsArg) {
            const bool cmp = IsMax ? (v < x) : (v > x);
            v = cmp ? x : v;
            pos = cmp ? p : pos;
        } else {
            v = IsMax ? kmax(v, x) : kmin(v, x);
        }
        v = isn ? knan<T>() : v;
    }
    __device__ __forceinline__ void then(const RExt &b) {
        const bool isn = kisnan(v) || kisnan(b.v);
        if (IsArg) {
            const bool cmp = IsMax ? (v < b.v) : (v > b.v);
            v = cmp ? b.v : v;
            pos = cmp ? b.pos : pos;
        } else {
            v = IsMax ? kmax(v, b.v) : kmin(v, b.v);
        }
        v = isn ? knan<T>() : v;
    }
    // RArg's index of the window ending at `row`: the distance back to the
    // chosen position, 0 when no value beat the starting infinity
    __device__ __forceinline__ T arg(T row) const {
        if (kisnan(v)) return knan<T>();
        return v == (IsMax ? -kinf<T>() : kinf<T>()) ? T(0) : ksub(row, pos);
    }
};
// row accessor of a GenericCrossSectionalOp body: input_N[i], output_N[i]
template <typename T> struct CsRow {
    T *p;
    __device__ __forceinline__ T &operator[](size_t i) const { return p[i]; }
};
template <typename T> struct RVal {
    T v;
    __device__ __forceinline__ T value() const { return v; }
};
template <typename T> struct RRank {
    T v, less = 0, eq = 0;
    __device__ __forceinline__ RRank() {}
    __device__ __forceinline__ explicit RRank(T cur) : v(cur) {}
    __device__ __forceinline__ void reset(T cur) { v = cur; less = 0; eq = 0; }
    __device__ __forceinline__ void step(T x) {
        bool isn = kisnan(v) || kisnan(x);
        less = isn ? knan<T>() : less;
        less = (x < v) ? kadd(less, T(1.0)) : less;
        eq = (x == v) ? kadd(eq, T(1.0)) : eq;
    }
    __device__ __forceinline__ T value() const { return kadd(less, kdiv(kadd(eq, T(1.0)), T(2.0))); }
};
template <typename T, int W> struct RDecay {
    static constexpr double kStep = 1.0 / ((1.0 + W) * W / 2);
    T weight = T(kStep), v = 0;
    __device__ __forceinline__ void step(T x) {
        v = kfma(x, weight, v);
        weight = kadd(weight, T(kStep));
    }
    __device__ __forceinline__ T value() const { return v; }
};

// ---------------- stateful ops carried over time
// FastWindowedSum, cpp/Kun/Ops.hpp:324-356
template <typename T> struct FWSum {
    T v = 0, cadd = 0, csub = 0;
    int nn;
    __device__ __forceinline__ explicit FWSum(int window) : nn(window) {}
    __device__ __forceinline__ T step(T old, T cur) {
        bool on = kisnan(old), cn = kisnan(cur);
        if (!on) {
            T y = ksub(ksub(T(0), old), csub);
            T t = kadd(v, y);
            csub = ksub(ksub(t, v), y);
            v = t;
        }
        if (!cn) {
            T y = ksub(cur, cadd);
            T t = kadd(v, y);
            cadd = ksub(ksub(t, v), y);
            v = t;
        }
        nn = nn - (int)on + (int)cn;
        return nn == 0 ? v : knan<T>();
    }
};

template <> struct FWSum<DFloat> {
    DFloat v;
    int nn;
    __device__ __forceinline__ explicit FWSum(int window) : nn(window) {}
    __device__ __forceinline__ DFloat step(float old, float cur) {
        const bool on = old != old, cn = cur != cur;
        if (!on) v = df_add_f(v, -old);
        if (!cn) v = df_add_f(v, cur);
        nn = nn - (int)on + (int)cn;
        return nn == 0 ? v : knan<DFloat>();
    }
};

// ExpMovingAvg, cpp/Kun/Ops.hpp:358-375
template <typename T, int W> struct EMA {
    T v;
    __device__ __forceinline__ explicit EMA(T init) : v(init) {}
    __device__ __forceinline__ T step(T cur) {
        const T w = kdiv(T(2.0), T(W + 1));
        T nv = kfma(cur, w, kmul(v, ksub(T(1), w)));
        T r = kisnan(cur) ? v : nv;
        r = kisnan(v) ? cur : r;
        v = r;
        return r;
    }
};

// WindowedLinearRegression, cpp/Kun/Ops.hpp:377-466
template <typename T, int W> struct LinReg {
    T isum = 0, xsum = 0, x2sum = 0, ysum = 0, y2sum = 0, xysum = 0;
    int nn = W;
    // SharedSq: cur*cur is shared with another regression of the stage in
    // the reference build and is then not contracted
    template <bool SharedSq>
    __device__ __forceinline__ void step(T old, T cur) {
        const T w = T(W);
        xysum = ksub(xysum, ysum);
        x2sum = ksub(kadd(x2sum, isum), kmul(T(2.0), xsum));
        xsum = ksub(xsum, isum);
        bool on = kisnan(old), cn = kisnan(cur);
        if (!on) {
            isum = ksub(isum, T(1));
            ysum = ksub(ysum, old);
            y2sum = kfma(-old, old, y2sum);
        }
        nn = nn - (int)on + (int)cn;
        if (!cn) {
            isum = kadd(isum, T(1));
            xsum = kadd(xsum, w);
            x2sum = kadd(x2sum, kmul(w, w));
            ysum = kadd(ysum, cur);
            y2sum = SharedSq ? kadd(y2sum, kmul(cur, cur)) : kfma(cur, cur, y2sum);
            xysum = kfma(w, cur, xysum);
        }
    }
    __device__ __forceinline__ T n() const { return (T)(W - nn); }
    __device__ __forceinline__ T rsq() const {
        T N = n();
        T r1 = kfma(-xsum, ysum, kmul(N, xysum));
        r1 = kmul(r1, r1);
        T r2 = kmul(kfma(-xsum, xsum, kmul(N, x2sum)), kfma(-ysum, ysum, kmul(N, y2sum)));
        return kdiv(r1, r2);
    }
    __device__ __forceinline__ T slope() const {
        T N = n();
        return kdiv(kfma(-xsum, ysum, kmul(N, xysum)), kfma(-xsum, xsum, kmul(N, x2sum)));
    }
    __device__ __forceinline__ T resi(T val) const {
        T N = n();
        T s = slope();
        T xm = kdiv(xsum, N), ym = kdiv(ysum, N);
        T interp = kfma(-s, xm, ym);
        return ksub(val, kfma(s, T(W), interp));
    }
};

// The windowed regression of the sliding-moment form: the same recurrences
// and NaN rules as LinReg (cpp/Kun/Ops.hpp:377-466), with the index sums
// (isum, xsum, x2sum: integers below 2^24, exact in float) kept in float and
// the value sums (ysum, y2sum, xysum) in unnormalised two-float accumulators;
// the outputs are formed from those sums without the cancellation of fp32.
template <int W> struct SlideLinReg {
    float isum = 0, xsum = 0, x2sum = 0;
    // The value sums are taken about an origin c, the first non-NaN value the
    // state sees, with each difference y - c kept exactly as a pair.  The
    // state starts empty and a value leaves the window only after it entered
    // it, so every value is added and taken out about the same origin.  The
    // variance N*sum(d^2) - sum(d)^2 of a window of nearly equal values then
    // cancels at the level of their spread, not of their price (two closes
    // 1e-5 apart at 327 would otherwise lose ~1e10 x 2^-48 of it); slope,
    // R^2 and the residual do not depend on the origin.
    DFloat ysum, y2sum, xysum;
    float c = 0.f;
    bool has_c = false;
    int nn = W;
    template <bool SharedSq>
    __device__ __forceinline__ void step(float old, float cur) {
        const float w = (float)W;
        df_acc_pair(xysum, -ysum);
        x2sum = __fsub_rn(__fadd_rn(x2sum, isum), __fmul_rn(2.f, xsum));
        xsum = __fsub_rn(xsum, isum);
        const bool on = old != old, cn = cur != cur;
        if (!cn && !has_c) {
            c = cur;  // nothing has been added yet, so no old value is pending
            has_c = true;
        }
        if (!on) {
            const DFloat d = df_two_sum(old, -c);
            isum = __fsub_rn(isum, 1.f);
            df_acc(ysum, -d.hi);
            ysum.lo = __fsub_rn(ysum.lo, d.lo);
            df_acc_prod_neg(y2sum, d.hi, d.hi);
            y2sum.lo = __fmaf_rn(-2.f * d.hi, d.lo, y2sum.lo);
        }
        nn = nn - (int)on + (int)cn;
        if (!cn) {
            const DFloat d = df_two_sum(cur, -c);
            isum = __fadd_rn(isum, 1.f);
            xsum = __fadd_rn(xsum, w);
            x2sum = __fadd_rn(x2sum, w * w);
            df_acc(ysum, d.hi);
            ysum.lo = __fadd_rn(ysum.lo, d.lo);
            df_acc_prod(y2sum, d.hi, d.hi);
            y2sum.lo = __fmaf_rn(2.f * d.hi, d.lo, y2sum.lo);
            df_acc_prod(xysum, w, d.hi);
            xysum.lo = __fmaf_rn(w, d.lo, xysum.lo);
        }
    }
    __device__ __forceinline__ float n() const { return (float)(W - nn); }
    // N*xysum - xsum*ysum, as a normalised pair
    __device__ __forceinline__ DFloat cov() const {
        const float N = n();
        DFloat a = df_scale(xysum, N);
        df_acc_pair(a, df_scale(ysum, -xsum));
        return df_two_sum(a.hi, a.lo);  // hi may have cancelled below lo
    }
    // N*x2sum - xsum*xsum: exact in float
    __device__ __forceinline__ float varx() const {
        return __fsub_rn(__fmul_rn(n(), x2sum), __fmul_rn(xsum, xsum));
    }
    __device__ __forceinline__ float rsq() const {
        const float N = n();
        const DFloat ys = df_two_sum(ysum.hi, ysum.lo);
        DFloat vy = df_scale(y2sum, N);
        df_acc_pair(vy, -kmul(ys, ys));
        const float r = (float)cov();
        return __fdiv_rn(__fmul_rn(r, r), __fmul_rn(varx(), (float)vy));
    }
    __device__ __forceinline__ float slope() const { return __fdiv_rn((float)cov(), varx()); }
    // val - (slope*W + ym - slope*xm) = (N*(val-c) - ysum - slope*(W*N - xsum)) / N,
    // with the slope kept as a pair: the residual is a small difference of
    // large terms
    __device__ __forceinline__ float resi(float val) const {
        const float N = n();
        const DFloat sd = kdiv(cov(), DFloat(varx()));
        const DFloat dv = df_two_sum(val, -c);
        DFloat r = df_prod(N, dv.hi);
        r.lo = __fmaf_rn(N, dv.lo, r.lo);
        df_acc_pair(r, -ysum);
        df_acc_pair(r, -kmul(sd, DFloat(__fsub_rn(__fmul_rn((float)W, N), xsum))));
        return __fdiv_rn((float)r, N);
    }
};

// Order-statistic window of the skip-list ops (cpp/Kun/Ops/Quantile.hpp:16-170,
// cpp/Kun/SkipList.cpp:125-273): the last `W` non-NaN values kept sorted, equal
// values in insertion order.  Values are kept as double like the skip list.
template <int W> struct SortedWindow {
    double v[W + 1];
    int idx[W + 1];
    int size = 0;
    int last_rank = 0;
    __device__ __forceinline__ void remove(double x) {
        int p = 0;
        while (p < size && v[p] < x) p++;
        if (p >= size || v[p] != x) return;
        for (int j = p; j < size - 1; j++) { v[j] = v[j + 1]; idx[j] = idx[j + 1]; }
        size--;
    }
    __device__ __forceinline__ int insert(double x, int index) {
        int p = 0;
        while (p < size && v[p] <= x) p++;
        for (int j = size; j > p; j--) { v[j] = v[j - 1]; idx[j] = idx[j - 1]; }
        v[p] = x;
        idx[p] = index;
        size++;
        return p;
    }
    __device__ __forceinline__ int min_rank(double x) const {
        int p = 0;
        while (p < size && v[p] < x) p++;
        return p;
    }
    template <typename T>
    __device__ __forceinline__ void step(T oldv, T newv, int index) {
        if (!kisnan(oldv)) remove((double)oldv);
        if (!kisnan(newv)) last_rank = insert((double)newv, index);
    }
    template <typename T> __device__ __forceinline__ T quantile(T q) const {
        if (size != W) return knan<T>();
        T iwf = kmul(q, (T)(size - 1));
        int id = (int)iwf;
        if ((T)id == iwf) return (T)v[id];
        double lo = v[id], hi = v[id + 1];
        T frac = ksub(iwf, (T)id);
        return (T)__fma_rn(__dsub_rn(hi, lo), (double)frac, lo);
    }
    template <typename T> __device__ __forceinline__ T vmin() const {
        return size != W ? knan<T>() : (T)v[0];
    }
    template <typename T> __device__ __forceinline__ T vmax() const {
        return size != W ? knan<T>() : (T)v[W - 1];
    }
    template <typename T> __device__ __forceinline__ T argmin(long long cur_idx) const {
        if (size != W) return knan<T>();
        return (T)(unsigned long long)((unsigned long long)idx[0] + (unsigned long long)size -
                                       (unsigned long long)cur_idx);
    }
    template <typename T> __device__ __forceinline__ T rank(T cur) const {
        if (size != W) return knan<T>();
        double r = last_rank + 1;
        double rmin = min_rank((double)cur) + 1;
        r = (((r * (r + 1) / 2) - ((rmin - 1) * rmin / 2)) / (r - rmin + 1));
        return (T)r;
    }
};

// Register-resident form of the order-statistic window for W <= 64: the
// window is a sorted array of W registers, empty slots hold NaN (they never
// compare true, so they stay at the end and drop out of every count).  Every
// update is a fixed, branch-free compare/select network over the W slots, so
// all stocks of a warp execute the same instructions.  Semantics are those of
// SortedWindow above: removal takes the first equal value, insertion goes
// after equal values.
template <typename T, int W, bool IDX> struct RegWindow {
    T v[W];
    int ix[IDX ? W : 1];
    int size = 0;
    int last_rank = 0;
    __device__ __forceinline__ RegWindow() {
#pragma unroll
        for (int j = 0; j < W; j++) v[j] = knan<T>();
    }
    // x must be present (the caller removes only values it inserted)
    __device__ __forceinline__ void remove(T x) {
        int p = 0;
#pragma unroll
        for (int j = 0; j < W; j++) p += (v[j] < x) ? 1 : 0;
#pragma unroll
        for (int j = 0; j < W - 1; j++) {
            const bool sh = j >= p;
            v[j] = sh ? v[j + 1] : v[j];
            if (IDX) ix[j] = sh ? ix[j + 1] : ix[j];
        }
        v[W - 1] = knan<T>();
        size--;
    }
    __device__ __forceinline__ int insert(T y, int index) {
        int q = 0;
#pragma unroll
        for (int j = 0; j < W; j++) q += (v[j] <= y) ? 1 : 0;
#pragma unroll
        for (int j = W - 1; j > 0; j--) {
            v[j] = (j > q) ? v[j - 1] : ((j == q) ? y : v[j]);
            if (IDX) ix[j] = (j > q) ? ix[j - 1] : ((j == q) ? index : ix[j]);
        }
        v[0] = (q == 0) ? y : v[0];
        if (IDX) ix[0] = (q == 0) ? index : ix[0];
        size++;
        return q;
    }
    __device__ __forceinline__ int min_rank(T x) const {
        int p = 0;
#pragma unroll
        for (int j = 0; j < W; j++) p += (v[j] < x) ? 1 : 0;
        return p;
    }
    __device__ __forceinline__ void step(T oldv, T newv, int index) {
        if (!kisnan(oldv)) remove(oldv);
        if (!kisnan(newv)) last_rank = insert(newv, index);
    }
    // quantile with the rank arithmetic done at compile time: ID =
    // int(q * (W - 1)) and frac = q * (W - 1) - ID in the module dtype
    template <int ID, bool EXACT> __device__ __forceinline__ T quantile(T frac) const {
        if (size != W) return knan<T>();
        if (EXACT) return v[ID];
        double lo = (double)v[ID], hi = (double)v[ID + 1];
        return (T)__fma_rn(__dsub_rn(hi, lo), (double)frac, lo);
    }
    __device__ __forceinline__ T vmin() const { return size != W ? knan<T>() : v[0]; }
    __device__ __forceinline__ T vmax() const { return size != W ? knan<T>() : v[W - 1]; }
    __device__ __forceinline__ T argmin(long long cur_idx) const {
        if (size != W) return knan<T>();
        return (T)(unsigned long long)((unsigned long long)ix[0] + (unsigned long long)size -
                                       (unsigned long long)cur_idx);
    }
    __device__ __forceinline__ T rank(T cur) const {
        if (size != W) return knan<T>();
        double r = last_rank + 1;
        double rmin = min_rank(cur) + 1;
        r = (((r * (r + 1) / 2) - ((rmin - 1) * rmin / 2)) / (r - rmin + 1));
        return (T)r;
    }
};

}  // namespace kun
