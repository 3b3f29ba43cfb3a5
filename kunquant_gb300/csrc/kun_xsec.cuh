// Cross-sectional kernels: one thread block per time step (row of the [T][S]
// layout).
//  - Rank (cpp/Kun/Rank.hpp:13-57): the row's non-NaN values are sorted by a
//    register/shuffle/shared-memory bitonic network over order-preserving
//    integer keys (NaNs sort last), or for long rows an 8-bit LSD radix sort;
//    every stock then finds its equal range;
//    out = T(sum) / T(cnt) / T(n) with the integer rank sum of the range.
//  - Scale (cpp/Kun/Scale.hpp:14-46): the sum of |x| over non-NaN stocks in
//    stock order (sequential, as the reference adds), then x / sum.
//  - DiffWithWeightedSum (KunQuant/ops/MiscOp.py:220-240).
#pragma once
#include "kun_device.cuh"

namespace kun {

template <typename T> struct SortKey;
template <> struct SortKey<float> {
    using K = uint32_t;
    static __device__ __forceinline__ K enc(float x) {
        if (x != x) return 0xffffffffu;
        uint32_t u = __float_as_uint(x);
        return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
    }
    static __device__ __forceinline__ float dec(K k) {
        uint32_t u = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
        return __uint_as_float(u);
    }
    static constexpr K kMax = 0xffffffffu;
};
template <> struct SortKey<double> {
    using K = unsigned long long;
    static __device__ __forceinline__ K enc(double x) {
        if (x != x) return ~0ull;
        unsigned long long u = (unsigned long long)__double_as_longlong(x);
        return (u & 0x8000000000000000ull) ? ~u : (u | 0x8000000000000000ull);
    }
    static __device__ __forceinline__ double dec(K k) {
        unsigned long long u = (k & 0x8000000000000000ull) ? (k & 0x7fffffffffffffffull) : ~k;
        return __longlong_as_double((long long)u);
    }
    static constexpr K kMax = ~0ull;
};

constexpr int kRankThreads = 1024;
// dynamic shared memory above which a launch first raises the kernel's
// limit: 48 KB less room for the kernels' static arrays
constexpr size_t kSmemOptIn = 40 * 1024;
constexpr int kRadixMinP = 2048;  // rows at least this long (padded) use the radix sort
__host__ __device__ inline int skew(int p) { return p + (p >> 5); }
// keys per thread for a sort of P keys by kRankThreads threads
__host__ __device__ inline int rank_items(int P) {
    return P <= 8 * kRankThreads ? 8 : (P <= 16 * kRankThreads ? 16 : 32);
}
// key slots of a rank block's shared memory for rows padded to P: the radix
// sort works on all kRankThreads * ITEMS positions
__host__ __device__ inline int rank_key_slots(int P) {
    return (P >= kRadixMinP ? skew(kRankThreads * rank_items(P)) : skew(P)) + 1;
}

// Rank of one row by the whole block.  The row's keys (NaN -> max key) are
// sorted with a bitonic network over P = a power of two >= the row length:
// thread t holds positions [t*ITEMS, (t+1)*ITEMS) in registers, so the
// network's exchanges at distance j < ITEMS stay in registers, j < 32*ITEMS
// go through warp shuffles, and only the longer ones pass through shared
// memory (keys[e*nt + t], conflict-free) with a block barrier.  Each stock
// then binary-searches the equal range of its value in the sorted keys.
template <typename K>
__device__ __forceinline__ void bitonic_keep(K &mine, K other, bool lower, bool up) {
    K mn = other < mine ? other : mine, mx = other < mine ? mine : other;
    mine = (lower == up) ? mn : mx;
}

// out[i] from the sorted non-NaN values (at(p), p < n): the average rank of
// x's equal range over n (cpp/Kun/Rank.hpp:40-53)
template <typename T, typename At>
__device__ __forceinline__ void rank_from_sorted(const T *__restrict__ row, T *__restrict__ orow, long long S, int n,
                                                 At at) {
    for (long long i = threadIdx.x; i < S; i += blockDim.x) {
        T x = row[i];
        T res;
        if (x != x) {
            res = knan<T>();
        } else {
            int lo = 0, hi = n;
            while (lo < hi) { int m = (lo + hi) >> 1; if (at(m) < x) lo = m + 1; else hi = m; }
            long long start = lo;
            hi = n;
            while (lo < hi) { int m = (lo + hi) >> 1; if (x < at(m)) hi = m; else lo = m + 1; }
            long long end = lo;
            long long sum = (start + end + 1) * (end - start) / 2;
            res = kdiv(kdiv((T)sum, (T)(end - start)), (T)n);
        }
        orow[i] = res;
    }
    __syncthreads();
}

template <typename T, int ITEMS>
__device__ __forceinline__ void rank_one_row(const T *__restrict__ row, T *__restrict__ orow, long long S, int P,
                                             typename SortKey<T>::K *keys, int *cnt_warp) {
    using SK = SortKey<T>;
    using K = typename SK::K;
    const int tid = threadIdx.x;
    const int nt = P / ITEMS;  // threads holding keys (P >= ITEMS)
    K r[ITEMS];
    int local = 0;
#pragma unroll
    for (int e = 0; e < ITEMS; e++) {
        r[e] = SK::kMax;
        const long long i = (long long)tid * ITEMS + e;
        if (tid < nt && i < S) {
            T x = row[i];
            r[e] = SK::enc(x);
            local += (x == x);
        }
    }
    for (int o = 16; o > 0; o >>= 1) local += __shfl_xor_sync(0xffffffffu, local, o);
    if ((tid & 31) == 0) cnt_warp[tid >> 5] = local;
    __syncthreads();
    int n = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) n += cnt_warp[w];
    for (int k = 2; k <= P; k <<= 1) {
        for (int j = k >> 1; j >= ITEMS; j >>= 1) {
            if (j >= ITEMS * 32) {
                const int m = j / ITEMS;
                if (tid < nt) {
#pragma unroll
                    for (int e = 0; e < ITEMS; e++) keys[e * nt + tid] = r[e];
                }
                __syncthreads();
                if (tid < nt) {
                    const int pt = tid ^ m;
                    const bool lower = (tid & m) == 0;
#pragma unroll
                    for (int e = 0; e < ITEMS; e++) {
                        const int i = tid * ITEMS + e;
                        bitonic_keep(r[e], keys[e * nt + pt], lower, (i & k) == 0);
                    }
                }
                __syncthreads();
            } else {
                const int m = j / ITEMS;
                const bool lower = (tid & m) == 0;
#pragma unroll
                for (int e = 0; e < ITEMS; e++) {
                    const int i = tid * ITEMS + e;
                    K o = __shfl_xor_sync(0xffffffffu, r[e], m);
                    bitonic_keep(r[e], o, lower, (i & k) == 0);
                }
            }
        }
        // distances below ITEMS: within the thread, unrolled so that r stays
        // in registers
#pragma unroll
        for (int j = ITEMS / 2; j > 0; j >>= 1) {
            if (j < k) {
#pragma unroll
                for (int e = 0; e < ITEMS; e++) {
                    if ((e & j) == 0) {
                        const int i = tid * ITEMS + e;
                        const bool up = (i & k) == 0;
                        K a = r[e], b = r[e ^ j];
                        if ((a > b) == up) {
                            r[e] = b;
                            r[e ^ j] = a;
                        }
                    }
                }
            }
        }
    }
    // sorted position p = t*ITEMS + e lives at keys[e*nt + t]
    if (tid < nt) {
#pragma unroll
        for (int e = 0; e < ITEMS; e++) keys[e * nt + tid] = r[e];
    }
    __syncthreads();
    rank_from_sorted<T>(row, orow, S, n, [&](int p) { return SK::dec(keys[(p % ITEMS) * nt + p / ITEMS]); });
}

// Rank of one row by LSD radix sort (8-bit digits, stable), for long rows
// where the bitonic network's P log^2 P exchanges cost more than the digit
// passes.  blockDim.x must be kRankThreads.  Between passes the values sit in
// layout order: warp w, item e, lane l holds position w*32*ITEMS + e*32 + l.
// Only the non-NaN values are sorted, each with its stock index, and only
// the digits in which they differ are passed over.  A pass counts digits per
// warp (peers of a digit found with match.any, so an item's offset is the
// warp's running count of its digit plus its peers in lower lanes), scans
// the counts in (digit, warp) order and scatters.  The ranks then come from
// the sorted run of equal values around each position (two block scans)
// instead of binary searches.  Shared memory: keys and 16-bit stock indices
// (skewed by one slot every 32), and kRankThreads/32 x 257 digit counters.
constexpr int kRadixHistStride = 257;  // 256 digits + 1: warps' rows skewed by one bank
__host__ __device__ inline int radix_hist_slots() { return (kRankThreads / 32) * kRadixHistStride; }

template <typename T, int ITEMS>
__device__ __forceinline__ void rank_one_row_radix(const T *__restrict__ row, T *__restrict__ orow, long long S,
                                                   typename SortKey<T>::K *keys, uint32_t *hist,
                                                   uint16_t *idx, int *cnt_warp) {
    using SK = SortKey<T>;
    using K = typename SK::K;
    constexpr int NT = kRankThreads;
    constexpr int NW = NT / 32;
    static_assert(NT == 1024, "the digit-count scan gives each thread 8 of 256 x 32 counts");
    constexpr int BITS = (int)sizeof(K) * 8;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const unsigned lt_mask = (1u << lane) - 1u;
    __shared__ int warp_tot[NW], warp_tot2[NW];
    __shared__ K red_or[NW], red_and[NW];
    K r[ITEMS];
    uint16_t ix[ITEMS];
    bool real[ITEMS];
    int local = 0;
    K o_or = 0, o_and = ~K(0);
    const int wbase = warp * 32 * ITEMS + lane;  // layout position of item 0
#pragma unroll
    for (int e = 0; e < ITEMS; e++) {
        const int i = wbase + e * 32;
        real[e] = false;
        r[e] = SK::kMax;
        ix[e] = (uint16_t)i;
        if (i < S) {
            T x = row[i];
            if (x == x) {
                real[e] = true;
                r[e] = SK::enc(x);
                local++;
                o_or |= r[e];
                o_and &= r[e];
            } else {
                orow[i] = knan<T>();
            }
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        local += __shfl_xor_sync(0xffffffffu, local, o);
        o_or |= __shfl_xor_sync(0xffffffffu, o_or, o);
        o_and &= __shfl_xor_sync(0xffffffffu, o_and, o);
    }
    if (lane == 0) {
        cnt_warp[warp] = local;
        red_or[warp] = o_or;
        red_and[warp] = o_and;
    }
    __syncthreads();
    int n = 0;
    K orv = 0, andv = ~K(0);
    for (int w = 0; w < NW; w++) {
        n += cnt_warp[w];
        orv |= red_or[w];
        andv &= red_and[w];
    }
    if (n == 0) {  // an all-NaN row: its outputs are written above
        __syncthreads();
        return;
    }
    // digits in which the values differ (at least one pass, which also
    // compacts the non-NaN values to positions [0, n))
    K todo = orv ^ andv;
    if (todo == 0) todo = 1;
    int last_shift = 0;
    for (int sh = 0; sh < BITS; sh += 8)
        if ((todo >> sh) & 255) last_shift = sh;
    uint32_t *my_hist = hist + warp * kRadixHistStride;
    for (int shift = 0; shift < BITS; shift += 8) {
        if (((todo >> shift) & 255) == 0) continue;
        for (int d = lane; d < 256; d += 32) my_hist[d] = 0;
        __syncwarp();
        // per-warp counts; off[e] = the item's place among its warp's items
        // of the same digit, in layout order
        uint16_t off[ITEMS];
#pragma unroll
        for (int e = 0; e < ITEMS; e++) {
            const int d = real[e] ? (int)((r[e] >> shift) & 255) : 256;
            const unsigned peers = __match_any_sync(0xffffffffu, d);
            const int leader = __ffs(peers) - 1;
            uint32_t base = 0;
            if (lane == leader && d < 256) {
                base = my_hist[d];
                my_hist[d] = base + (uint32_t)__popc(peers);
            }
            base = __shfl_sync(0xffffffffu, base, leader);
            off[e] = (uint16_t)(base + (uint32_t)__popc(peers & lt_mask));
            __syncwarp();
        }
        __syncthreads();
        // exclusive scan of the counts in (digit, warp) order: thread t takes
        // the 8 entries of digit t/4, warps (t%4)*8 .. +8
        {
            const int d = tid >> 2, w0 = (tid & 3) * 8;
            uint32_t c[8];
            int sum = 0;
#pragma unroll
            for (int j = 0; j < 8; j++) {
                c[j] = hist[(w0 + j) * kRadixHistStride + d];
                sum += (int)c[j];
            }
            int incl = sum;
            for (int o = 1; o < 32; o <<= 1) {
                int v = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += v;
            }
            if (lane == 31) warp_tot[warp] = incl;
            __syncthreads();
            if (tid < 32) {
                int v = tid < NW ? warp_tot[tid] : 0;
                int x = v;
                for (int o = 1; o < 32; o <<= 1) {
                    int y = __shfl_up_sync(0xffffffffu, x, o);
                    if (tid >= o) x += y;
                }
                if (tid < NW) warp_tot[tid] = x - v;  // exclusive
            }
            __syncthreads();
            uint32_t run = (uint32_t)(warp_tot[warp] + incl - sum);
#pragma unroll
            for (int j = 0; j < 8; j++) {
                hist[(w0 + j) * kRadixHistStride + d] = run;
                run += c[j];
            }
        }
        __syncthreads();
#pragma unroll
        for (int e = 0; e < ITEMS; e++) {
            if (real[e]) {
                const int d = (int)((r[e] >> shift) & 255);
                const int pos = skew((int)my_hist[d] + off[e]);
                keys[pos] = r[e];
                idx[pos] = ix[e];
            }
        }
        __syncthreads();
        if (shift != last_shift) {
#pragma unroll
            for (int e = 0; e < ITEMS; e++) {
                const int p = wbase + e * 32;
                real[e] = p < n;
                if (real[e]) {
                    r[e] = keys[skew(p)];
                    ix[e] = idx[skew(p)];
                }
            }
        }
        __syncthreads();
    }
    // Equal runs of the sorted values: start(p) = the last run boundary at or
    // before p (block max-scan), end(p) = one past the run (block min-scan
    // from the right).  Equality is the values' (-0 == +0), not the keys'.
    T v[ITEMS];
#pragma unroll
    for (int e = 0; e < ITEMS; e++) {
        const int p = tid * ITEMS + e;
        v[e] = p < n ? SK::dec(keys[skew(p)]) : T(0);
    }
    const int p0 = tid * ITEMS;
    const T before = (p0 > 0 && p0 - 1 < n) ? SK::dec(keys[skew(p0 - 1)]) : T(0);
    const T after = (p0 + ITEMS < n) ? SK::dec(keys[skew(p0 + ITEMS)]) : T(0);
    int st[ITEMS], en[ITEMS];
    int m = -1;
#pragma unroll
    for (int e = 0; e < ITEMS; e++) {
        const int p = p0 + e;
        const T prev = e == 0 ? before : v[e - 1];
        if (p < n && (p == 0 || !(v[e] == prev))) m = p;
        st[e] = m;
    }
    int mn = 1 << 30;
#pragma unroll
    for (int e = ITEMS - 1; e >= 0; e--) {
        const int p = p0 + e;
        const T next = e == ITEMS - 1 ? after : v[e + 1];
        if (p < n && (p == n - 1 || !(v[e] == next))) mn = p + 1;
        en[e] = mn;
    }
    // forward exclusive max over threads of m, backward exclusive min of mn
    int fx = m, bx = mn;
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, fx, o);
        if (lane >= o) fx = max(fx, y);
        int z = __shfl_down_sync(0xffffffffu, bx, o);
        if (lane + o < 32) bx = min(bx, z);
    }
    if (lane == 31) warp_tot[warp] = fx;
    if (lane == 0) warp_tot2[warp] = bx;
    int fex = __shfl_up_sync(0xffffffffu, fx, 1);
    int bex = __shfl_down_sync(0xffffffffu, bx, 1);
    if (lane == 0) fex = -1;
    if (lane == 31) bex = 1 << 30;
    __syncthreads();
    if (tid < 32) {
        int a = warp_tot[tid], b = warp_tot2[tid];
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, a, o);
            if (tid >= o) a = max(a, y);
            int z = __shfl_down_sync(0xffffffffu, b, o);
            if (tid + o < 32) b = min(b, z);
        }
        int ae = __shfl_up_sync(0xffffffffu, a, 1);
        int be = __shfl_down_sync(0xffffffffu, b, 1);
        warp_tot[tid] = tid == 0 ? -1 : ae;
        warp_tot2[tid] = tid == 31 ? (1 << 30) : be;
    }
    __syncthreads();
    const int start_in = max(fex, warp_tot[warp]);
    const int end_in = min(bex, warp_tot2[warp]);
    T res[ITEMS];
    int sidx[ITEMS];
#pragma unroll
    for (int e = 0; e < ITEMS; e++) {
        const int p = p0 + e;
        sidx[e] = -1;
        if (p < n) {
            const long long start = max(st[e], start_in);
            const long long end = min(en[e], end_in);
            const long long sum = (start + end + 1) * (end - start) / 2;
            res[e] = kdiv(kdiv((T)sum, (T)(end - start)), (T)n);
            sidx[e] = idx[skew(p)];
        }
    }
    // the results go to shared memory by stock index (over the keys, no
    // longer needed), then out in one coalesced pass over the row
    __syncthreads();
    T *out_s = reinterpret_cast<T *>(keys);
#pragma unroll
    for (int e = 0; e < ITEMS; e++)
        if (sidx[e] >= 0) out_s[sidx[e]] = res[e];
    __syncthreads();
    for (long long i = tid; i < S; i += NT) {
        const T x = row[i];
        orow[i] = x == x ? out_s[i] : knan<T>();
    }
    __syncthreads();
}

// Rank of one long row without sorting it: each non-NaN value goes to one
// of kBucketN buckets by a monotone map of its value, and from the bucket
// counts' exclusive scan a value's rank start is the number of values in
// lower buckets plus those in its own bucket that are smaller; its end adds
// the equal ones.  These are exactly the start and end of its equal range in
// the sorted row (cpp/Kun/Rank.hpp:40-53), so the result is the sort's bit
// for bit.  Two maps are counted and the one with the smaller largest bucket
// is used: linear in the value (floor((x - min) * scale), monotone because
// each rounded step is) for values spread evenly, and linear in the
// order-preserving key (logarithmic in the value; -0 keyed as +0 so equal
// values share a bucket) for values spread over many binades.  Work is O(n)
// plus the bucket sizes; a row whose largest bucket under both maps holds
// more than kBucketMax values (heavy ties, outliers) is left to the radix
// sort: the function then returns false before writing anything.  Shared
// memory: the bucketed values over `keys`, the two maps' counts and the fill
// counters over `counters`.
constexpr int kBucketLog = 11;
constexpr int kBucketN = 1 << kBucketLog;
constexpr int kBucketMax = 48;

template <typename T, int ITEMS>
__device__ __forceinline__ bool rank_one_row_bucket(const T *__restrict__ row, T *__restrict__ orow, long long S,
                                                    typename SortKey<T>::K *keys, uint32_t *counters) {
    using SK = SortKey<T>;
    using K = typename SK::K;
    constexpr int NT = kRankThreads;
    constexpr int NW = NT / 32;
    static_assert(kBucketN * 3 <= (NT / 32) * kRadixHistStride, "bucket counters fit the radix counters");
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    __shared__ K red_lo[NW], red_hi[NW];
    __shared__ T red_vlo[NW], red_vhi[NW];
    __shared__ int red_n[NW], red_c[NW], red_c2[NW];
    __shared__ int scan_w[NW];
    uint32_t *hist_v = counters, *hist_k = counters + kBucketN, *fill = counters + 2 * kBucketN;
    T v[ITEMS];
    K k[ITEMS];
    int local = 0;
    K lo = SK::kMax, hi = 0;
    T vlo = kinf<T>(), vhi = -kinf<T>();
#pragma unroll
    for (int e = 0; e < ITEMS; e++) {
        const long long i = (long long)e * NT + tid;
        v[e] = knan<T>();
        k[e] = 0;
        if (i < S) {
            const T x = row[i];
            v[e] = x;
            if (x == x) {
                k[e] = SK::enc(x == T(0) ? T(0) : x);
                local++;
                lo = k[e] < lo ? k[e] : lo;
                hi = k[e] > hi ? k[e] : hi;
                vlo = x < vlo ? x : vlo;
                vhi = x > vhi ? x : vhi;
            }
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        local += __shfl_xor_sync(0xffffffffu, local, o);
        const K l2 = __shfl_xor_sync(0xffffffffu, lo, o), h2 = __shfl_xor_sync(0xffffffffu, hi, o);
        lo = l2 < lo ? l2 : lo;
        hi = h2 > hi ? h2 : hi;
        const T vl2 = __shfl_xor_sync(0xffffffffu, vlo, o), vh2 = __shfl_xor_sync(0xffffffffu, vhi, o);
        vlo = vl2 < vlo ? vl2 : vlo;
        vhi = vh2 > vhi ? vh2 : vhi;
    }
    if (lane == 0) {
        red_n[warp] = local;
        red_lo[warp] = lo;
        red_hi[warp] = hi;
        red_vlo[warp] = vlo;
        red_vhi[warp] = vhi;
    }
    for (int b = tid; b < 3 * kBucketN; b += NT) counters[b] = 0;
    __syncthreads();
    // warp 0 combines the warps' partials and leaves the row's in slot 0
    if (warp == 0) {
        local = lane < NW ? red_n[lane] : 0;
        lo = lane < NW ? red_lo[lane] : SK::kMax;
        hi = lane < NW ? red_hi[lane] : K(0);
        vlo = lane < NW ? red_vlo[lane] : kinf<T>();
        vhi = lane < NW ? red_vhi[lane] : -kinf<T>();
        for (int o = 16; o > 0; o >>= 1) {
            local += __shfl_xor_sync(0xffffffffu, local, o);
            const K l2 = __shfl_xor_sync(0xffffffffu, lo, o), h2 = __shfl_xor_sync(0xffffffffu, hi, o);
            lo = l2 < lo ? l2 : lo;
            hi = h2 > hi ? h2 : hi;
            const T vl2 = __shfl_xor_sync(0xffffffffu, vlo, o), vh2 = __shfl_xor_sync(0xffffffffu, vhi, o);
            vlo = vl2 < vlo ? vl2 : vlo;
            vhi = vh2 > vhi ? vh2 : vhi;
        }
        if (lane == 0) {
            red_n[0] = local;
            red_lo[0] = lo;
            red_hi[0] = hi;
            red_vlo[0] = vlo;
            red_vhi[0] = vhi;
        }
    }
    __syncthreads();
    const int n = red_n[0];
    lo = red_lo[0];
    hi = red_hi[0];
    vlo = red_vlo[0];
    vhi = red_vhi[0];
    if (n > 0) {
        const K range = hi - lo;
        int bits = 0;
        while (bits < (int)(sizeof(K) * 8) && (range >> bits) != 0) bits++;
        const int shift = bits > kBucketLog ? bits - kBucketLog : 0;
        // linear map: scale so that the largest value lands in the last
        // bucket (a non-finite or zero spread puts every value in bucket 0)
        const T spread = vhi - vlo;
        const T scale = (spread > T(0) && spread < kinf<T>()) ? T(kBucketN - 1) / spread : T(0);
        auto bucket_v = [&](T x) {
            const T f = (x - vlo) * scale;
            const int b = f >= T(kBucketN - 1) ? kBucketN - 1 : (f > T(0) ? (int)f : 0);
            return b;
        };
        auto bucket_k = [&](K key) { return (int)((key - lo) >> shift); };
#pragma unroll
        for (int e = 0; e < ITEMS; e++)
            if (v[e] == v[e]) {
                atomicAdd(&hist_v[bucket_v(v[e])], 1u);
                atomicAdd(&hist_k[bucket_k(k[e])], 1u);
            }
        __syncthreads();
        // the map with the smaller largest bucket; the radix sort if both
        // overflow
        int mv = 0, mk = 0;
        for (int b = tid; b < kBucketN; b += NT) {
            mv = max(mv, (int)hist_v[b]);
            mk = max(mk, (int)hist_k[b]);
        }
        for (int o = 16; o > 0; o >>= 1) {
            mv = max(mv, __shfl_xor_sync(0xffffffffu, mv, o));
            mk = max(mk, __shfl_xor_sync(0xffffffffu, mk, o));
        }
        if (lane == 0) {
            red_c[warp] = mv;
            red_c2[warp] = mk;
        }
        __syncthreads();
        if (warp == 0) {
            mv = lane < NW ? red_c[lane] : 0;
            mk = lane < NW ? red_c2[lane] : 0;
            for (int o = 16; o > 0; o >>= 1) {
                mv = max(mv, __shfl_xor_sync(0xffffffffu, mv, o));
                mk = max(mk, __shfl_xor_sync(0xffffffffu, mk, o));
            }
            if (lane == 0) {
                red_c[0] = mv;
                red_c2[0] = mk;
            }
        }
        __syncthreads();
        mv = red_c[0];
        mk = red_c2[0];
        if (mv > kBucketMax && mk > kBucketMax) {
            __syncthreads();
            return false;
        }
        const bool lin = mv <= mk;
        uint32_t *hist = lin ? hist_v : hist_k;
        // exclusive scan of the counts (kBucketN / NT per thread, in order)
        constexpr int PER = kBucketN / NT;
        uint32_t c[PER], sum = 0;
#pragma unroll
        for (int j = 0; j < PER; j++) {
            c[j] = hist[tid * PER + j];
            sum += c[j];
        }
        uint32_t incl = sum;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        if (lane == 31) scan_w[warp] = (int)incl;
        __syncthreads();
        if (tid < 32) {
            int x = tid < NW ? scan_w[tid] : 0;
            const int v0 = x;
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, x, o);
                if (tid >= o) x += y;
            }
            if (tid < NW) scan_w[tid] = x - v0;
        }
        __syncthreads();
        uint32_t run = (uint32_t)scan_w[warp] + incl - sum;
#pragma unroll
        for (int j = 0; j < PER; j++) {
            hist[tid * PER + j] = run;
            run += c[j];
        }
        __syncthreads();
        // the values by bucket (unordered inside a bucket)
        T *vals = reinterpret_cast<T *>(keys);
        int bk[ITEMS];
#pragma unroll
        for (int e = 0; e < ITEMS; e++) {
            bk[e] = 0;
            if (v[e] == v[e]) {
                bk[e] = lin ? bucket_v(v[e]) : bucket_k(k[e]);
                vals[hist[bk[e]] + atomicAdd(&fill[bk[e]], 1u)] = v[e];
            }
        }
        __syncthreads();
#pragma unroll
        for (int e = 0; e < ITEMS; e++) {
            const long long i = (long long)e * NT + tid;
            if (i >= S) continue;
            T res = knan<T>();
            if (v[e] == v[e]) {
                const int b = bk[e];
                const int p0 = (int)hist[b], p1 = b + 1 < kBucketN ? (int)hist[b + 1] : n;
                int less = p0, eq = 0;
                for (int p = p0; p < p1; p++) {
                    const T y = vals[p];
                    less += (y < v[e]);
                    eq += (y == v[e]);
                }
                const long long start = less, end = (long long)less + eq;
                const long long rsum = (start + end + 1) * (end - start) / 2;
                res = kdiv(kdiv((T)rsum, (T)(end - start)), (T)n);
            }
            orow[i] = res;
        }
    } else {
#pragma unroll
        for (int e = 0; e < ITEMS; e++) {
            const long long i = (long long)e * NT + tid;
            if (i < S) orow[i] = knan<T>();
        }
    }
    __syncthreads();
    return true;
}

// shared memory of a rank block sorting up to P keys
template <typename T>
inline size_t rank_smem_bytes(int P) {
    using K = typename SortKey<T>::K;
    size_t keys = ((size_t)rank_key_slots(P) * sizeof(K) + 15) / 16 * 16;
    return P >= kRadixMinP ? keys + (size_t)radix_hist_slots() * sizeof(uint32_t) +
                                 (size_t)rank_key_slots(P) * sizeof(uint16_t)
                           : keys;
}

template <typename T, int ITEMS>
__global__ void __launch_bounds__(kRankThreads) rank_rows(const T *__restrict__ in, T *__restrict__ out,
                                                          long long S, long long length, int P) {
    using K = typename SortKey<T>::K;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int cnt_warp[kRankThreads / 32];
    K *keys = reinterpret_cast<K *>(smem_raw);
    uint32_t *counters = reinterpret_cast<uint32_t *>(smem_raw + ((size_t)rank_key_slots(P) * sizeof(K) + 15) / 16 * 16);
    uint16_t *idx = reinterpret_cast<uint16_t *>(counters + radix_hist_slots());
    for (long long t = blockIdx.x; t < length; t += gridDim.x) {
        if (P >= kRadixMinP) {
            if (!rank_one_row_bucket<T, ITEMS>(in + t * S, out + t * S, S, keys, counters))
                rank_one_row_radix<T, ITEMS>(in + t * S, out + t * S, S, keys, counters, idx, cnt_warp);
        } else {
            rank_one_row<T, ITEMS>(in + t * S, out + t * S, S, P, keys, cnt_warp);
        }
    }
}

// stream mode: one block per segment, each at its own ring row
template <typename T, int ITEMS>
__global__ void __launch_bounds__(kRankThreads) rank_segments(const T *__restrict__ in, int w_in, T *__restrict__ out,
                                                              int w_out, long long cap, const int32_t *seg_off,
                                                              const int32_t *seg_stock0, const long long *seg_tick,
                                                              int P, const int32_t *cnt) {
    using K = typename SortKey<T>::K;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int cnt_warp[kRankThreads / 32];
    const int k = blockIdx.x;
    if (cnt && k >= cnt[0]) return;
    const long long len = seg_off[k + 1] - seg_off[k], s0 = seg_stock0[k], n = seg_tick[k];
    // sort only the power of two this segment needs (P bounds every segment)
    if (len > P) return;
    int Pk = ITEMS;
    while (Pk < len) Pk <<= 1;
    K *keys = reinterpret_cast<K *>(smem_raw);
    uint32_t *counters = reinterpret_cast<uint32_t *>(smem_raw + ((size_t)rank_key_slots(P) * sizeof(K) + 15) / 16 * 16);
    uint16_t *idx = reinterpret_cast<uint16_t *>(counters + radix_hist_slots());
    if (Pk >= kRadixMinP) {
        if (!rank_one_row_bucket<T, ITEMS>(in + (n % w_in) * cap + s0, out + (n % w_out) * cap + s0, len, keys,
                                           counters))
            rank_one_row_radix<T, ITEMS>(in + (n % w_in) * cap + s0, out + (n % w_out) * cap + s0, len, keys,
                                         counters, idx, cnt_warp);
    } else
        rank_one_row<T, ITEMS>(in + (n % w_in) * cap + s0, out + (n % w_out) * cap + s0, len, Pk, keys, cnt_warp);
}

// Stream mode, several Rank stages at once: block (k, j) ranks segment k
// for stage j of the job table (the stages of one level of the stage graph,
// which do not depend on each other).  Each job names the stage's input and
// output rings; the segment table is the step's.
struct RankJob {
    const void *in;
    void *out;
    int32_t w_in, w_out;
};

// Segments of at most kRankSmallMax stocks go to blocks of kRankSmallThreads
// threads (a bitonic sort of at most 1024 keys, 8 per thread); longer ones to
// kRankThreads-thread blocks.  A step's table lists its small segments first
// and holds their number in cnt[3].
constexpr int kRankSmallMax = 1024;
constexpr int kRankSmallThreads = kRankSmallMax / 8;

template <typename T, int ITEMS, bool SMALL>
__global__ void __launch_bounds__(SMALL ? kRankSmallThreads : kRankThreads)
    rank_multi_segments(const RankJob *__restrict__ jobs, long long cap, const int32_t *seg_off,
                        const int32_t *seg_stock0, const long long *seg_tick, int P, const int32_t *cnt) {
    using K = typename SortKey<T>::K;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int cnt_warp[kRankThreads / 32];
    const int k = blockIdx.x;
    if (cnt && (k >= cnt[0] || (SMALL ? k >= cnt[3] : k < cnt[3]))) return;
    const RankJob jb = jobs[blockIdx.y];
    const long long len = seg_off[k + 1] - seg_off[k], s0 = seg_stock0[k], n = seg_tick[k];
    if (len > P || len <= 0 || (SMALL && len > kRankSmallMax)) return;
    int Pk = ITEMS;
    while (Pk < len) Pk <<= 1;
    const T *in = (const T *)jb.in + (n % jb.w_in) * cap + s0;
    T *out = (T *)jb.out + (n % jb.w_out) * cap + s0;
    K *keys = reinterpret_cast<K *>(smem_raw);
    uint32_t *counters = reinterpret_cast<uint32_t *>(smem_raw + ((size_t)rank_key_slots(P) * sizeof(K) + 15) / 16 * 16);
    uint16_t *idx = reinterpret_cast<uint16_t *>(counters + radix_hist_slots());
    if (SMALL)
        rank_one_row<T, ITEMS>(in, out, len, Pk, keys, cnt_warp);
    else if (Pk >= kRadixMinP) {
        if (!rank_one_row_bucket<T, ITEMS>(in, out, len, keys, counters))
            rank_one_row_radix<T, ITEMS>(in, out, len, keys, counters, idx, cnt_warp);
    } else
        rank_one_row<T, ITEMS>(in, out, len, Pk, keys, cnt_warp);
}

template <typename T>
__global__ void __launch_bounds__(256) scale_rows(const T *__restrict__ in, T *__restrict__ out, long long S,
                                                  long long length) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *row_s = reinterpret_cast<T *>(smem_raw);
    __shared__ T total;
    for (long long t = blockIdx.x; t < length; t += gridDim.x) {
        const T *row = in + t * S;
        for (long long i = threadIdx.x; i < S; i += blockDim.x) row_s[i] = row[i];
        __syncthreads();
        if (threadIdx.x == 0) {
            T sum = 0;
            for (long long i = 0; i < S; i++) {
                T x = row_s[i];
                if (x == x) sum = kadd(sum, kabs(x));
            }
            total = sum;
        }
        __syncthreads();
        T sum = total;
        for (long long i = threadIdx.x; i < S; i += blockDim.x) {
            T x = row_s[i];
            out[t * S + i] = (x == T(0) && sum == T(0)) ? knan<T>() : kdiv(x, sum);
        }
        __syncthreads();
    }
}

template <typename T>
__global__ void __launch_bounds__(256) diffwsum_rows(const T *__restrict__ in0, const T *__restrict__ in1,
                                                    T *__restrict__ out, long long S, long long length) {
    __shared__ T total;
    for (long long t = blockIdx.x; t < length; t += gridDim.x) {
        if (threadIdx.x == 0) {
            T sum = 0;
            for (long long i = 0; i < S; i++) sum = kadd(sum, kmul(in0[t * S + i], in1[t * S + i]));
            total = sum;
        }
        __syncthreads();
        T sum = total;
        for (long long i = threadIdx.x; i < S; i += blockDim.x) out[t * S + i] = ksub(in0[t * S + i], sum);
        __syncthreads();
    }
}

template <typename T>
__global__ void __launch_bounds__(256) scale_segments(const T *__restrict__ in, int w_in, T *__restrict__ out,
                                                      int w_out, long long cap, const int32_t *seg_off,
                                                      const int32_t *seg_stock0, const long long *seg_tick,
                                                      const int32_t *cnt, int max_len) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *row_s = reinterpret_cast<T *>(smem_raw);
    __shared__ T total;
    const int k = blockIdx.x;
    if (cnt && k >= cnt[0]) return;
    const long long len = seg_off[k + 1] - seg_off[k], s0 = seg_stock0[k], n = seg_tick[k];
    if (len > max_len) return;
    const T *row = in + (n % w_in) * cap + s0;
    T *orow = out + (n % w_out) * cap + s0;
    // stage the row in shared memory, then one thread adds in stock order
    // (the reference's sequential sum)
    for (long long i = threadIdx.x; i < len; i += blockDim.x) row_s[i] = row[i];
    __syncthreads();
    if (threadIdx.x == 0) {
        T sum = 0;
        for (long long i = 0; i < len; i++) {
            T x = row_s[i];
            if (x == x) sum = kadd(sum, kabs(x));
        }
        total = sum;
    }
    __syncthreads();
    const T sum = total;
    for (long long i = threadIdx.x; i < len; i += blockDim.x) {
        T x = row_s[i];
        orow[i] = (x == T(0) && sum == T(0)) ? knan<T>() : kdiv(x, sum);
    }
}

template <typename T>
__global__ void __launch_bounds__(256) diffwsum_segments(const T *__restrict__ in0, int w0, const T *__restrict__ in1,
                                                         int w1, T *__restrict__ out, int w_out, long long cap,
                                                         const int32_t *seg_off, const int32_t *seg_stock0,
                                                         const long long *seg_tick, const int32_t *cnt) {
    __shared__ T total;
    const int k = blockIdx.x;
    if (cnt && k >= cnt[0]) return;
    const long long len = seg_off[k + 1] - seg_off[k], s0 = seg_stock0[k], n = seg_tick[k];
    const T *a = in0 + (n % w0) * cap + s0, *b = in1 + (n % w1) * cap + s0;
    T *orow = out + (n % w_out) * cap + s0;
    if (threadIdx.x == 0) {
        T sum = 0;
        for (long long i = 0; i < len; i++) sum = kadd(sum, kmul(a[i], b[i]));
        total = sum;
    }
    __syncthreads();
    const T sum = total;
    for (long long i = threadIdx.x; i < len; i += blockDim.x) orow[i] = ksub(a[i], sum);
}

// STs <-> TS row copies around the cross-sectional kernels: rows
// [row0, row0 + length) of an [S/L][T_in][L] buffer to a [length][S] one, and
// back to an [S/L][length][L] buffer.
template <typename T>
__global__ void sts_rows_to_ts(const T *__restrict__ in, T *__restrict__ out, long long S, long long T_in,
                               long long row0, long long length, int L) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= length * S) return;
    const long long t = i / S, s = i % S;
    out[i] = in[(s / L) * T_in * L + (row0 + t) * L + s % L];
}
template <typename T>
__global__ void ts_rows_to_sts(const T *__restrict__ in, T *__restrict__ out, long long S, long long length, int L) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= length * S) return;
    const long long t = i / S, s = i % S;
    out[(s / L) * length * L + t * L + s % L] = in[i];
}
template <typename T>
inline int launch_sts_to_ts(const T *in, T *out, long long S, long long T_in, long long row0, long long length, int L,
                            cudaStream_t st) {
    const long long n = length * S;
    sts_rows_to_ts<T><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(in, out, S, T_in, row0, length, L);
    return (int)cudaGetLastError();
}
template <typename T>
inline int launch_ts_to_sts(const T *in, T *out, long long S, long long length, int L, cudaStream_t st) {
    const long long n = length * S;
    ts_rows_to_sts<T><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(in, out, S, length, L);
    return (int)cudaGetLastError();
}

inline int kun_num_sms() {
    static int n = 0;
    if (!n) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 132;
    }
    return n;
}

template <typename T, int ITEMS>
inline int launch_rank_items(const T *in, T *out, long long S, long long length, int P, cudaStream_t st) {
    size_t smem = rank_smem_bytes<T>(P);
    if (smem > kSmemOptIn) {
        cudaError_t e =
            cudaFuncSetAttribute(rank_rows<T, ITEMS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return (int)e;
    }
    long long grid = length < (long long)kun_num_sms() * 2 ? length : (long long)kun_num_sms() * 2;
    rank_rows<T, ITEMS><<<(unsigned)grid, kRankThreads, smem, st>>>(in, out, S, length, P);
    return (int)cudaGetLastError();
}

// Batch runs of several universes: the rows of one Rank stage of every job
// in one launch.  Job j ranks rows [row0, row0 + length) of the launch's
// row space, reading `in` and writing `out` ([length][S], TS).
struct RankRowsJob {
    const void *in;
    void *out;
    long long S, length, row0;
};

template <typename T, int ITEMS>
__global__ void __launch_bounds__(kRankThreads) rank_rows_multi(const RankRowsJob *__restrict__ jobs, int njobs,
                                                                long long total_rows, int P) {
    using K = typename SortKey<T>::K;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int cnt_warp[kRankThreads / 32];
    K *keys = reinterpret_cast<K *>(smem_raw);
    uint32_t *counters = reinterpret_cast<uint32_t *>(smem_raw + ((size_t)rank_key_slots(P) * sizeof(K) + 15) / 16 * 16);
    uint16_t *idx = reinterpret_cast<uint16_t *>(counters + radix_hist_slots());
    for (long long r = blockIdx.x; r < total_rows; r += gridDim.x) {
        int lo = 0, hi = njobs - 1;  // the job whose rows hold r
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (jobs[mid].row0 <= r) lo = mid;
            else hi = mid - 1;
        }
        const RankRowsJob jb = jobs[lo];
        const long long t = r - jb.row0, S = jb.S;
        if (t < 0 || t >= jb.length || S <= 0 || S > P) continue;
        const T *in = (const T *)jb.in + t * S;
        T *out = (T *)jb.out + t * S;
        int Pk = ITEMS;
        while (Pk < S) Pk <<= 1;
        if (Pk >= kRadixMinP) {
            if (!rank_one_row_bucket<T, ITEMS>(in, out, S, keys, counters))
                rank_one_row_radix<T, ITEMS>(in, out, S, keys, counters, idx, cnt_warp);
        } else {
            rank_one_row<T, ITEMS>(in, out, S, Pk, keys, cnt_warp);
        }
    }
}

// max_S: the longest row of the jobs (sizes the keys per thread and the
// shared memory)
template <typename T>
inline int launch_rank_rows_multi(const RankRowsJob *d_jobs, int njobs, long long total_rows, long long max_S,
                                  cudaStream_t st) {
    if (njobs <= 0 || total_rows <= 0) return 0;
    int P = 8;
    while (P < max_S) P <<= 1;
    const size_t smem = rank_smem_bytes<T>(P);
    if (smem > 227 * 1024 || P > 32 * kRankThreads) return (int)cudaErrorInvalidValue;
    const long long grid = total_rows < (long long)kun_num_sms() * 2 ? total_rows : (long long)kun_num_sms() * 2;
    auto go = [&](auto kernel) {
        if (smem > kSmemOptIn) {
            cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) return (int)e;
        }
        kernel<<<(unsigned)grid, kRankThreads, smem, st>>>(d_jobs, njobs, total_rows, P);
        return (int)cudaGetLastError();
    };
    switch (rank_items(P)) {
    case 8: return go(rank_rows_multi<T, 8>);
    case 16: return go(rank_rows_multi<T, 16>);
    default: return go(rank_rows_multi<T, 32>);
    }
}

template <typename T>
inline int launch_rank(const T *in, T *out, long long S, long long length, cudaStream_t st) {
    int P = 8;
    while (P < S) P <<= 1;
    if (rank_smem_bytes<T>(P) > 227 * 1024 || P > 32 * kRankThreads) return (int)cudaErrorInvalidValue;
    switch (rank_items(P)) {
    case 8: return launch_rank_items<T, 8>(in, out, S, length, P, st);
    case 16: return launch_rank_items<T, 16>(in, out, S, length, P, st);
    default: return launch_rank_items<T, 32>(in, out, S, length, P, st);
    }
}

template <typename T>
inline int launch_scale(const T *in, T *out, long long S, long long length, cudaStream_t st) {
    size_t smem = (size_t)S * sizeof(T);
    if (smem > 200 * 1024) return (int)cudaErrorInvalidValue;
    if (smem > kSmemOptIn) {
        cudaError_t e = cudaFuncSetAttribute(scale_rows<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return (int)e;
    }
    long long grid = length < (long long)kun_num_sms() * 4 ? length : (long long)kun_num_sms() * 4;
    scale_rows<T><<<(unsigned)grid, 256, smem, st>>>(in, out, S, length);
    return (int)cudaGetLastError();
}

template <typename T>
inline int launch_diffwsum(const T *in0, const T *in1, T *out, long long S, long long length, cudaStream_t st) {
    long long grid = length < (long long)kun_num_sms() * 4 ? length : (long long)kun_num_sms() * 4;
    diffwsum_rows<T><<<(unsigned)grid, 256, 0, st>>>(in0, in1, out, S, length);
    return (int)cudaGetLastError();
}

template <typename T>
inline int launch_rank_segments(const T *in, int w_in, T *out, int w_out, long long cap, const int32_t *seg_off,
                                const int32_t *seg_stock0, const long long *seg_tick, int nseg, int max_len,
                                const int32_t *cnt, cudaStream_t st) {
    int P = 8;
    while (P < max_len) P <<= 1;
    size_t smem = rank_smem_bytes<T>(P);
    if (smem > 227 * 1024 || P > 32 * kRankThreads) return (int)cudaErrorInvalidValue;
    auto go = [&](auto kernel) {
        if (smem > kSmemOptIn) {
            cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) return (int)e;
        }
        kernel<<<(unsigned)nseg, kRankThreads, smem, st>>>(in, w_in, out, w_out, cap, seg_off, seg_stock0, seg_tick,
                                                           P, cnt);
        return (int)cudaGetLastError();
    };
    switch (rank_items(P)) {
    case 8: return go(rank_segments<T, 8>);
    case 16: return go(rank_segments<T, 16>);
    default: return go(rank_segments<T, 32>);
    }
}

// njobs Rank stages over the step's segments: one launch for the segments
// of at most kRankSmallMax stocks and one for the longer ones.  With a
// device table (cnt: nseg, stocks, longest, number of small segments) both
// launch and each takes its part; without one every segment goes to the
// launch that max_len picks.
template <typename T>
inline int launch_rank_multi_segments(const RankJob *d_jobs, int njobs, long long cap, const int32_t *seg_off,
                                      const int32_t *seg_stock0, const long long *seg_tick, int nseg, int max_len,
                                      const int32_t *cnt, cudaStream_t st, cudaStream_t st_long = nullptr) {
    if (njobs <= 0 || nseg <= 0) return 0;
    if (njobs > 65535) return (int)cudaErrorInvalidValue;
    const dim3 grid((unsigned)nseg, (unsigned)njobs);
    if (cnt || max_len <= kRankSmallMax) {
        const size_t smem = rank_smem_bytes<T>(kRankSmallMax);
        rank_multi_segments<T, 8, true><<<grid, kRankSmallThreads, smem, st>>>(d_jobs, cap, seg_off, seg_stock0,
                                                                            seg_tick, kRankSmallMax, cnt);
        if (cudaError_t e = cudaGetLastError()) return (int)e;
    }
    if (!cnt && max_len <= kRankSmallMax) return 0;
    if (st_long) st = st_long;
    int P = 8;
    while (P < max_len) P <<= 1;
    size_t smem = rank_smem_bytes<T>(P);
    if (smem > 227 * 1024 || P > 32 * kRankThreads) return (int)cudaErrorInvalidValue;
    auto go = [&](auto kernel) {
        if (smem > kSmemOptIn) {
            cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) return (int)e;
        }
        kernel<<<grid, kRankThreads, smem, st>>>(d_jobs, cap, seg_off, seg_stock0, seg_tick, P, cnt);
        return (int)cudaGetLastError();
    };
    switch (rank_items(P)) {
    case 8: return go(rank_multi_segments<T, 8, false>);
    case 16: return go(rank_multi_segments<T, 16, false>);
    default: return go(rank_multi_segments<T, 32, false>);
    }
}

template <typename T>
inline int launch_scale_segments(const T *in, int w_in, T *out, int w_out, long long cap, const int32_t *seg_off,
                                 const int32_t *seg_stock0, const long long *seg_tick, int nseg, int max_len,
                                 const int32_t *cnt, cudaStream_t st) {
    size_t smem = (size_t)max_len * sizeof(T);
    if (smem > 200 * 1024) return (int)cudaErrorInvalidValue;
    if (smem > kSmemOptIn) {
        cudaError_t e = cudaFuncSetAttribute(scale_segments<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return (int)e;
    }
    scale_segments<T><<<(unsigned)nseg, 256, smem, st>>>(in, w_in, out, w_out, cap, seg_off, seg_stock0, seg_tick,
                                                         cnt, max_len);
    return (int)cudaGetLastError();
}

template <typename T>
inline int launch_diffwsum_segments(const T *in0, int w0, const T *in1, int w1, T *out, int w_out, long long cap,
                                    const int32_t *seg_off, const int32_t *seg_stock0, const long long *seg_tick,
                                    int nseg, int max_len, const int32_t *cnt, cudaStream_t st) {
    (void)max_len;
    diffwsum_segments<T><<<(unsigned)nseg, 256, 0, st>>>(in0, w0, in1, w1, out, w_out, cap, seg_off, seg_stock0,
                                                         seg_tick, cnt);
    return (int)cudaGetLastError();
}

}  // namespace kun
