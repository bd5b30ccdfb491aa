// sg_stream.cuh -- the adjoint pass over an axis k >= 1 as a warp-specialized stream:
// one producer warp moves whole row segments into a shared-memory ring with bulk
// copies (cp.async.bulk) and stages each stage's basis rows beside them; eight
// consumer warps sum them.
//
// The pass reads its input X[M, ns, Q] (for the first adjoint pass: the cotangent on
// eval, the largest array of the adjoint) exactly once and spends d+1 FMAs per value,
// so it is bound by how many bytes are in flight and by per-row bookkeeping.  Here
//   * a tile is a column q, a chunk of control points [c0, c1) and up to W = 256*NV
//     consecutive m (all of M when M <= W): each of the 256 consumer threads owns the
//     NV values m_lo + t + 256*v, so a row of 1024 Float32 values costs each thread 4
//     shared loads and the row's bookkeeping once; two rows are loaded ahead of their
//     sums for latency tolerance;
//   * the producer (one lane) copies R rows per stage, NS stages ahead.  When the
//     tile spans whole rows of a sorted axis, the R rows are consecutive in memory and
//     move as ONE copy; otherwise each row is one copy of its 16-byte-aligned
//     superset.  Stages complete on `full` mbarriers (transaction bytes); consumer
//     warps release them on `empty` mbarriers -- no CTA-wide barrier on the data path;
//   * the d+1 rolling accumulators and the summation order are those of the other
//     adjoint kernels (sg_contract.cuh): each control point sums its samples in
//     increasing view order, deterministic and without atomics.
// A copy never extends past the last 16-byte boundary of the column's slab
// X[:, :, q]; the at most 3 values beyond it are read with plain loads.
#pragma once

#include "sg_contract.cuh"
#include "sg_mbar.cuh"

namespace sg {

constexpr int kStreamConsumers = 8;                          // consumer warps
constexpr int kStreamLanes = 32 * kStreamConsumers;          // consumer threads
constexpr int kStreamThreads = 32 * (kStreamConsumers + 1);  // + the producer warp
constexpr int kStreamStages = 2;
constexpr int kStreamStageBytes = 25600;  // one stage buffer: 6 rows of 1024 Float32 + slack
constexpr int kStreamMaxRows = 32;        // rows per stage at most (one producer lane each)

template <typename T>
__host__ __device__ constexpr int stream_nv() { return sizeof(T) == 4 ? 4 : 2; }
template <typename T>
__host__ __device__ constexpr int stream_width() { return kStreamLanes * stream_nv<T>(); }

// Bytes a row of L values may occupy in a stage buffer (aligned superset + slack).
__host__ __device__ constexpr int64_t stream_row_cap(int64_t L, int es) {
    return (L * es + 15) / 16 * 16 + 16;
}

// Rows per stage for tile rows of L values: as many as fit a stage buffer, at most
// kStreamMaxRows.
inline int stream_rows_per_stage(int64_t L, int es) {
    const int64_t fit = kStreamStageBytes / stream_row_cap(L, es);
    return (int)(fit < 1 ? 1 : (fit > kStreamMaxRows ? kStreamMaxRows : fit));
}

// Per stage slot, written by the producer warp with the slot's rows: the rows' basis
// values as 8-byte elements [kStreamMaxRows][DP], their support starts and sample
// indices [kStreamMaxRows] each.
template <int D, typename T>
__host__ __device__ constexpr int64_t stream_header_bytes() {
    return (int64_t)kStreamMaxRows * (DegreeTraits<D>::DP * 8 + 8);
}

template <int D, typename T>
__host__ __device__ constexpr int64_t stream_smem_bytes() {
    return 16 * kStreamStages                                 /* full + empty barriers */
           + 32                                                /* abort flag, stage flags */
           + 2 * kStreamStages * kStreamMaxRows * 4            /* row offsets, counts */
           + 16                                                /* run-start masks */
           + kStreamStages * stream_header_bytes<D, T>()       /* basis headers */
           + (int64_t)kStreamStages * kStreamStageBytes;
}

// Arithmetic elements of the stream consumers: Float32 values travel in pairs (float2;
// one fma.rn.f32x2 per pair, each half rounded as an FFMA), Float64 values singly.
// Basis values are staged in shared memory already in element form -- a Float32 value
// duplicated into both halves of a pair -- so every FMA operand is a ready register
// pair and no instruction repacks it.
template <typename T>
struct StreamElem;
template <>
struct StreamElem<float> {
    using A = float2;
    static constexpr int W = 2;  // values per element
    static __device__ __forceinline__ A zero() { return make_float2(0.f, 0.f); }
    static __device__ __forceinline__ A dup(float b) { return make_float2(b, b); }
    static __device__ __forceinline__ A fma(A b, A x, A c) { return __ffma2_rn(b, x, c); }
    static __device__ __forceinline__ float get(A a, int w) { return w ? a.y : a.x; }
    static __device__ __forceinline__ A make(const float (&v)[2]) { return make_float2(v[0], v[1]); }
};
template <>
struct StreamElem<double> {
    using A = double;
    static constexpr int W = 1;
    static __device__ __forceinline__ A zero() { return 0.0; }
    static __device__ __forceinline__ A dup(double b) { return b; }
    static __device__ __forceinline__ A fma(A b, A x, A c) { return ::fma(b, x, c); }
    static __device__ __forceinline__ double get(A a, int) { return a; }
    static __device__ __forceinline__ A make(const double (&v)[1]) { return v[0]; }
};

// The DA basis elements of one staged row (DP entries of 8 bytes: two 16-byte loads).
template <typename T, int DA, int DP>
__device__ __forceinline__ void basis_elems(const typename StreamElem<T>::A *row,
                                           typename StreamElem<T>::A (&bv)[DA]) {
#pragma unroll
    for (int i = 0; i < DA; ++i) bv[i] = row[i];
}

// Rotating accumulator window (DA <= 4): with phase P the accumulator of control point
// cur + i is acc[(P + i) % DA].  Each phase is its own unrolled instance, so the window
// rotates by changing the phase instead of moving DA*NA registers.
template <int P, int DA, int NA, typename T>
__device__ __forceinline__ void rot_fma(typename StreamElem<T>::A (&acc)[DA][NA],
                                        const typename StreamElem<T>::A (&bv)[DA],
                                        const typename StreamElem<T>::A (&x)[NA]) {
#pragma unroll
    for (int i = 0; i < DA; ++i)
#pragma unroll
        for (int h = 0; h < NA; ++h)
            acc[(P + i) % DA][h] = StreamElem<T>::fma(bv[i], x[h], acc[(P + i) % DA][h]);
}

// store (when keep) the accumulator of phase P -- the completed control point -- with
// lane stride kStreamLanes (value v = h*W + w of element h), and clear it for control
// point cur + DA
template <int P, int DA, int NA, typename T>
__device__ __forceinline__ void rot_flush(typename StreamElem<T>::A (&acc)[DA][NA], T *dst,
                                          bool keep, int nvt) {
    using E = StreamElem<T>;
    if (keep) {
#pragma unroll
        for (int h = 0; h < NA; ++h)
#pragma unroll
            for (int w = 0; w < E::W; ++w)
                if (h * E::W + w < nvt) dst[kStreamLanes * (h * E::W + w)] = E::get(acc[P][h], w);
    }
#pragma unroll
    for (int h = 0; h < NA; ++h) acc[P][h] = E::zero();
}

// the thread's values of one row: element h holds values h*W .. h*W+W-1 at
// row[kStreamLanes * v] (v < nvt; 0 past it)
template <int NA, typename T>
__device__ __forceinline__ void load_elems(const T *row, int nvt, typename StreamElem<T>::A (&x)[NA]) {
    using E = StreamElem<T>;
#pragma unroll
    for (int h = 0; h < NA; ++h) {
        T v[E::W];
#pragma unroll
        for (int w = 0; w < E::W; ++w)
            v[w] = (h * E::W + w < nvt) ? row[kStreamLanes * (h * E::W + w)] : T(0);
        x[h] = E::make(v);
    }
}

// Rows [r, e) of a stage whose values all lie in the shared buffer, at fixed phase P:
// row k's values for this thread are base[off[k] + kStreamLanes*v] (v < nvt), its basis
// row sB[k*DP ..].  Two rows are loaded ahead of their FMAs.
template <int P, int DA, int DP, int NA, typename T>
__device__ __forceinline__ void run_rows(typename StreamElem<T>::A (&acc)[DA][NA], const T *base,
                                         const int32_t *off, const typename StreamElem<T>::A *sB,
                                         int r, int e, int nvt) {
    using A = typename StreamElem<T>::A;
    for (; r + 1 < e; r += 2) {
        A xa[NA], xb[NA], ba[DA], bb[DA];
        load_elems<NA, T>(base + off[r], nvt, xa);
        load_elems<NA, T>(base + off[r + 1], nvt, xb);
        basis_elems<T, DA, DP>(sB + r * DP, ba);
        basis_elems<T, DA, DP>(sB + (r + 1) * DP, bb);
        rot_fma<P, DA, NA, T>(acc, ba, xa);
        rot_fma<P, DA, NA, T>(acc, bb, xb);
    }
    if (r < e) {
        A xa[NA], ba[DA];
        load_elems<NA, T>(base + off[r], nvt, xa);
        basis_elems<T, DA, DP>(sB + r * DP, ba);
        rot_fma<P, DA, NA, T>(acc, ba, xa);
    }
}

// ---------------------------------------------------------------------------------
// One tile: Y[m, c, q] = sum_{j : b(j) <= c <= b(j)+d} B[j, c - b(j)] X[m, j, q]
// for m in [m_lo, m_lo + L), c in [c0, c1).  R = rows per stage (stream_rows_per_stage
// of L).  X must be 16-byte aligned.  Launched with kStreamThreads threads; on a
// timeout *status is set to SG_ERR_TIMEOUT and the tile's results are invalid.
// Ends with a CTA barrier after which the shared memory may be reused.
// ---------------------------------------------------------------------------------
template <int D, typename T>
__device__ __forceinline__ void
adj_stream_tile(int64_t m_lo, int64_t L, int64_t chunk, int64_t q, int R, unsigned char *smem,
                const int32_t *__restrict__ idx, const int32_t *__restrict__ perm,
                const int32_t *__restrict__ lb, const T *__restrict__ B, int64_t ns, int d,
                const T *__restrict__ X, int64_t M, int64_t n, int CC, T *__restrict__ Y,
                int *status) {
    using DT = DegreeTraits<D>;
    static_assert(D >= 1 && D <= 4, "stream tiles take degrees 0..3");
    static_assert(kStreamStages <= 4, "stage flags hold 4 stages");
    constexpr int DA = DT::DA;
    constexpr int DP = DT::DP;
    constexpr int NV = stream_nv<T>();
    constexpr int NS = kStreamStages;
    constexpr int ES = (int)sizeof(T);
    constexpr int STAGE_ELEMS = kStreamStageBytes / ES;
    using E = StreamElem<T>;
    using A = typename E::A;
    const int dd = DT::deg(d);
    uint64_t *full = reinterpret_cast<uint64_t *>(smem);
    uint64_t *empty = full + NS;
    volatile int *s_abort = reinterpret_cast<volatile int *>(smem + 16 * NS);
    int32_t *s_whole = reinterpret_cast<int32_t *>(smem + 16 * NS + 16);  // [NS]: every row complete
    int32_t *s_off = reinterpret_cast<int32_t *>(smem + 16 * NS + 32);  // [NS][kStreamMaxRows]
    int32_t *s_cnt = s_off + NS * kStreamMaxRows;
    uint32_t *s_run = reinterpret_cast<uint32_t *>(s_cnt + NS * kStreamMaxRows);  // [NS] (16 B)
    A *s_B = reinterpret_cast<A *>(s_run + 4);                          // [NS][kStreamMaxRows][DP]
    int32_t *s_bs = reinterpret_cast<int32_t *>(s_B + NS * kStreamMaxRows * DP);  // [NS][kStreamMaxRows]
    int32_t *s_js = s_bs + NS * kStreamMaxRows;                         // [NS][kStreamMaxRows]
    T *ring = reinterpret_cast<T *>(s_js + NS * kStreamMaxRows);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int c0 = (int)(chunk * CC);
    const int c1 = (c0 + CC < n) ? c0 + CC : (int)n;  // exclusive
    const int64_t s_lo = support_lb(lb, idx, perm, ns, dd, n, c0 - dd);
    const int64_t nrows = support_lb(lb, idx, perm, ns, dd, n, c1) - s_lo;
    const int64_t nst = (nrows + R - 1) / R;
    if (threadIdx.x == 0) {
        for (int s = 0; s < NS; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], kStreamConsumers);
        }
        *s_abort = 0;
        mbar_init_fence();
    }
    __syncthreads();

    if (warp == kStreamConsumers) {
        // ------------------------------------------------------------- producer
        // Lane r stages row r of each stage's basis header (fetched one stage ahead);
        // lane 0 waits for free slots and issues the copies.  The header and the row
        // table are published by lane 0's arrive on full[slot] after a warp barrier.
        if (lane == 0) fence_proxy_async_global();
        const bool whole = perm == nullptr && m_lo == 0 && L == M;
        const uintptr_t lim = (uintptr_t)(X + M * ns * (q + 1)) & ~(uintptr_t)15;
        const int64_t rowcap = stream_row_cap(L, ES) / ES;  // elements
        int32_t pj = 0, pbs = 0;
        T pB[DP];
#pragma unroll
        for (int i = 0; i < DP; ++i) pB[i] = T(0);
        auto fetch = [&](int64_t g) {  // row `lane` of stage g into registers
            const int64_t rr = g * R + lane;
            if (lane < R && rr < nrows) {
                const int64_t j = view_sample(perm, s_lo + rr);
                pj = (int32_t)j;
                pbs = (int32_t)support_start(idx[j], dd, n);
#pragma unroll
                for (int i = 0; i < DP; ++i) pB[i] = (i <= dd) ? B[j + ns * i] : T(0);
            }
        };
        fetch(0);
        int64_t g = 0;
        for (; g < nst; ++g) {
            const int slot = (int)(g % NS);
            int ok = 1;
            if (lane == 0 && g >= NS) ok = mbar_wait(&empty[slot], (unsigned)((g / NS - 1) & 1), s_abort);
            ok = __shfl_sync(0xffffffffu, ok, 0);
            if (!ok) {
                if (lane == 0) {
                    if (status) atomicExch(status, SG_ERR_TIMEOUT);
                    *s_abort = 1;
                }
                break;
            }
            // (the consumers' reads of the slot happened before their arrivals on
            // empty[slot], which this wait acquired: neither the header writes nor the
            // copies can overtake them)
            const int64_t r0 = g * R;
            const int nr = (int)((nrows - r0) < R ? (nrows - r0) : R);
            if (lane < nr) {
                const int h = slot * kStreamMaxRows + lane;
                s_bs[h] = pbs;
                s_js[h] = pj;
#pragma unroll
                for (int i = 0; i < DP; ++i) s_B[h * DP + i] = E::dup(pB[i]);
            }
            // bit r: row r starts a run (its support start differs from row r-1's)
            const int prev = __shfl_up_sync(0xffffffffu, pbs, 1);
            const unsigned runs = __ballot_sync(0xffffffffu, lane > 0 && lane < nr && pbs != prev);
            fetch(g + 1);
            __syncwarp();
            if (lane == 0) {
                s_run[slot] = runs;
                T *dst = ring + (int64_t)slot * STAGE_ELEMS;
                int32_t *off = s_off + slot * kStreamMaxRows;
                int32_t *cnt = s_cnt + slot * kStreamMaxRows;
                if (whole) {
                    const uintptr_t a = (uintptr_t)(X + M * (s_lo + r0 + ns * q));
                    const uintptr_t a0 = a & ~(uintptr_t)15;
                    uintptr_t e = (a + (uintptr_t)nr * M * ES + 15) & ~(uintptr_t)15;
                    if (e > lim) e = lim;
                    const int64_t got = e > a0 ? (int64_t)(e - a0) / ES : 0;
                    const int64_t lead = (int64_t)(a - a0) / ES;
                    int complete = 1;
                    for (int r = 0; r < nr; ++r) {
                        const int64_t o = lead + r * M;
                        off[r] = (int32_t)o;
                        const int64_t c = got - o;
                        cnt[r] = (int32_t)(c < 0 ? 0 : (c > L ? L : c));
                        complete &= (c >= L);
                    }
                    s_whole[slot] = complete;
                    mbar_arrive_expect_tx(&full[slot], (unsigned)(got * ES));
                    if (got > 0) bulk_g2s(dst, (const void *)a0, (unsigned)(got * ES), &full[slot]);
                } else {
                    unsigned total = 0;
                    int complete = 1;
                    for (int r = 0; r < nr; ++r) {
                        const int64_t j = s_js[slot * kStreamMaxRows + r];
                        const uintptr_t a = (uintptr_t)(X + m_lo + M * (j + ns * q));
                        const uintptr_t a0 = a & ~(uintptr_t)15;
                        uintptr_t e = (a + (uintptr_t)L * ES + 15) & ~(uintptr_t)15;
                        if (e > lim) e = lim;
                        const int64_t got = e > a0 ? (int64_t)(e - a0) / ES : 0;
                        const int64_t lead = (int64_t)(a - a0) / ES;
                        off[r] = (int32_t)(r * rowcap + lead);
                        const int64_t c = got - lead;
                        cnt[r] = (int32_t)(c < 0 ? 0 : (c > L ? L : c));
                        complete &= (c >= L);
                        total += (unsigned)(got * ES);
                    }
                    s_whole[slot] = complete;
                    mbar_arrive_expect_tx(&full[slot], total);
                    for (int r = 0; r < nr; ++r) {
                        const int64_t j = s_js[slot * kStreamMaxRows + r];
                        const uintptr_t a = (uintptr_t)(X + m_lo + M * (j + ns * q));
                        const uintptr_t a0 = a & ~(uintptr_t)15;
                        uintptr_t e = (a + (uintptr_t)L * ES + 15) & ~(uintptr_t)15;
                        if (e > lim) e = lim;
                        if (e > a0) bulk_g2s(dst + r * rowcap, (const void *)a0, (unsigned)(e - a0), &full[slot]);
                    }
                }
            }
        }
        // after an abort, let the copies already issued land before the shared
        // memory is reused (the last NS issued stages may be outstanding)
        if (lane == 0 && *s_abort)
            for (int64_t h = (g > NS ? g - NS : 0); h < g; ++h)
                (void)mbar_wait(&full[h % NS], (unsigned)((h / NS) & 1), nullptr);
    } else {
        // ------------------------------------------------------------- consumers
        const int t = threadIdx.x;  // 0 .. kStreamLanes - 1
        const int64_t nvl = (L - t + kStreamLanes - 1) / kStreamLanes;
        const int nvt = (L > t) ? (int)(nvl < NV ? nvl : NV) : 0;
        constexpr int NA = NV / E::W;  // arithmetic elements per thread and row
        // Rolling window of DA accumulators that rotates instead of moving: the
        // accumulator of control point cur + i is acc[(p + i) % DA].
        A acc[DA][NA];
#pragma unroll
        for (int i = 0; i < DA; ++i)
#pragma unroll
            for (int h = 0; h < NA; ++h) acc[i][h] = E::zero();
        int cur = c0 - dd;
        int p = 0;
        T *yq = Y + m_lo + t + M * n * q;
        auto shift = [&]() {  // control point `cur` is complete: store and clear its slot
            T *dst = yq + M * cur;
            const bool keep = cur >= c0;
            switch (p) {
                case 0: rot_flush<0, DA, NA, T>(acc, dst, keep, nvt); break;
                case 1: rot_flush<1 % DA, DA, NA, T>(acc, dst, keep, nvt); break;
                case 2: rot_flush<2 % DA, DA, NA, T>(acc, dst, keep, nvt); break;
                default: rot_flush<3 % DA, DA, NA, T>(acc, dst, keep, nvt); break;
            }
            p = (p + 1 == DA) ? 0 : p + 1;
            ++cur;
        };
        for (int64_t g = 0; g < nst; ++g) {
            const int slot = (int)(g % NS);
            const int64_t r0 = g * R;
            const int nr = (int)((nrows - r0) < R ? (nrows - r0) : R);
            if (!mbar_wait(&full[slot], (unsigned)((g / NS) & 1), s_abort)) {
                if (status) atomicExch(status, SG_ERR_TIMEOUT);
                *s_abort = 1;
                break;
            }
            const T *buf = ring + (int64_t)slot * STAGE_ELEMS;
            const int32_t *bs = s_bs + slot * kStreamMaxRows;
            const A *sB = s_B + slot * kStreamMaxRows * DP;
            if (s_whole[slot]) {
                // Runs of rows with the same support start (from the producer's run
                // mask): the window shifts and the phase is chosen once per run; the
                // rows of a run are straight-line shared loads and packed FMAs.
                const T *base = buf + t;
                const unsigned runs = s_run[slot];
                int r = 0;
                while (r < nr) {
                    const int b = bs[r];
                    while (cur < b) shift();
                    const unsigned rest = runs & ~((2u << r) - 1u);  // run starts after r
                    const int e = rest ? __ffs(rest) - 1 : nr;
                    switch (p) {
                        case 0: run_rows<0, DA, DP, NA, T>(acc, base, s_off + slot * kStreamMaxRows, sB, r, e, nvt); break;
                        case 1: run_rows<1 % DA, DA, DP, NA, T>(acc, base, s_off + slot * kStreamMaxRows, sB, r, e, nvt); break;
                        case 2: run_rows<2 % DA, DA, DP, NA, T>(acc, base, s_off + slot * kStreamMaxRows, sB, r, e, nvt); break;
                        default: run_rows<3 % DA, DA, DP, NA, T>(acc, base, s_off + slot * kStreamMaxRows, sB, r, e, nvt); break;
                    }
                    r = e;
                }
            } else {
                // a stage reaching past the copied part (the column's last values): rows
                // one at a time, lanes past the copy read global memory
                const int32_t *js = s_js + slot * kStreamMaxRows;
                for (int r = 0; r < nr; ++r) {
                    const int b = bs[r];
                    while (cur < b) shift();
                    const T *row = buf + s_off[slot * kStreamMaxRows + r] + t;
                    const int cnt = s_cnt[slot * kStreamMaxRows + r];
                    const T *gx = X + m_lo + t + M * (js[r] + ns * q);
                    A x[NA];
#pragma unroll
                    for (int h = 0; h < NA; ++h) {
                        T v2[E::W];
#pragma unroll
                        for (int w = 0; w < E::W; ++w) {
                            const int v = h * E::W + w;
                            v2[w] = (v < nvt) ? (t + kStreamLanes * v < cnt ? row[kStreamLanes * v]
                                                                             : gx[kStreamLanes * v])
                                              : T(0);
                        }
                        x[h] = E::make(v2);
                    }
                    A bv[DA];
                    basis_elems<T, DA, DP>(sB + r * DP, bv);
                    switch (p) {
                        case 0: rot_fma<0, DA, NA, T>(acc, bv, x); break;
                        case 1: rot_fma<1 % DA, DA, NA, T>(acc, bv, x); break;
                        case 2: rot_fma<2 % DA, DA, NA, T>(acc, bv, x); break;
                        default: rot_fma<3 % DA, DA, NA, T>(acc, bv, x); break;
                    }
                }
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(&empty[slot]);
        }
        if (!*s_abort)
            while (cur < c1) shift();
    }
    __syncthreads();
    if (threadIdx.x == 0)
        for (int s = 0; s < NS; ++s) {
            mbar_inval(&full[s]);
            mbar_inval(&empty[s]);
        }
}

// Per-grid kernel: block -> tile (m block fastest, then the chunk, then q).
template <int D, typename T>
__global__ void __launch_bounds__(kStreamThreads, 3)
k_adj_stream(const int32_t *__restrict__ idx, const int32_t *__restrict__ perm,
             const int32_t *__restrict__ lb, const T *__restrict__ B, int64_t ns, int d,
             const T *__restrict__ X, int64_t M, int64_t n, int64_t Q, int CC, int64_t nmb,
             int64_t chunks, int R, T *__restrict__ Y, int *status) {
    extern __shared__ __align__(16) unsigned char s_dyn[];
    const int64_t tile = blockIdx.x;
    const int64_t mb = tile % nmb, r = tile / nmb;
    constexpr int64_t W = stream_width<T>();
    const int64_t m_lo = mb * W;
    const int64_t L = (M - m_lo) < W ? (M - m_lo) : W;
    adj_stream_tile<D, T>(m_lo, L, r % chunks, r / chunks, R, s_dyn, idx, perm, lb, B, ns, d, X, M,
                          n, CC, Y, status);
}

}  // namespace sg
