// sg_warp.cuh -- the separable passes over an axis k >= 1 as independent warp tasks.
//
// A pass over axis k views its input as X[M, nk, Q] (M = product of the sample
// counts of the axes before k, Q = product of the extents after it, channels last)
// and walks axis k for every (m, q).  Here the unit of work is one warp:
//   32*VEC consecutive m  x  a run of axis-k rows  x  one column q.
// Warps never wait for each other (no CTA barrier on the data path), and an awkward
// M (an odd sample count, a row of 537 values) wastes at most one partly filled warp
// per row instead of a partly filled CTA.
//
// Lane layouts along m (VEC values per lane):
//   contiguous (ST = false): lane l holds m = mw*W + l*VEC + v and moves them as one
//     16-byte access; needs M % VEC == 0 and 16-byte aligned X and Y.
//   strided (ST = true): lane l holds m = mw*W + l + 32*v (v < VEC), moved as VEC
//     4/8-byte accesses that are coalesced across the warp; any M, any alignment.
// W = 32*VEC values (128 for Float32, 64 for Float64).
//
// The basis rows a warp needs are staged by the warp itself (one row per lane) in a
// private slice of shared memory; __syncwarp orders them.
#pragma once

#include "sg_contract.cuh"

namespace sg {

constexpr int kWarpRows = 32;     // rows staged per batch (one per lane)
constexpr int kAdjGroup = 4;      // adjoint: rows loaded ahead per group (two groups in flight)
constexpr int kFwdTaskRows = 128;  // forward: samples per warp task at most (batched tasks)
constexpr int kFwdGridRows = 32;  // forward: samples per warp task of the per-grid kernel

template <typename T>
__host__ __device__ constexpr int warp_width() { return 32 * (16 / (int)sizeof(T)); }

// Shared memory of one warp (bytes, 16-byte multiple).
template <int D, typename T>
__host__ __device__ constexpr int warp_adj_smem() {
    return 2 * (int)align16(kWarpRows * DegreeTraits<D>::DP * (int64_t)sizeof(T)) + 2 * 2 * kWarpRows * 4;
}
template <int D, typename T>
__host__ __device__ constexpr int warp_fwd_smem() {
    return (int)align16(kFwdTaskRows * DegreeTraits<D>::DP * (int64_t)sizeof(T)) + kFwdTaskRows * 4;
}

// m-lanes of one warp task
template <bool ST, int VEC>
struct WarpLanes {
    int64_t m0;  // first m of the lane
    int nv;      // valid values of the lane (0..VEC)
    __device__ __forceinline__ WarpLanes(int64_t mw, int lane, int64_t M) {
        const int64_t base = mw * 32 * VEC;
        m0 = ST ? base + lane : base + (int64_t)lane * VEC;
        if (m0 >= M) {
            nv = 0;
        } else if constexpr (!ST) {
            nv = VEC;
        } else {
            const int64_t r = (M - m0 + 31) / 32;
            nv = r < VEC ? (int)r : VEC;
        }
    }
};

template <bool ST, typename T, int VEC>
__device__ __forceinline__ Pack<T, VEC> ldw(const T *p, int nv) {
    if constexpr (!ST) {
        return ldp<T, VEC>(p);
    } else {
        Pack<T, VEC> r;
#pragma unroll
        for (int v = 0; v < VEC; ++v) r.v[v] = (v < nv) ? p[32 * v] : T(0);
        return r;
    }
}

template <bool STREAM, bool ST, typename T, int VEC>
__device__ __forceinline__ void stw(T *p, const Pack<T, VEC> &a, int nv) {
    if constexpr (!ST) {
        if constexpr (STREAM) stp_stream<T, VEC>(p, a);
        else stp<T, VEC>(p, a);
    } else {
#pragma unroll
        for (int v = 0; v < VEC; ++v)
            if (v < nv) {
                if constexpr (STREAM) __stcs(p + 32 * v, a.v[v]);
                else p[32 * v] = a.v[v];
            }
    }
}

// ---------------------------------------------------------------------------------
// Adjoint pass over axis k >= 1 (gather form, the map of adj_axis_tile):
//   Y[m, c, q] = sum_{j : b(j) <= c <= b(j)+d} B[j, c - b(j)] X[m, j, q].
// Task = (mw, chunk, q) with chunk = control points [c0, c0+CC): the warp walks the
// contiguous range of the sorted sample view whose supports meet the chunk, with d+1
// rolling accumulators per value (accumulator i belongs to control point cur+i).
// When the support start passes cur, control point cur is complete and is stored
// (also when no sample touched it: 0, as the reference's zeroed output).  Each control
// point sums its samples in increasing view order -- the order of the per-grid and
// batched kernels alike, so both give identical bits -- with no atomics.
// Rows are loaded kAdjGroup at a time, one group ahead of the group being summed;
// basis rows are staged 32 at a time, one batch ahead.
// ---------------------------------------------------------------------------------
template <int D, typename T, bool ST>
__device__ __forceinline__ void
adj_axis_warp(int64_t mw, int64_t chunk, int64_t q, int lane, unsigned char *wsmem,
              const int32_t *__restrict__ idx, const int32_t *__restrict__ perm,
              const int32_t *__restrict__ lb, const T *__restrict__ B, int64_t ns, int d,
              const T *__restrict__ X, int64_t M, int64_t n, int CC, T *__restrict__ Y) {
    using DT = DegreeTraits<D>;
    constexpr int DA = DT::DA;
    constexpr int DP = DT::DP;
    constexpr int VEC = 16 / (int)sizeof(T);
    constexpr int U = kAdjGroup;
    static_assert(kWarpRows % (2 * U) == 0, "a batch holds whole group pairs");
    const int dd = DT::deg(d);
    T *s_B = reinterpret_cast<T *>(wsmem);  // [2][kWarpRows][DP]
    int32_t *s_j = reinterpret_cast<int32_t *>(wsmem + 2 * align16(kWarpRows * DP * (int64_t)sizeof(T)));
    int32_t *s_b = s_j + 2 * kWarpRows;     // [2][kWarpRows]

    const int c0 = (int)(chunk * CC);
    const int c1 = (c0 + CC < n) ? c0 + CC : (int)n;  // exclusive
    const int64_t s_lo = support_lb(lb, idx, perm, ns, dd, n, c0 - dd);
    const int64_t nrows = support_lb(lb, idx, perm, ns, dd, n, c1) - s_lo;
    const WarpLanes<ST, VEC> ln(mw, lane, M);
    const T *xq = X + ln.m0 + M * ns * q;
    T *yq = Y + ln.m0 + M * n * q;

    auto stage = [&](int64_t bi) {  // basis batch bi -> slot bi & 1
        const int64_t r = bi * kWarpRows + lane;
        if (r < nrows) {
            const int slot = (int)(bi & 1);
            const int64_t j = view_sample(perm, s_lo + r);
            s_j[slot * kWarpRows + lane] = (int32_t)j;
            s_b[slot * kWarpRows + lane] = (int32_t)support_start(idx[j], dd, n);
#pragma unroll
            for (int i = 0; i < DP; ++i)
                s_B[(slot * kWarpRows + lane) * DP + i] = (i <= dd) ? B[j + ns * i] : T(0);
        }
    };
    auto load = [&](Pack<T, VEC> (&x)[U], int64_t r0) {  // rows r0 .. r0+U-1
        const int base = (int)((r0 / kWarpRows) & 1) * kWarpRows + (int)(r0 % kWarpRows);
#pragma unroll
        for (int u = 0; u < U; ++u)
            if (ln.nv > 0 && r0 + u < nrows) x[u] = ldw<ST, T, VEC>(xq + M * s_j[base + u], ln.nv);
    };

    Pack<T, VEC> acc[DA];
#pragma unroll
    for (int i = 0; i < DA; ++i)
#pragma unroll
        for (int v = 0; v < VEC; ++v) acc[i].v[v] = T(0);
    int cur = c0 - dd;  // control point of acc[0]
    auto shift = [&]() {  // control point `cur` is complete
        if (cur >= c0 && ln.nv > 0) stw<false, ST, T, VEC>(yq + M * cur, acc[0], ln.nv);
#pragma unroll
        for (int i = 0; i + 1 < DA; ++i) acc[i] = acc[i + 1];
#pragma unroll
        for (int v = 0; v < VEC; ++v) acc[DA - 1].v[v] = T(0);
        ++cur;
    };
    auto sum = [&](const Pack<T, VEC> (&x)[U], int64_t r0) {
        const int base = (int)((r0 / kWarpRows) & 1) * kWarpRows + (int)(r0 % kWarpRows);
#pragma unroll
        for (int u = 0; u < U; ++u) {
            if (r0 + u < nrows) {
                const int b = s_b[base + u];
                while (cur < b) shift();
                T bv[DA];
                basis_row<T, DA, DP>(s_B + (base + u) * DP, bv);
#pragma unroll
                for (int i = 0; i < DA; ++i)
                    if (i <= dd)
#pragma unroll
                        for (int v = 0; v < VEC; ++v) acc[i].v[v] += bv[i] * x[u].v[v];
            }
        }
    };
    // at the first group of batch bi (bi >= 1) batch bi-1 is summed: stage bi+1
    auto next_batch = [&](int64_t r0) {
        if (r0 > 0 && r0 % kWarpRows == 0) {
            __syncwarp();
            stage(r0 / kWarpRows + 1);
            __syncwarp();
        }
    };

    if (nrows > 0) {
        stage(0);
        stage(1);
        __syncwarp();
        Pack<T, VEC> xa[U], xb[U];
        load(xa, 0);
        for (int64_t r0 = 0; r0 < nrows; r0 += 2 * U) {
            next_batch(r0);
            if (r0 + U < nrows) load(xb, r0 + U);
            sum(xa, r0);
            if (r0 + U >= nrows) break;
            if (r0 + 2 * U < nrows) load(xa, r0 + 2 * U);
            sum(xb, r0 + U);
        }
    }
    while (cur < c1) shift();
}

// ---------------------------------------------------------------------------------
// Forward pass over axis k >= 1 (kPlain):  Y[m, j, q] = sum_i B[j, i] X[m, b(j)+i, q].
// Task = (mw, jchunk, q) with jchunk = samples [j0, j0 + rows), rows <= kFwdTaskRows.  The warp keeps
// the d+1 input rows of the current knot span in a rotating register window (phase p:
// win[(p + i) % DA] holds row b + i) plus the row after it, fetched one run ahead; a
// run of samples with one support start is evaluated with packed FMAs and no window
// checks, and the window rotates by one row per advance of the support start (sorted
// samples) or reloads on any other change.  FINAL passes write eval with streaming
// stores.
// ---------------------------------------------------------------------------------
template <int P, int DA, int VEC, typename T>
__device__ __forceinline__ Pack<T, VEC> rot_dot_pack(const Pack<T, VEC> (&win)[DA], const T (&bv)[DA]) {
    Pack<T, VEC> y;
    if constexpr (sizeof(T) == 4 && VEC % 2 == 0) {
#pragma unroll
        for (int h = 0; h < VEC / 2; ++h) {
            float2 a = make_float2(0.f, 0.f);
#pragma unroll
            for (int i = 0; i < DA; ++i)
                a = __ffma2_rn(make_float2(bv[i], bv[i]),
                               make_float2(win[(P + i) % DA].v[2 * h], win[(P + i) % DA].v[2 * h + 1]), a);
            y.v[2 * h] = a.x;
            y.v[2 * h + 1] = a.y;
        }
    } else {
#pragma unroll
        for (int v = 0; v < VEC; ++v) {
            T a = T(0);
#pragma unroll
            for (int i = 0; i < DA; ++i) a += bv[i] * win[(P + i) % DA].v[v];
            y.v[v] = a;
        }
    }
    return y;
}

template <int D, typename T, bool ST, bool FINAL>
__device__ __forceinline__ void
fwd_axis_warp(int64_t mw, int64_t jchunk, int rows, int64_t q, int lane, unsigned char *wsmem,
              const int32_t *__restrict__ idx, const T *__restrict__ B, int64_t ns, int d,
              const T *__restrict__ X, int64_t M, int64_t n, T *__restrict__ Y) {
    using DT = DegreeTraits<D>;
    static_assert(D >= 1 && D <= 4, "warp tasks take degrees 0..3");
    constexpr int DA = DT::DA;
    constexpr int DP = DT::DP;
    constexpr int VEC = 16 / (int)sizeof(T);
    const int dd = DT::deg(d);
    T *s_B = reinterpret_cast<T *>(wsmem);  // [kFwdTaskRows][DP]
    int32_t *s_b = reinterpret_cast<int32_t *>(wsmem + align16(kFwdTaskRows * DP * (int64_t)sizeof(T)));

    const int64_t j0 = jchunk * rows;
    const int jn = (int)((ns - j0) < rows ? (ns - j0) : rows);
    __syncwarp();
    for (int r = lane; r < jn; r += 32) {
        const int64_t j = j0 + r;
        s_b[r] = (int32_t)support_start(idx[j], dd, n);
#pragma unroll
        for (int i = 0; i < DP; ++i) s_B[r * DP + i] = (i <= dd) ? B[j + ns * i] : T(0);
    }
    __syncwarp();
    const WarpLanes<ST, VEC> ln(mw, lane, M);
    if (ln.nv == 0) return;
    const T *xq = X + ln.m0 + M * n * q;
    T *yq = Y + ln.m0 + M * (j0 + ns * q);
    Pack<T, VEC> win[DA], nxt;
    int p = 0, bprev = -2;
    int t = 0;
    while (t < jn) {
        const int b = s_b[t];
        int e = t + 1;
        while (e < jn && s_b[e] == b) ++e;
        if (b == bprev + 1) {  // rotate: the prefetched row after the window joins it
            switch (p) {
                case 0: win[0] = nxt; break;
                case 1: win[1 % DA] = nxt; break;
                case 2: win[2 % DA] = nxt; break;
                default: win[3 % DA] = nxt; break;
            }
            p = (p + 1 == DA) ? 0 : p + 1;
        } else if (b != bprev) {
#pragma unroll
            for (int i = 0; i < DA; ++i) win[i] = ldw<ST, T, VEC>(xq + M * (b + i), ln.nv);
            p = 0;
        }
        bprev = b;
        if (b + dd + 1 < n) nxt = ldw<ST, T, VEC>(xq + M * (b + dd + 1), ln.nv);
        switch (p) {
#define SG_FWD_RUN(P)                                                          \
    for (; t < e; ++t) {                                                       \
        T bv[DA];                                                              \
        basis_row<T, DA, DP>(s_B + t * DP, bv);                                \
        stw<FINAL, ST, T, VEC>(yq + M * t, rot_dot_pack<(P) % DA>(win, bv), ln.nv); \
    }                                                                          \
    break;
            case 0: SG_FWD_RUN(0)
            case 1: SG_FWD_RUN(1)
            case 2: SG_FWD_RUN(2)
            default: SG_FWD_RUN(3)
#undef SG_FWD_RUN
        }
    }
}

// ---------------------------------------------------------------------------------
// Adjoint pass over axis 0 (M = 1) as warp tasks:
//   Y[c, q] = sum_{j : b(j) <= c <= b(j)+d} B[j, c - b(j)] X[j, q],  X [ns, Q], Y [n, Q].
// Task = 32 consecutive columns q0 + lane and the control points [c_lo, c_hi), walked
// over the samples of their supports in view order with the rolling accumulator window
// of the other adjoint kernels (one column per lane;
// every lane meets the same support starts, so the window moves in lockstep and each
// control point sums its samples in increasing view order).  Batches of 16 samples x
// 32 columns arrive by cp.async (coalesced along the samples) in a double-buffered
// per-warp transpose tile, one batch ahead of the batch being summed, so no register
// holds data in flight.  Runs of samples with one support start are summed without
// per-sample window checks; completed control points are stored as they leave the
// window.
// ---------------------------------------------------------------------------------
constexpr int kAdj0Batch16 = 16;  // samples per staged batch

template <int D, typename T>
__host__ __device__ constexpr int warp_adj0_smem() {
    return (int)(2 * align16(32 * (kAdj0Batch16 + 1) * (int64_t)sizeof(T)) +
                 2 * align16(kAdj0Batch16 * DegreeTraits<D>::DP * (int64_t)sizeof(T)) + 2 * kAdj0Batch16 * 4);
}

template <int P, int DA, typename T>
__device__ __forceinline__ void rot_fma1(T (&acc)[DA], const T (&bv)[DA], T x) {
#pragma unroll
    for (int i = 0; i < DA; ++i) acc[(P + i) % DA] += bv[i] * x;
}

template <int D, typename T>
__device__ __forceinline__ void
adj0_warp(int64_t q0, int64_t c_lo, int64_t c_hi, int lane, unsigned char *wsmem,
          const int32_t *__restrict__ idx, const int32_t *__restrict__ perm,
          const int32_t *__restrict__ lb, const T *__restrict__ B, int64_t ns, int d,
          const T *__restrict__ X, int64_t n, int64_t Q, T *__restrict__ Y) {
    using DT = DegreeTraits<D>;
    static_assert(D >= 1 && D <= 4, "warp tasks take degrees 0..3");
    constexpr int DA = DT::DA;
    constexpr int DP = DT::DP;
    constexpr int SB = kAdj0Batch16;
    constexpr int XS = 32 * (SB + 1);                     // one transpose tile
    constexpr int64_t XB = align16(XS * (int64_t)sizeof(T));
    constexpr int64_t BB = align16(SB * DP * (int64_t)sizeof(T));
    const int dd = DT::deg(d);
    T *s_x = reinterpret_cast<T *>(wsmem);                          // [2][32 columns][SB + 1]
    T *s_B = reinterpret_cast<T *>(wsmem + 2 * XB);                 // [2][SB][DP]
    int32_t *s_i = reinterpret_cast<int32_t *>(wsmem + 2 * XB + 2 * BB);  // [2][SB] raw indices
    const bool col_ok = q0 + lane < Q;
    // basis padding entries (DA..DP-1) stay zero
    if (DA < DP && lane < SB)
#pragma unroll
        for (int b = 0; b < 2; ++b)
#pragma unroll
            for (int i = DA; i < DP; ++i) s_B[(b * SB + lane) * DP + i] = T(0);
    // stage samples [sb, sb + SB) into buffer `buf`: lane l copies sample l % SB for the
    // columns 16*(l / SB) .. +15, and lanes < SB its basis row and index
    // the samples whose supports meet [c_lo, c_hi): support starts c_lo - d .. c_hi - 1
    const int64_t s_begin = support_lb(lb, idx, perm, ns, dd, n, c_lo - dd);
    const int64_t s_end = support_lb(lb, idx, perm, ns, dd, n, c_hi);
    auto stage = [&](int buf, int64_t sb) {
        const int nb = (int)((s_end - sb) < SB ? (s_end - sb) : SB);
        const int r = lane % SB;
        if (r < nb) {
            const int64_t j = view_sample(perm, sb + r);
            if (lane < SB) {
                cp_async<4>(s_i + buf * SB + r, idx + j);
#pragma unroll
                for (int i = 0; i < DA; ++i) cp_async<sizeof(T)>(s_B + (buf * SB + r) * DP + i, B + j + ns * i);
            }
            const int kb = (lane / SB) * 16;
            const T *xj = X + j + ns * (q0 + kb);
            T *dst = s_x + buf * XS + kb * (SB + 1) + r;
#pragma unroll
            for (int k = 0; k < 16; ++k)
                if (q0 + kb + k < Q) cp_async<sizeof(T)>(dst + k * (SB + 1), xj + ns * k);
        }
        cp_async_commit();
    };
    T acc[DA];
#pragma unroll
    for (int i = 0; i < DA; ++i) acc[i] = T(0);
    int64_t cur = c_lo - dd;  // control point of acc[p]
    int p = 0;
    T *yc = Y + n * (q0 + lane);
    auto flush = [&]() {  // control point `cur` is complete
        T v;
        switch (p) {
            case 0: v = acc[0]; acc[0] = T(0); break;
            case 1: v = acc[1 % DA]; acc[1 % DA] = T(0); break;
            case 2: v = acc[2 % DA]; acc[2 % DA] = T(0); break;
            default: v = acc[3 % DA]; acc[3 % DA] = T(0); break;
        }
        if (cur >= c_lo && col_ok) yc[cur] = v;
        p = (p + 1 == DA) ? 0 : p + 1;
        ++cur;
    };
    if (s_end > s_begin) stage(0, s_begin);
    int buf = 0;
    for (int64_t sb = s_begin; sb < s_end; sb += SB, buf ^= 1) {
        const int nb = (int)((s_end - sb) < SB ? (s_end - sb) : SB);
        if (sb + SB < s_end) {
            stage(buf ^ 1, sb + SB);
            cp_async_wait<1>();  // this batch's copies have landed (the next may fly)
        } else {
            cp_async_wait<0>();
        }
        __syncwarp();
        const T *xs = s_x + buf * XS + lane * (SB + 1);
        const T *sB = s_B + buf * SB * DP;
        const int32_t *si = s_i + buf * SB;
        int t = 0;
        while (t < nb) {
            const int b = (int)support_start(si[t], dd, n);
            while (cur < b) flush();
            int e = t + 1;
            while (e < nb && si[e] == si[t]) ++e;
            switch (p) {
#define SG_ADJ0_RUN(P)                                                   \
    for (; t < e; ++t) {                                                 \
        T bv[DA];                                                        \
        basis_row<T, DA, DP>(sB + t * DP, bv);                           \
        rot_fma1<(P) % DA>(acc, bv, col_ok ? xs[t] : T(0));              \
    }                                                                    \
    break;
                case 0: SG_ADJ0_RUN(0)
                case 1: SG_ADJ0_RUN(1)
                case 2: SG_ADJ0_RUN(2)
                default: SG_ADJ0_RUN(3)
#undef SG_ADJ0_RUN
            }
        }
        __syncwarp();  // the buffer is refilled two batches later
    }
    while (cur < c_hi) flush();
}

// ---------------------------------------------------------------------------------
// Forward pass over axis 0 (M = 1, kPlain) as warp tasks:
//   Y[j, q] = sum_i B[j, i] X[b(j) + i, q],  X [n, Q], Y [ns, Q].
// Task = 32 consecutive columns q0 + lane over samples [s_begin, s_end).  Each lane keeps the d+1
// inputs of its column's current knot span in a rotating register window; consecutive
// support starts (sorted samples) rotate it and fetch one input, any other change
// reloads it.  Results leave through a per-warp transpose tile (32 samples x 32
// columns), so the stores are coalesced along the samples.
// ---------------------------------------------------------------------------------
template <int D, typename T>
__host__ __device__ constexpr int warp_fwd0_smem() {
    return (int)(align16(32 * 33 * (int64_t)sizeof(T)) + align16(32 * DegreeTraits<D>::DP * (int64_t)sizeof(T)) + 32 * 4);
}

template <int P, int DA, typename T>
__device__ __forceinline__ T rot_dot(const T (&win)[DA], const T (&bv)[DA]) {
    T a = T(0);
#pragma unroll
    for (int i = 0; i < DA; ++i) a += bv[i] * win[(P + i) % DA];
    return a;
}

template <int D, typename T>
__device__ __forceinline__ void
fwd0_warp(int64_t q0, int64_t s_begin, int64_t s_end, int lane, unsigned char *wsmem,
          const int32_t *__restrict__ idx, const T *__restrict__ B, int64_t ns, int d,
          const T *__restrict__ X, int64_t n, int64_t Q, T *__restrict__ Y) {
    using DT = DegreeTraits<D>;
    static_assert(D >= 1 && D <= 4, "warp tasks take degrees 0..3");
    constexpr int DA = DT::DA;
    constexpr int DP = DT::DP;
    const int dd = DT::deg(d);
    T *s_t = reinterpret_cast<T *>(wsmem);  // [32 samples][33]
    T *s_B = reinterpret_cast<T *>(wsmem + align16(32 * 33 * (int64_t)sizeof(T)));
    int32_t *s_b = reinterpret_cast<int32_t *>(reinterpret_cast<unsigned char *>(s_B) +
                                               align16(32 * DP * (int64_t)sizeof(T)));
    const bool col_ok = q0 + lane < Q;
    const T *xc = X + n * (q0 + lane);  // this lane's column
    T win[DA];
#pragma unroll
    for (int i = 0; i < DA; ++i) win[i] = T(0);
    int p = 0;        // win[(p + i) % DA] holds X[bprev + i]
    int bprev = -2;
    T nxt = T(0);     // X[bprev + d + 1], fetched ahead of the next rotation
    // the next batch's support start and basis row (one sample per lane), fetched while
    // the current batch is evaluated
    T nB[DP];
    int32_t nidx = 0;
    auto fetch = [&](int64_t sb) {
        if (sb + lane < s_end) {
            nidx = idx[sb + lane];
#pragma unroll
            for (int i = 0; i < DP; ++i) nB[i] = (i <= dd) ? B[sb + lane + ns * i] : T(0);
        }
    };
    if (s_begin < s_end) fetch(s_begin);
    for (int64_t sb = s_begin; sb < s_end; sb += 32) {
        const int nb = (int)((s_end - sb) < 32 ? (s_end - sb) : 32);
        __syncwarp();
        if (lane < nb) {
            s_b[lane] = (int32_t)support_start(nidx, dd, n);
#pragma unroll
            for (int i = 0; i < DP; ++i) s_B[lane * DP + i] = nB[i];
        }
        __syncwarp();
        if (sb + 32 < s_end) fetch(sb + 32);
        for (int t = 0; t < nb; ++t) {
            const int b = s_b[t];
            if (b != bprev) {
                if (b == bprev + 1) {  // the window's oldest input leaves, X[b + d] enters
                    switch (p) {
                        case 0: win[0] = nxt; break;
                        case 1: win[1 % DA] = nxt; break;
                        case 2: win[2 % DA] = nxt; break;
                        default: win[3 % DA] = nxt; break;
                    }
                    p = (p + 1 == DA) ? 0 : p + 1;
                } else {
#pragma unroll
                    for (int i = 0; i < DA; ++i) win[i] = (col_ok && i <= dd) ? xc[b + i] : T(0);
                    p = 0;
                }
                bprev = b;
                nxt = (col_ok && b + dd + 1 < n) ? xc[b + dd + 1] : T(0);
            }
            T bv[DA];
            basis_row<T, DA, DP>(s_B + t * DP, bv);
            T y;
            switch (p) {
                case 0: y = rot_dot<0>(win, bv); break;
                case 1: y = rot_dot<1 % DA>(win, bv); break;
                case 2: y = rot_dot<2 % DA>(win, bv); break;
                default: y = rot_dot<3 % DA>(win, bv); break;
            }
            s_t[t * 33 + lane] = y;
        }
        __syncwarp();
        // samples [sb, sb + nb) of the 32 columns, coalesced along the samples
        T *yo = Y + sb + lane;
#pragma unroll 4
        for (int k = 0; k < 32; ++k)
            if (lane < nb && q0 + k < Q) yo[ns * (q0 + k)] = s_t[lane * 33 + k];
    }
}

// ---------------------------------------------------------------------------------
// Per-grid kernels: warp w of block x runs task x*4 + w; tasks are numbered m-fastest
// (mw, then the chunk, then q), so the 4 warps of a block usually read 4 adjacent
// segments of the same rows.
// ---------------------------------------------------------------------------------
constexpr int kWarpsPerBlock = 4;

template <int D, typename T, bool ST>
__global__ void __launch_bounds__(32 * kWarpsPerBlock)
k_adj_warp(const int32_t *__restrict__ idx, const int32_t *__restrict__ perm,
           const int32_t *__restrict__ lb, const T *__restrict__ B, int64_t ns, int d,
           const T *__restrict__ X, int64_t M, int64_t n, int64_t Q, int CC, int64_t gxw,
           int64_t chunks, T *__restrict__ Y) {
    __shared__ __align__(16) unsigned char smem[kWarpsPerBlock * warp_adj_smem<D, T>()];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t task = (int64_t)blockIdx.x * kWarpsPerBlock + w;
    if (task >= gxw * chunks * Q) return;
    const int64_t mw = task % gxw, r = task / gxw;
    adj_axis_warp<D, T, ST>(mw, r % chunks, r / chunks, lane, smem + w * warp_adj_smem<D, T>(), idx,
                            perm, lb, B, ns, d, X, M, n, CC, Y);
}

// task = column group (fastest) x chunk of CC control points
template <int D, typename T>
__global__ void __launch_bounds__(32 * kWarpsPerBlock)
k_adj0_warp(const int32_t *__restrict__ idx, const int32_t *__restrict__ perm,
            const int32_t *__restrict__ lb, const T *__restrict__ B, int64_t ns, int d,
            const T *__restrict__ X, int64_t n, int64_t Q, int64_t CC, T *__restrict__ Y) {
    extern __shared__ __align__(16) unsigned char s_dyn[];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t task = (int64_t)blockIdx.x * kWarpsPerBlock + w;
    const int64_t groups = (Q + 31) / 32, chunks = (n + CC - 1) / CC;
    if (task >= groups * chunks) return;
    const int64_t cg = task % groups, c_lo = (task / groups) * CC;
    const int64_t c_hi = c_lo + CC < n ? c_lo + CC : n;
    adj0_warp<D, T>(cg * 32, c_lo, c_hi, lane, s_dyn + w * warp_adj0_smem<D, T>(), idx, perm, lb,
                    B, ns, d, X, n, Q, Y);
}

// task = column group (fastest) x chunk of SC samples
template <int D, typename T>
__global__ void __launch_bounds__(32 * kWarpsPerBlock)
k_fwd0_warp(const int32_t *__restrict__ idx, const T *__restrict__ B, int64_t ns, int d,
            const T *__restrict__ X, int64_t n, int64_t Q, int64_t SC, T *__restrict__ Y) {
    __shared__ __align__(16) unsigned char smem[kWarpsPerBlock * warp_fwd0_smem<D, T>()];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t task = (int64_t)blockIdx.x * kWarpsPerBlock + w;
    const int64_t groups = (Q + 31) / 32, chunks = (ns + SC - 1) / SC;
    if (task >= groups * chunks) return;
    const int64_t cg = task % groups, s0 = (task / groups) * SC;
    const int64_t s1 = s0 + SC < ns ? s0 + SC : ns;
    fwd0_warp<D, T>(cg * 32, s0, s1, lane, smem + w * warp_fwd0_smem<D, T>(), idx, B, ns, d, X, n, Q, Y);
}

template <int D, typename T, bool ST, bool FINAL>
__global__ void __launch_bounds__(32 * kWarpsPerBlock)
k_fwd_warp(const int32_t *__restrict__ idx, const T *__restrict__ B, int64_t ns, int d,
           const T *__restrict__ X, int64_t M, int64_t n, int64_t Q, int64_t gxw,
           T *__restrict__ Y) {
    __shared__ __align__(16) unsigned char smem[kWarpsPerBlock * warp_fwd_smem<D, T>()];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t task = (int64_t)blockIdx.x * kWarpsPerBlock + w;
    const int64_t jchunks = (ns + kFwdGridRows - 1) / kFwdGridRows;
    if (task >= gxw * jchunks * Q) return;
    const int64_t mw = task % gxw, r = task / gxw;
    fwd_axis_warp<D, T, ST, FINAL>(mw, r % jchunks, kFwdGridRows, r / jchunks, lane, smem + w * warp_fwd_smem<D, T>(),
                                   idx, B, ns, d, X, M, n, Y);
}

}  // namespace sg
