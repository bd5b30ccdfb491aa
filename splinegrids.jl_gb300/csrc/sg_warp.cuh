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

template <typename T>
__host__ __device__ constexpr int warp_width() { return 32 * (16 / (int)sizeof(T)); }

// Shared memory of one warp (bytes, 16-byte multiple).
template <int D, typename T>
__host__ __device__ constexpr int warp_adj_smem() {
    return 2 * (int)align16(kWarpRows * DegreeTraits<D>::DP * (int64_t)sizeof(T)) + 2 * 2 * kWarpRows * 4;
}
template <int D, typename T>
__host__ __device__ constexpr int warp_fwd_smem() {
    return (int)align16(kWarpRows * DegreeTraits<D>::DP * (int64_t)sizeof(T)) + kWarpRows * 4;
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
// Task = (mw, jchunk, q) with jchunk = samples [j0, j0 + 32).  The warp keeps the d+1
// input rows of the current support in registers (a window) plus the row after it,
// loaded ahead: when the support start advances by one (sorted samples), the window
// shifts and only the row after the new window is fetched; any other change reloads
// the window.  FINAL passes write eval with streaming stores.
// ---------------------------------------------------------------------------------
template <int D, typename T, bool ST, bool FINAL>
__device__ __forceinline__ void
fwd_axis_warp(int64_t mw, int64_t jchunk, int64_t q, int lane, unsigned char *wsmem,
              const int32_t *__restrict__ idx, const T *__restrict__ B, int64_t ns, int d,
              const T *__restrict__ X, int64_t M, int64_t n, T *__restrict__ Y) {
    using DT = DegreeTraits<D>;
    constexpr int DA = DT::DA;
    constexpr int DP = DT::DP;
    constexpr int VEC = 16 / (int)sizeof(T);
    const int dd = DT::deg(d);
    T *s_B = reinterpret_cast<T *>(wsmem);  // [kWarpRows][DP]
    int32_t *s_b = reinterpret_cast<int32_t *>(wsmem + align16(kWarpRows * DP * (int64_t)sizeof(T)));

    const int64_t j0 = jchunk * kWarpRows;
    const int jn = (int)((ns - j0) < kWarpRows ? (ns - j0) : kWarpRows);
    __syncwarp();
    if (lane < jn) {
        const int64_t j = j0 + lane;
        s_b[lane] = (int32_t)support_start(idx[j], dd, n);
#pragma unroll
        for (int i = 0; i < DP; ++i) s_B[lane * DP + i] = (i <= dd) ? B[j + ns * i] : T(0);
    }
    __syncwarp();
    const WarpLanes<ST, VEC> ln(mw, lane, M);
    if (ln.nv == 0) return;
    const T *xq = X + ln.m0 + M * n * q;
    T *yq = Y + ln.m0 + M * (j0 + ns * q);
    Pack<T, VEC> win[DA], nxt;
    int bprev = -2;
    for (int t = 0; t < jn; ++t) {
        const int b = s_b[t];
        if (b != bprev) {
            if (b == bprev + 1) {  // shift by one: the prefetched row joins the window
#pragma unroll
                for (int i = 0; i + 1 < DA; ++i) win[i] = win[i + 1];
                win[dd < DA - 1 ? dd : DA - 1] = nxt;
            } else {
#pragma unroll
                for (int i = 0; i < DA; ++i)
                    if (i <= dd) win[i] = ldw<ST, T, VEC>(xq + M * (b + i), ln.nv);
            }
            if (b + dd + 1 < n) nxt = ldw<ST, T, VEC>(xq + M * (b + dd + 1), ln.nv);
            bprev = b;
        }
        Pack<T, VEC> acc;
#pragma unroll
        for (int v = 0; v < VEC; ++v) acc.v[v] = T(0);
        T bv[DA];
        basis_row<T, DA, DP>(s_B + t * DP, bv);
#pragma unroll
        for (int i = 0; i < DA; ++i)
            if (i <= dd)
#pragma unroll
                for (int v = 0; v < VEC; ++v) acc.v[v] += bv[i] * win[i].v[v];
        stw<FINAL, ST, T, VEC>(yq + M * t, acc, ln.nv);
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

template <int D, typename T, bool ST, bool FINAL>
__global__ void __launch_bounds__(32 * kWarpsPerBlock)
k_fwd_warp(const int32_t *__restrict__ idx, const T *__restrict__ B, int64_t ns, int d,
           const T *__restrict__ X, int64_t M, int64_t n, int64_t Q, int64_t gxw,
           T *__restrict__ Y) {
    __shared__ __align__(16) unsigned char smem[kWarpsPerBlock * warp_fwd_smem<D, T>()];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t task = (int64_t)blockIdx.x * kWarpsPerBlock + w;
    const int64_t jchunks = (ns + kWarpRows - 1) / kWarpRows;
    if (task >= gxw * jchunks * Q) return;
    const int64_t mw = task % gxw, r = task / gxw;
    fwd_axis_warp<D, T, ST, FINAL>(mw, r % jchunks, r / jchunks, lane, smem + w * warp_fwd_smem<D, T>(),
                                   idx, B, ns, d, X, M, n, Y);
}

}  // namespace sg
