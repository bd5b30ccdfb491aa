// sg_contract.cuh -- the separable tensor-product contraction of evaluate! and
// evaluate_adjoint!, one input axis per pass.
//
// The reference's spline_eval_kernel (src/spline_grid.jl:119-183) forms, for every
// sample, the full (d+1)^Nin basis product and accumulates into eval in place.  The
// same linear map is the Kronecker product of the per-dimension banded basis
// matrices B_k (n_samples_k x n_basis_k, row j nonzero on columns b_k(j)..b_k(j)+d_k),
//     eval = (B_1 (x) ... (x) B_Nin) P,
// so it is applied here one axis at a time.  A pass over axis k reads a tensor viewed
// as [M, N_in, Q] (M = product of the axes before k, Q = product of the axes after k,
// column-major) and writes [M, N_out, Q]:
//     forward   Y[m, j, q] = sum_i B_k[j, i] X[m, b_k(j) + i, q]
//     adjoint   Y[m, c, q] = sum_{j : b_k(j) <= c <= b_k(j)+d} B_k[j, c - b_k(j)] X[m, j, q]
// Per output value a pass costs d+1 multiply-adds instead of the reference's
// (d+1)^Nin * (Nin + Nout) work, and the last forward pass (the one that writes
// eval) and the first adjoint pass (the one that reads the cotangent) stream
// through HBM exactly once with coalesced vector accesses along m.
//
// Every pass is a tile function: it processes the tile (bx, by, bz) of a grid of
// tiles with extents (gy, gz), using the shared memory it is handed.  The per-grid
// kernels below call them with blockIdx; the batched persistent kernel (sg_batch.cu)
// calls them for the work items it dequeues.  CG = true makes loads of X bypass L1
// (ld.global.cg), for inputs written earlier in the same launch by other CTAs.
//
// Degree handling: template D = d+1 for D in 1..4; D = 0 is the generic kernel for
// any degree up to SG_MAX_DEGREE with register arrays of kDMax entries.
#pragma once

#include "sg_common.cuh"

namespace sg {

template <int D>
struct DegreeTraits {
    static constexpr int DA = D > 0 ? D : kDMax;  // register array extent
    // staged basis rows are padded to 4 entries for degrees <= 3, so one row is one
    // 16-byte (float) or two 16-byte (double) shared-memory loads
    static constexpr int DP = DA <= 4 ? 4 : DA;
    static __device__ __forceinline__ int deg(int runtime_d) { return D > 0 ? D - 1 : runtime_d; }
};

// The DA basis values of one staged row (padded to DP entries, 16-byte aligned).
template <typename T, int DA, int DP>
__device__ __forceinline__ void basis_row(const T *row, T (&bv)[DA]) {
    if constexpr (DP == 4 && sizeof(T) == 4) {
        const float4 r = *reinterpret_cast<const float4 *>(row);
        const float tmp[4] = {r.x, r.y, r.z, r.w};
#pragma unroll
        for (int i = 0; i < DA; ++i) bv[i] = (T)tmp[i];
    } else if constexpr (DP == 4 && sizeof(T) == 8) {
        const double2 a = *reinterpret_cast<const double2 *>(row);
        const double2 b = *reinterpret_cast<const double2 *>(row + 2);
        const double tmp[4] = {a.x, a.y, b.x, b.y};
#pragma unroll
        for (int i = 0; i < DA; ++i) bv[i] = (T)tmp[i];
    } else {
#pragma unroll
        for (int i = 0; i < DA; ++i) bv[i] = row[i];
    }
}

constexpr int kChunk = 32;        // forward: samples of axis k per tile
constexpr int kAdjBatch = 128;    // adjoint: samples whose basis rows are staged per batch
constexpr int kAdj0Batch = 128;   // axis-0 adjoint: samples staged per batch

// Rows of the adjoint's input in flight per thread (cp.async ring stages): about
// 256 bytes per thread whatever the vector width.
template <typename T, int VEC>
struct AdjRing {
    static constexpr int S = (256 / (VEC * (int)sizeof(T))) < 32 ? (256 / (VEC * (int)sizeof(T))) : 32;
};

// ---------------------------------------------------------------------------------
// Asynchronous global->shared copies (cp.async).  Each thread copies and later reads
// only its own slots, so cp.async.wait_group alone orders a copy before the read.
// ---------------------------------------------------------------------------------
template <int BYTES>
__device__ __forceinline__ void cp_async(void *smem_dst, const void *gmem_src) {
    const unsigned dst = (unsigned)__cvta_generic_to_shared(smem_dst);
    if constexpr (BYTES == 16)
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(dst), "l"(gmem_src) : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(dst), "l"(gmem_src), "n"(BYTES)
                     : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}
constexpr int kThreads = 128;     // threads of the per-grid forward/adjoint kernels
constexpr int kAdj0Threads = 256; // threads of the axis-0 adjoint tiles

// Homogeneous (rational) channel layout of NURBS grids: channel 0 carries the weight,
// channel o >= 1 carries w * P[..., o-1].  The last forward pass divides channels
// 1..nout by channel 0 (the `denom` of src/spline_grid.jl:160-182).
enum FwdMode : int { kPlain = 0, kHomog = 1, kRational = 2 };

// Block coordinates of one tile and the extents of its tile grid along y and z.
struct Tile {
    int64_t bx, by, bz;
    int64_t gy, gz;
};

__device__ __forceinline__ Tile grid_tile() {
    return Tile{(int64_t)blockIdx.x, (int64_t)blockIdx.y, (int64_t)blockIdx.z,
                (int64_t)gridDim.y, (int64_t)gridDim.z};
}

template <bool CG, typename T>
__device__ __forceinline__ T ldx(const T *p) {
    if constexpr (CG) return __ldcg(p);
    else return *p;
}

template <bool CG, typename T, int VEC>
__device__ __forceinline__ Pack<T, VEC> ldpx(const T *p) {
    if constexpr (!CG) {
        return ldp<T, VEC>(p);
    } else {
        Pack<T, VEC> r;
        if constexpr (VEC == 4 && sizeof(T) == 4) {
            const float4 t = __ldcg(reinterpret_cast<const float4 *>(p));
            r.v[0] = t.x; r.v[1] = t.y; r.v[2] = t.z; r.v[3] = t.w;
        } else if constexpr (VEC == 2 && sizeof(T) == 8) {
            const double2 t = __ldcg(reinterpret_cast<const double2 *>(p));
            r.v[0] = t.x; r.v[1] = t.y;
        } else {
#pragma unroll
            for (int i = 0; i < VEC; ++i) r.v[i] = __ldcg(p + i);
        }
        return r;
    }
}

// Carves 16-byte aligned arrays out of a shared-memory buffer.
struct SmemCarver {
    unsigned char *p;
    template <typename U>
    __device__ __forceinline__ U *take(int64_t count) {
        U *r = reinterpret_cast<U *>(p);
        p += ((count * (int64_t)sizeof(U) + 15) / 16) * 16;
        return r;
    }
};

__host__ __device__ constexpr int64_t align16(int64_t b) { return ((b + 15) / 16) * 16; }

// ---------------------------------------------------------------------------------
// The VEC values a thread owns along the contiguous axis m of a pass.
//   contiguous (ST = false): m0 .. m0+VEC-1, moved as one 16-byte access; needs
//     M % VEC == 0 and 16-byte aligned bases.
//   strided (ST = true): m0 + v*blockDim, v < VEC, moved as VEC 4/8-byte accesses that
//     are still coalesced across the warp; any M and any alignment.  Lanes past M are
//     masked.
// Either way each thread amortizes its per-row work (basis values, support start,
// loop and copy bookkeeping) over VEC values.
// ---------------------------------------------------------------------------------
template <bool ST, int VEC>
__device__ __forceinline__ int64_t m_first(int64_t bx) {
    return ST ? bx * blockDim.x * VEC + threadIdx.x : (bx * blockDim.x + threadIdx.x) * VEC;
}

template <bool ST>
__device__ __forceinline__ int64_t m_lane_stride() {
    return ST ? (int64_t)blockDim.x : 1;
}

template <bool ST, int VEC>
__device__ __forceinline__ int m_valid(int64_t m0, int64_t M) {
    if (m0 >= M) return 0;
    if constexpr (!ST) return VEC;
    const int64_t n = (M - m0 + blockDim.x - 1) / blockDim.x;
    return n < VEC ? (int)n : VEC;
}

template <bool CG, bool ST, typename T, int VEC>
__device__ __forceinline__ Pack<T, VEC> ldm(const T *p, int64_t ls, int nv) {
    if constexpr (!ST) {
        return ldpx<CG, T, VEC>(p);
    } else {
        Pack<T, VEC> r;
#pragma unroll
        for (int v = 0; v < VEC; ++v) r.v[v] = (v < nv) ? ldx<CG>(p + v * ls) : T(0);
        return r;
    }
}

template <bool STREAM, bool ST, typename T, int VEC>
__device__ __forceinline__ void stm(T *p, const Pack<T, VEC> &a, int64_t ls, int nv) {
    if constexpr (!ST) {
        if constexpr (STREAM) stp_stream<T, VEC>(p, a);
        else stp<T, VEC>(p, a);
    } else {
#pragma unroll
        for (int v = 0; v < VEC; ++v) {
            if (v < nv) {
                if constexpr (STREAM) __stcs(p + v * ls, a.v[v]);
                else p[v * ls] = a.v[v];
            }
        }
    }
}

// ---------------------------------------------------------------------------------
// Forward pass over axis 0 (M = 1): Y[j, q] = sum_i B[j, i] X[b(j) + i, q].
// One thread per sample j keeps its d+1 basis values in registers and walks the
// columns q = by, by + gy, ...; neighbouring threads read the same control-point
// rows, which stay in L1.
//   kPlain:    X is the control-point tensor [n, Q] (TX may be bfloat16).
//   kHomog:    X is [n, Qr, nch] with weights w [n, Qr]; Y is [ns, Qr, nch+1] in the
//              homogeneous layout above (NURBS grids with Nin >= 2).
//   kRational: Nin == 1 NURBS: Y[j, o] = sum B w P / sum B w, divided in Float64.
// ---------------------------------------------------------------------------------
template <int D, typename TX, typename T, int MODE>
__device__ __forceinline__ void
fwd_axis0_tile(const Tile &tl, const int32_t *__restrict__ idx, const T *__restrict__ B,
               int64_t ns, int d, const TX *__restrict__ X, const T *__restrict__ w, int64_t n,
               int64_t Qr, int nch, T *__restrict__ Y) {
    using DT = DegreeTraits<D>;
    constexpr int DA = DT::DA;
    const int dd = DT::deg(d);
    const int64_t j = tl.bx * blockDim.x + threadIdx.x;
    if (j >= ns) return;
    const int64_t b = support_start(idx[j], dd, n);
    T bw[DA];
#pragma unroll
    for (int i = 0; i < DA; ++i) bw[i] = (i <= dd) ? B[j + ns * i] : T(0);

    if constexpr (MODE == kRational) {
        if (tl.by != 0) return;
        T wb[DA];
        T den = T(0);
#pragma unroll
        for (int i = 0; i < DA; ++i) {
            wb[i] = (i <= dd) ? bw[i] * w[b + i] : T(0);
            den += wb[i];
        }
        for (int o = 0; o < nch; ++o) {
            const TX *xp = X + b + n * (int64_t)o;
            T num = T(0);
#pragma unroll
            for (int i = 0; i < DA; ++i)
                if (i <= dd) num += wb[i] * ld_as<T>(xp + i);
            __stcs(Y + j + ns * (int64_t)o, (T)((double)num / (double)den));
        }
        return;
    } else {
        const int64_t Qy = (MODE == kHomog) ? Qr * (int64_t)(nch + 1) : Qr * (int64_t)nch;
#pragma unroll 4
        for (int64_t q = tl.by; q < Qy; q += tl.gy) {
            T acc = T(0);
            if constexpr (MODE == kPlain) {
                const TX *xp = X + b + n * q;
#pragma unroll
                for (int i = 0; i < DA; ++i)
                    if (i <= dd) acc += bw[i] * ld_as<T>(xp + i);
            } else {  // kHomog
                const int64_t r = q % Qr;
                const int64_t o = q / Qr;  // 0: weight channel, o >= 1: w * P[..., o-1]
                const T *wp = w + b + n * r;
                if (o == 0) {
#pragma unroll
                    for (int i = 0; i < DA; ++i)
                        if (i <= dd) acc += bw[i] * wp[i];
                } else {
                    const TX *xp = X + b + n * (r + Qr * (o - 1));
#pragma unroll
                    for (int i = 0; i < DA; ++i)
                        if (i <= dd) acc += (bw[i] * wp[i]) * ld_as<T>(xp + i);
                }
            }
            Y[j + ns * q] = acc;
        }
    }
}

// ---------------------------------------------------------------------------------
// Forward pass over axis k >= 1: Y[m, j, q] = sum_i B[j, i] X[m, b(j) + i, q].
// Tile = blockDim*VEC consecutive m (coalesced VEC-wide accesses) x kChunk samples of
// axis k x the columns q = bz, bz + gz, ...  The chunk's basis rows and support starts
// are staged in shared memory; each thread keeps a register window of the d+1 input
// rows of the current knot span and reloads it only when the span changes (every
// n_samples/n_basis samples), so X is read ~once per span while each output costs d+1
// FMAs.  FINAL passes write eval with streaming stores.
//   kRational (NURBS, last axis): Q is the NC channel axis of the homogeneous layout;
//   the thread keeps NC windows and divides channels 1..nch by channel 0 in Float64.
// ns: sample count of the axis (stride of B and Y); jcount: samples addressed by this
// call, counted from the (possibly shifted) idx/B/Y bases.
// ---------------------------------------------------------------------------------
template <int D, typename T>
__host__ __device__ constexpr int64_t fwd_axis_smem_bytes() {
    return align16(kChunk * 8) + align16(kChunk * DegreeTraits<D>::DP * (int64_t)sizeof(T));
}

template <int D, typename T, int VEC, int MODE, int NC, bool FINAL, bool CG, bool ST>
__device__ __forceinline__ void
fwd_axis_tile(const Tile &tl, unsigned char *smem, const int32_t *__restrict__ idx,
              const T *__restrict__ B, int64_t ns, int64_t jcount, int d,
              const T *__restrict__ X, int64_t M, int64_t n, int64_t Q, int nch,
              T *__restrict__ Y) {
    using DT = DegreeTraits<D>;
    constexpr int DA = DT::DA;
    constexpr int DP = DT::DP;
    const int dd = DT::deg(d);
    SmemCarver sc{smem};
    int64_t *s_b = sc.take<int64_t>(kChunk);
    T *s_B = sc.take<T>(kChunk * DP);

    const int64_t j0 = tl.by * kChunk;
    for (int t = threadIdx.x; t < kChunk; t += blockDim.x) {
        const int64_t j = j0 + t;
        if (j < jcount) {
            s_b[t] = support_start(idx[j], dd, n);
#pragma unroll
            for (int i = 0; i < DP; ++i) s_B[t * DP + i] = (i <= dd) ? B[j + ns * i] : T(0);
        }
    }
    __syncthreads();
    const int64_t m0 = m_first<ST, VEC>(tl.bx);
    const int64_t ls = m_lane_stride<ST>();
    const int nv = m_valid<ST, VEC>(m0, M);
    if (nv == 0) return;
    const int jn = (int)((jcount - j0) < kChunk ? (jcount - j0) : kChunk);

    if constexpr (MODE == kPlain) {
        for (int64_t q = tl.bz; q < Q; q += tl.gz) {
            const T *xq = X + m0 + M * n * q;
            T *yq = Y + m0 + M * (j0 + ns * q);
            Pack<T, VEC> win[DA];
            int64_t bprev = -1;
            for (int t = 0; t < jn; ++t) {
                const int64_t b = s_b[t];
                if (b != bprev) {
#pragma unroll
                    for (int i = 0; i < DA; ++i)
                        if (i <= dd) win[i] = ldm<CG, ST, T, VEC>(xq + M * (b + i), ls, nv);
                    bprev = b;
                }
                Pack<T, VEC> acc;
#pragma unroll
                for (int v = 0; v < VEC; ++v) acc.v[v] = T(0);
                T bv[DA];
                basis_row<T, DA, DP>(s_B + t * DP, bv);
#pragma unroll
                for (int i = 0; i < DA; ++i) {
                    if (i <= dd) {
#pragma unroll
                        for (int v = 0; v < VEC; ++v) acc.v[v] += bv[i] * win[i].v[v];
                    }
                }
                stm<FINAL, ST, T, VEC>(yq + M * t, acc, ls, nv);
            }
        }
    } else {  // kRational: channels 0..nch in-thread (nch + 1 <= NC)
        if (tl.bz != 0) return;
        Pack<T, VEC> win[NC][DA];
        int64_t bprev = -1;
        for (int t = 0; t < jn; ++t) {
            const int64_t b = s_b[t];
            if (b != bprev) {
#pragma unroll
                for (int c = 0; c < NC; ++c)
                    if (c <= nch) {
                        const T *xc = X + m0 + M * n * c;
#pragma unroll
                        for (int i = 0; i < DA; ++i)
                            if (i <= dd) win[c][i] = ldm<CG, ST, T, VEC>(xc + M * (b + i), ls, nv);
                    }
                bprev = b;
            }
            Pack<T, VEC> acc[NC];
#pragma unroll
            for (int c = 0; c < NC; ++c)
#pragma unroll
                for (int v = 0; v < VEC; ++v) acc[c].v[v] = T(0);
            T bv[DA];
            basis_row<T, DA, DP>(s_B + t * DP, bv);
#pragma unroll
            for (int i = 0; i < DA; ++i) {
                if (i <= dd) {
#pragma unroll
                    for (int c = 0; c < NC; ++c)
                        if (c <= nch)
#pragma unroll
                            for (int v = 0; v < VEC; ++v) acc[c].v[v] += bv[i] * win[c][i].v[v];
                }
            }
#pragma unroll
            for (int c = 1; c < NC; ++c) {
                if (c <= nch) {
                    Pack<T, VEC> r;
#pragma unroll
                    for (int v = 0; v < VEC; ++v)
                        r.v[v] = (T)((double)acc[c].v[v] / (double)acc[0].v[v]);
                    stm<true, ST, T, VEC>(Y + m0 + M * ((j0 + t) + ns * (int64_t)(c - 1)), r, ls, nv);
                }
            }
        }
    }
}

// ---------------------------------------------------------------------------------
// Sorted view of the samples of one axis.  For sorted sample points (every
// SplineDimension the reference constructs, src/spline_dimension.jl:121-128) the
// view is the identity; otherwise `perm` is a stable sort of the samples by knot-span
// index, built by the plan.  Along the view the support starts are non-decreasing,
// so the samples that touch control points [c0, c1] are one contiguous range.
// ---------------------------------------------------------------------------------
__device__ __forceinline__ int64_t view_sample(const int32_t *perm, int64_t s) {
    return perm ? (int64_t)perm[s] : s;
}

// first position s in [0, ns) of the view with support start >= c (lower bound)
__device__ __forceinline__ int64_t view_lower_bound(const int32_t *idx, const int32_t *perm,
                                                    int64_t ns, int d, int64_t n, int64_t c) {
    int64_t lo = 0, hi = ns;
    while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if (support_start(idx[view_sample(perm, mid)], d, n) < c) lo = mid + 1; else hi = mid;
    }
    return lo;
}

// view_lower_bound(c) read from the axis' support table when the plan built one:
// lb[c + d] for c in [-d, n] (n + d + 1 entries); otherwise a binary search.
__device__ __forceinline__ int64_t support_lb(const int32_t *lb, const int32_t *idx,
                                              const int32_t *perm, int64_t ns, int d, int64_t n,
                                              int64_t c) {
    if (lb) {
        const int64_t i = c + d;
        return (int64_t)lb[i < 0 ? 0 : (i > n + d ? n + d : i)];
    }
    return view_lower_bound(idx, perm, ns, d, n, c);
}

// ---------------------------------------------------------------------------------
// Adjoint pass over axis k >= 1 (gather form):
//   Y[m, c, q] = sum_{j : b(j) <= c <= b(j)+d} B[j, c - b(j)] X[m, j, q].
// Tile = blockDim*VEC consecutive m x a chunk of CC control points [c0, c0+CC) x the
// columns q = bz, bz + gz, ...  The tile walks the contiguous sample range whose
// supports meet the chunk, in view order, with d+1 rolling accumulators per thread:
// accumulator i belongs to control point cur+i.  When the support start passes cur,
// control point cur is complete and is stored (also when no sample touched it, which
// stores 0 as the reference's zeroed output).  Each control point therefore sums its
// samples in increasing view order: deterministic, and no atomics.
// The input rows stream through a per-thread ring of S shared-memory slots filled by
// cp.async: S rows are always in flight, and no barrier sits on the data path (the
// basis rows of the range are staged separately in batches).  Neighbouring chunks
// share a halo of d knot spans.
// ---------------------------------------------------------------------------------
template <int D, typename T, int VEC>
__host__ __device__ constexpr int64_t adj_axis_smem_bytes(int threads) {
    return 16 + align16(kAdjBatch * 4) + align16(kAdjBatch * DegreeTraits<D>::DP * (int64_t)sizeof(T)) +
           align16((int64_t)AdjRing<T, VEC>::S * threads * VEC * (int64_t)sizeof(T));
}

template <int D, typename T, int VEC, bool CG, bool ST>
__device__ __forceinline__ void
adj_axis_tile(const Tile &tl, unsigned char *smem, const int32_t *__restrict__ idx,
              const int32_t *__restrict__ perm, const int32_t *__restrict__ lb,
              const T *__restrict__ B, int64_t ns, int d, const T *__restrict__ X, int64_t M,
              int64_t n, int64_t Q, int CC, T *__restrict__ Y) {
    using DT = DegreeTraits<D>;
    constexpr int DA = DT::DA;
    constexpr int DP = DT::DP;
    constexpr int S = AdjRing<T, VEC>::S;
    constexpr int CPB = ST ? (int)sizeof(T) : VEC * (int)sizeof(T);  // bytes per copy
    const int dd = DT::deg(d);
    SmemCarver sc{smem};
    int64_t *s_range = sc.take<int64_t>(2);
    int32_t *s_b = sc.take<int32_t>(kAdjBatch);
    T *s_B = sc.take<T>(kAdjBatch * DP);
    T *ring = sc.take<T>((int64_t)S * blockDim.x * VEC);  // [S][blockDim][VEC]

    const int c0 = (int)(tl.by * CC);
    const int c1 = (c0 + CC < n) ? c0 + CC : (int)n;  // exclusive
    if (threadIdx.x == 0) {
        s_range[0] = support_lb(lb, idx, perm, ns, dd, n, c0 - dd);
        s_range[1] = support_lb(lb, idx, perm, ns, dd, n, c1);
    }
    __syncthreads();
    const int64_t s_lo = s_range[0], s_hi = s_range[1];
    const int64_t total = s_hi - s_lo;
    const bool one_batch = total <= kAdjBatch;
    const int64_t m0 = m_first<ST, VEC>(tl.bx);
    const int64_t ls = m_lane_stride<ST>();
    const int nv = m_valid<ST, VEC>(m0, M);
    const bool active = nv > 0;
    T *const my_ring = ring + (int64_t)threadIdx.x * VEC;
    const int ring_stride = (int)blockDim.x * VEC;
    T *const ring_end = my_ring + S * ring_stride;
    // copy the thread's values of one input row into a ring slot
    auto fetch = [&](T *slot, const T *src) {
        if constexpr (!ST) {
            cp_async<CPB>(slot, src);
        } else {
#pragma unroll
            for (int v = 0; v < VEC; ++v)
                if (v < nv) cp_async<CPB>(slot + v, src + v * ls);
        }
    };
    auto flush = [&](T *yq, int c, const Pack<T, VEC> &a) {
        if (c >= c0) stm<false, ST, T, VEC>(yq + M * c, a, ls, nv);
    };

    for (int64_t q = tl.bz; q < Q; q += tl.gz) {
        const T *xq = X + m0 + M * ns * q;
        T *yq = Y + m0 + M * n * q;
        // prologue: rows 0..S-1 of the range in flight; src_next / next: the row the
        // next refill copies (consecutive rows are M apart unless the view permutes)
        int64_t next = s_lo;
        const T *src_next = xq + M * s_lo;
#pragma unroll
        for (int k = 0; k < S; ++k) {
            if (active && next < s_hi)
                fetch(my_ring + k * ring_stride, perm ? xq + M * perm[next] : src_next);
            ++next;
            src_next += M;
            cp_async_commit();
        }
        Pack<T, VEC> acc[DA];
#pragma unroll
        for (int i = 0; i < DA; ++i)
#pragma unroll
            for (int v = 0; v < VEC; ++v) acc[i].v[v] = T(0);
        int cur = c0 - dd;  // control point of acc[0]
        T *slot = my_ring;

        for (int64_t sb = s_lo; sb < s_hi; sb += kAdjBatch) {
            const int nb = (int)((s_hi - sb) < kAdjBatch ? (s_hi - sb) : kAdjBatch);
            // a range that fits one batch is staged once for all columns of the tile
            if (!one_batch || q == tl.bz) {
                __syncthreads();
                for (int t = threadIdx.x; t < nb; t += blockDim.x) {
                    const int64_t j = view_sample(perm, sb + t);
                    s_b[t] = (int32_t)support_start(idx[j], dd, n);
#pragma unroll
                    for (int i = 0; i < DP; ++i) s_B[t * DP + i] = (i <= dd) ? B[j + ns * i] : T(0);
                }
                __syncthreads();
            }
            for (int t = 0; t < nb; ++t) {
                cp_async_wait<S - 1>();  // the row in `slot` has landed
                if (active) {
                    const Pack<T, VEC> x = *reinterpret_cast<const Pack<T, VEC> *>(slot);
                    const int b = s_b[t];
                    while (cur < b) {  // control point `cur` is complete
                        flush(yq, cur, acc[0]);
#pragma unroll
                        for (int i = 0; i + 1 < DA; ++i) acc[i] = acc[i + 1];
#pragma unroll
                        for (int v = 0; v < VEC; ++v) acc[DA - 1].v[v] = T(0);
                        ++cur;
                    }
                    T bv[DA];
                    basis_row<T, DA, DP>(s_B + t * DP, bv);
#pragma unroll
                    for (int i = 0; i < DA; ++i) {
                        if (i <= dd) {
#pragma unroll
                            for (int v = 0; v < VEC; ++v) acc[i].v[v] += bv[i] * x.v[v];
                        }
                    }
                    // the slot's value is consumed above (in-order issue): refill it
                    if (next < s_hi) fetch(slot, perm ? xq + M * perm[next] : src_next);
                }
                ++next;
                src_next += M;
                cp_async_commit();
                slot += ring_stride;
                if (slot == ring_end) slot = my_ring;
            }
        }
        cp_async_wait<0>();
        if (active) {
            while (cur < c1) {
                flush(yq, cur, acc[0]);
#pragma unroll
                for (int i = 0; i + 1 < DA; ++i) acc[i] = acc[i + 1];
#pragma unroll
                for (int v = 0; v < VEC; ++v) acc[DA - 1].v[v] = T(0);
                ++cur;
            }
        }
    }
}

// ---------------------------------------------------------------------------------
// Adjoint pass over axis 0 (M = 1): Y[c, q] = sum_{j in S(c)} B[j, c - b(j)] X[j, q].
// Tile = CT control points x QT columns q (CT*QT = blockDim).  The samples whose
// supports meet the tile's control points form one contiguous range of the sorted
// view; it is walked in batches of kAdj0Batch samples whose support starts, basis
// rows and X values (QT columns, coalesced along j) are staged in shared memory.
// Thread (c, q) sums the samples of its own support S(c) in view order: deterministic
// and without atomics.
// ---------------------------------------------------------------------------------
template <int D, typename T>
__host__ __device__ constexpr int64_t adj_axis0_smem_bytes(int QT) {
    return 16 + kAdj0Batch * 4 + align16(kAdj0Batch * DegreeTraits<D>::DA * (int64_t)sizeof(T)) +
           align16(QT * (kAdj0Batch + 1) * (int64_t)sizeof(T));
}

template <int D, typename T, bool CG>
__device__ __forceinline__ void
adj_axis0_tile(const Tile &tl, unsigned char *smem, const int32_t *__restrict__ idx,
               const int32_t *__restrict__ perm, const int32_t *__restrict__ lb,
               const T *__restrict__ B, int64_t ns, int d, const T *__restrict__ X, int64_t n,
               int64_t Q, int QT, T *__restrict__ Y) {
    using DT = DegreeTraits<D>;
    constexpr int DA = DT::DA;
    const int dd = DT::deg(d);
    const int CT = (int)blockDim.x / QT;
    SmemCarver sc{smem};
    int64_t *s_range = sc.take<int64_t>(2);
    int32_t *s_bs = sc.take<int32_t>(kAdj0Batch);
    T *s_B = sc.take<T>(kAdj0Batch * DA);
    T *s_x = sc.take<T>((int64_t)QT * (kAdj0Batch + 1));  // [QT][kAdj0Batch + 1]

    const int64_t c0 = tl.bx * CT;
    const int64_t c1 = (c0 + CT < n) ? c0 + CT : n;
    // consecutive threads take consecutive columns q of one control point: they read
    // the same basis values (broadcast) and, with the padded row stride, different
    // banks of the staged X values
    const int tq = threadIdx.x % QT, tc = threadIdx.x / QT;
    const int64_t c = c0 + tc;
    if (threadIdx.x == 0) {
        s_range[0] = support_lb(lb, idx, perm, ns, dd, n, c0 - dd);
        s_range[1] = support_lb(lb, idx, perm, ns, dd, n, c1);
    }
    // this thread's own support [my_lo, my_hi) within the tile's range
    int64_t my_lo = 0, my_hi = 0;
    if (c < c1) {
        my_lo = support_lb(lb, idx, perm, ns, dd, n, c - dd);
        my_hi = support_lb(lb, idx, perm, ns, dd, n, c + 1);
    }
    __syncthreads();
    const int64_t s_lo = s_range[0], s_hi = s_range[1];
    for (int64_t q0 = tl.by * QT; q0 < Q; q0 += tl.gy * QT) {
        const int64_t q = q0 + tq;
        T acc = T(0);
        for (int64_t sb = s_lo; sb < s_hi; sb += kAdj0Batch) {
            const int nb = (int)((s_hi - sb) < kAdj0Batch ? (s_hi - sb) : kAdj0Batch);
            __syncthreads();
            for (int t = threadIdx.x; t < nb; t += blockDim.x) {
                const int64_t j = view_sample(perm, sb + t);
                s_bs[t] = (int32_t)support_start(idx[j], dd, n);
#pragma unroll
                for (int i = 0; i < DA; ++i) s_B[t * DA + i] = (i <= dd) ? B[j + ns * i] : T(0);
            }
            {   // one warp per column q, lanes along the samples: coalesced, no division
                const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
                const int nwarps = (int)blockDim.x >> 5;
                for (int qq = warp; qq < QT; qq += nwarps) {
                    const int64_t qg = q0 + qq;
                    const T *xc = X + ns * qg;
                    for (int t = lane; t < nb; t += 32)
                        s_x[qq * (kAdj0Batch + 1) + t] =
                            (qg < Q) ? ldx<CG>(xc + view_sample(perm, sb + t)) : T(0);
                }
            }
            __syncthreads();
            if (c < c1 && q < Q) {
                const int64_t a = my_lo > sb ? my_lo : sb;
                const int64_t z = my_hi < sb + nb ? my_hi : sb + nb;
                for (int64_t sv = a; sv < z; ++sv) {
                    const int t = (int)(sv - sb);
                    const int i = (int)(c - s_bs[t]);
                    if (i >= 0 && i <= dd) acc += s_B[t * DA + i] * s_x[tq * (kAdj0Batch + 1) + t];
                }
            }
        }
        if (c < c1 && q < Q) Y[c + n * q] = acc;
    }
}

// ---------------------------------------------------------------------------------
// Per-grid kernels: one tile per CTA.
// ---------------------------------------------------------------------------------
template <int D, typename TX, typename T, int MODE>
__global__ void __launch_bounds__(kThreads)
k_fwd_axis0(const int32_t *__restrict__ idx, const T *__restrict__ B, int64_t ns, int d,
            const TX *__restrict__ X, const T *__restrict__ w, int64_t n, int64_t Qr, int nch,
            T *__restrict__ Y) {
    fwd_axis0_tile<D, TX, T, MODE>(grid_tile(), idx, B, ns, d, X, w, n, Qr, nch, Y);
}

template <int D, typename T, int VEC, int MODE, int NC, bool FINAL, bool ST>
__global__ void __launch_bounds__(kThreads)
k_fwd_axis(const int32_t *__restrict__ idx, const T *__restrict__ B, int64_t ns,
           int64_t jcount, int d, const T *__restrict__ X, int64_t M, int64_t n, int64_t Q,
           int nch, T *__restrict__ Y) {
    __shared__ __align__(16) unsigned char smem[fwd_axis_smem_bytes<D, T>()];
    fwd_axis_tile<D, T, VEC, MODE, NC, FINAL, false, ST>(grid_tile(), smem, idx, B, ns, jcount, d,
                                                         X, M, n, Q, nch, Y);
}

template <int D, typename T, int VEC, bool ST>
__global__ void __launch_bounds__(kThreads)
k_adj_axis(const int32_t *__restrict__ idx, const int32_t *__restrict__ perm,
           const int32_t *__restrict__ lb, const T *__restrict__ B, int64_t ns, int d,
           const T *__restrict__ X, int64_t M, int64_t n, int64_t Q, int CC,
           T *__restrict__ Y) {
    extern __shared__ __align__(16) unsigned char s_dyn[];
    adj_axis_tile<D, T, VEC, false, ST>(grid_tile(), s_dyn, idx, perm, lb, B, ns, d, X, M, n, Q,
                                        CC, Y);
}

template <int D, typename T>
__global__ void __launch_bounds__(kAdj0Threads)
k_adj_axis0(const int32_t *__restrict__ idx, const int32_t *__restrict__ perm,
            const int32_t *__restrict__ lb, const T *__restrict__ B, int64_t ns, int d,
            const T *__restrict__ X, int64_t n, int64_t Q, int QT, T *__restrict__ Y) {
    extern __shared__ __align__(16) unsigned char s_dyn[];
    adj_axis0_tile<D, T, false>(grid_tile(), s_dyn, idx, perm, lb, B, ns, d, X, n, Q, QT, Y);
}

// Rational last pass for any channel count (nch + 1 > the in-thread bound) or degree:
// plain loads per output, one thread per m.
template <typename T>
__global__ void __launch_bounds__(kThreads)
k_fwd_axis_rational_generic(const int32_t *__restrict__ idx, const T *__restrict__ B,
                            int64_t ns, int d, const T *__restrict__ X, int64_t M, int64_t n,
                            int nch, T *__restrict__ Y) {
    const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= M) return;
    for (int64_t j = blockIdx.y; j < ns; j += gridDim.y) {
        const int64_t b = support_start(idx[j], d, n);
        T den = T(0);
        for (int i = 0; i <= d; ++i) den += B[j + ns * i] * X[m + M * (b + i)];
        for (int c = 1; c <= nch; ++c) {
            T num = T(0);
            for (int i = 0; i <= d; ++i) num += B[j + ns * i] * X[m + M * ((b + i) + n * c)];
            __stcs(Y + m + M * (j + ns * (int64_t)(c - 1)), (T)((double)num / (double)den));
        }
    }
}

}  // namespace sg
