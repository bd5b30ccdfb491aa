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
// Degree handling: template D = d+1 for D in 1..4; D = 0 is the generic kernel for
// any degree up to SG_MAX_DEGREE with register arrays of kDMax entries.
#pragma once

#include "sg_common.cuh"

namespace sg {

template <int D>
struct DegreeTraits {
    static constexpr int DA = D > 0 ? D : kDMax;  // register array extent
    static __device__ __forceinline__ int deg(int runtime_d) { return D > 0 ? D - 1 : runtime_d; }
};

// Samples of the basis table staged per CTA in shared memory.
constexpr int kChunk = 32;        // forward: samples of axis k per CTA
constexpr int kAdjBatch = 64;     // adjoint: samples staged per batch
constexpr int kAdjUnroll = 8;     // adjoint: cotangent loads in flight per thread
constexpr int kThreads = 128;

// Homogeneous (rational) channel layout of NURBS grids: channel 0 carries the weight,
// channel o >= 1 carries w * P[..., o-1].  The last forward pass divides channels
// 1..nout by channel 0 (the `denom` of src/spline_grid.jl:160-182).
enum FwdMode : int { kPlain = 0, kHomog = 1, kRational = 2 };

// ---------------------------------------------------------------------------------
// Forward pass over axis 0 (M = 1): Y[j, q] = sum_i B[j, i] X[b(j) + i, q].
// One thread per sample j keeps its d+1 basis values in registers and walks a range
// of q; neighbouring threads read the same control-point rows, which stay in L1.
//   kPlain:    X is the control-point tensor [n, Q] (TX may be bfloat16).
//   kHomog:    X is [n, Qr, nch] with weights w [n, Qr]; Y is [ns, Qr, nch+1] in the
//              homogeneous layout above (NURBS grids with Nin >= 2).
//   kRational: Nin == 1 NURBS: Y[j, o] = sum B w P / sum B w, divided in Float64.
// ---------------------------------------------------------------------------------
template <int D, typename TX, typename T, int MODE>
__global__ void __launch_bounds__(kThreads)
k_fwd_axis0(const int32_t *__restrict__ idx, const T *__restrict__ B, int64_t ns, int d,
            const TX *__restrict__ X, const T *__restrict__ w, int64_t n, int64_t Qr, int nch,
            T *__restrict__ Y) {
    using DT = DegreeTraits<D>;
    constexpr int DA = DT::DA;
    const int dd = DT::deg(d);
    const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (j >= ns) return;
    const int64_t b = support_start(idx[j], dd, n);
    T bw[DA];
#pragma unroll
    for (int i = 0; i < DA; ++i) bw[i] = (i <= dd) ? B[j + ns * i] : T(0);

    if constexpr (MODE == kRational) {
        if (blockIdx.y != 0) return;
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
        for (int64_t q = blockIdx.y; q < Qy; q += gridDim.y) {
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
// CTA = kThreads*VEC consecutive m (coalesced VEC-wide accesses) x kChunk samples of
// axis k x one q per gridDim.z step.  The chunk's basis rows and support starts are
// staged in shared memory; each thread keeps a register window of the d+1 input rows
// of the current knot span and reloads it only when the span changes (every
// n_samples/n_basis samples), so X is read ~once per span while each output costs d+1
// FMAs.  FINAL passes write eval with streaming stores.
//   kRational (NURBS, last axis): Q is the NC channel axis of the homogeneous layout;
//   the thread keeps NC windows and divides channels 1..nch by channel 0 in Float64.
// ---------------------------------------------------------------------------------
template <int D, typename T, int VEC, int MODE, int NC, bool FINAL>
__global__ void __launch_bounds__(kThreads)
k_fwd_axis(const int32_t *__restrict__ idx, const T *__restrict__ B, int64_t ns,
           int64_t jcount, int d, const T *__restrict__ X, int64_t M, int64_t n, int64_t Q,
           int nch, T *__restrict__ Y) {
    // ns: sample count of the axis (stride of B and Y); jcount: samples addressed by
    // this launch, counted from the (possibly shifted) idx/B/Y bases.
    using DT = DegreeTraits<D>;
    constexpr int DA = DT::DA;
    const int dd = DT::deg(d);
    __shared__ int64_t s_b[kChunk];
    __shared__ T s_B[kChunk * DA];

    const int64_t j0 = (int64_t)blockIdx.y * kChunk;
    for (int t = threadIdx.x; t < kChunk; t += blockDim.x) {
        const int64_t j = j0 + t;
        if (j < jcount) {
            s_b[t] = support_start(idx[j], dd, n);
#pragma unroll
            for (int i = 0; i < DA; ++i) s_B[t * DA + i] = (i <= dd) ? B[j + ns * i] : T(0);
        }
    }
    __syncthreads();
    const int64_t m0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * VEC;
    if (m0 >= M) return;
    const int jn = (int)((jcount - j0) < kChunk ? (jcount - j0) : kChunk);

    if constexpr (MODE == kPlain) {
        for (int64_t q = blockIdx.z; q < Q; q += gridDim.z) {
            const T *xq = X + m0 + M * n * q;
            T *yq = Y + m0 + M * (j0 + ns * q);
            Pack<T, VEC> win[DA];
            int64_t bprev = -1;
            for (int t = 0; t < jn; ++t) {
                const int64_t b = s_b[t];
                if (b != bprev) {
#pragma unroll
                    for (int i = 0; i < DA; ++i)
                        if (i <= dd) win[i] = ldp<T, VEC>(xq + M * (b + i));
                    bprev = b;
                }
                Pack<T, VEC> acc;
#pragma unroll
                for (int v = 0; v < VEC; ++v) acc.v[v] = T(0);
#pragma unroll
                for (int i = 0; i < DA; ++i) {
                    if (i <= dd) {
                        const T bv = s_B[t * DA + i];
#pragma unroll
                        for (int v = 0; v < VEC; ++v) acc.v[v] += bv * win[i].v[v];
                    }
                }
                if constexpr (FINAL) stp_stream<T, VEC>(yq + M * t, acc);
                else stp<T, VEC>(yq + M * t, acc);
            }
        }
    } else {  // kRational: channels 0..nch in-thread (nch + 1 <= NC)
        if (blockIdx.z != 0) return;
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
                            if (i <= dd) win[c][i] = ldp<T, VEC>(xc + M * (b + i));
                    }
                bprev = b;
            }
            Pack<T, VEC> acc[NC];
#pragma unroll
            for (int c = 0; c < NC; ++c)
#pragma unroll
                for (int v = 0; v < VEC; ++v) acc[c].v[v] = T(0);
#pragma unroll
            for (int i = 0; i < DA; ++i) {
                if (i <= dd) {
                    const T bv = s_B[t * DA + i];
#pragma unroll
                    for (int c = 0; c < NC; ++c)
                        if (c <= nch)
#pragma unroll
                            for (int v = 0; v < VEC; ++v) acc[c].v[v] += bv * win[c][i].v[v];
                }
            }
#pragma unroll
            for (int c = 1; c < NC; ++c) {
                if (c <= nch) {
                    Pack<T, VEC> r;
#pragma unroll
                    for (int v = 0; v < VEC; ++v)
                        r.v[v] = (T)((double)acc[c].v[v] / (double)acc[0].v[v]);
                    stp_stream<T, VEC>(Y + m0 + M * ((j0 + t) + ns * (int64_t)(c - 1)), r);
                }
            }
        }
    }
}

// Rational last pass for any channel count (nch + 1 > the in-thread bound): plain
// loads per output, one thread per m.
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

// ---------------------------------------------------------------------------------
// Adjoint pass over axis k >= 1 (gather form):
//   Y[m, c, q] = sum_{j : b(j) <= c <= b(j)+d} B[j, c - b(j)] X[m, j, q].
// CTA = kThreads*VEC consecutive m x a chunk of CC control points [c0, c0+CC) x one q.
// The CTA walks the contiguous sample range whose supports meet the chunk, in view
// order, with d+1 rolling accumulators per thread: accumulator i belongs to control
// point cur+i.  When the support start passes cur, control point cur is complete and
// is stored (also when no sample touched it, which stores 0 as the reference's zeroed
// output).  Each control point therefore sums its samples in increasing view order:
// deterministic, and no atomics.  X (the cotangent on the first pass) is read once
// per chunk; neighbouring chunks share a halo of d knot spans.
// ---------------------------------------------------------------------------------
template <int D, typename T, int VEC>
__global__ void __launch_bounds__(kThreads)
k_adj_axis(const int32_t *__restrict__ idx, const int32_t *__restrict__ perm,
           const T *__restrict__ B, int64_t ns, int d, const T *__restrict__ X, int64_t M,
           int64_t n, int64_t Q, int CC, T *__restrict__ Y) {
    using DT = DegreeTraits<D>;
    constexpr int DA = DT::DA;
    const int dd = DT::deg(d);
    __shared__ int64_t s_range[2];
    __shared__ int64_t s_b[kAdjBatch];
    __shared__ int64_t s_j[kAdjBatch];
    __shared__ T s_B[kAdjBatch * DA];

    const int64_t c0 = (int64_t)blockIdx.y * CC;
    const int64_t c1 = (c0 + CC < n) ? c0 + CC : n;  // exclusive
    if (threadIdx.x == 0) {
        s_range[0] = view_lower_bound(idx, perm, ns, dd, n, c0 - dd);
        s_range[1] = view_lower_bound(idx, perm, ns, dd, n, c1);
    }
    __syncthreads();
    const int64_t s_lo = s_range[0], s_hi = s_range[1];
    const int64_t m0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * VEC;
    const bool active = m0 < M;

    for (int64_t q = blockIdx.z; q < Q; q += gridDim.z) {
        const T *xq = X + m0 + M * ns * q;
        T *yq = Y + m0 + M * n * q;
        Pack<T, VEC> acc[DA];
#pragma unroll
        for (int i = 0; i < DA; ++i)
#pragma unroll
            for (int v = 0; v < VEC; ++v) acc[i].v[v] = T(0);
        int64_t cur = c0 - dd;  // control point of acc[0]

        for (int64_t sb = s_lo; sb < s_hi; sb += kAdjBatch) {
            const int nb = (int)((s_hi - sb) < kAdjBatch ? (s_hi - sb) : kAdjBatch);
            __syncthreads();
            for (int t = threadIdx.x; t < nb; t += blockDim.x) {
                const int64_t j = view_sample(perm, sb + t);
                s_j[t] = j;
                s_b[t] = support_start(idx[j], dd, n);
#pragma unroll
                for (int i = 0; i < DA; ++i) s_B[t * DA + i] = (i <= dd) ? B[j + ns * i] : T(0);
            }
            __syncthreads();
            if (active) {
                // kAdjUnroll independent loads are issued before any of them is consumed,
                // so each thread keeps that many cotangent rows in flight.
                for (int t0 = 0; t0 < nb; t0 += kAdjUnroll) {
                    Pack<T, VEC> xs[kAdjUnroll];
#pragma unroll
                    for (int u = 0; u < kAdjUnroll; ++u)
                        if (t0 + u < nb) xs[u] = ldp<T, VEC>(xq + M * s_j[t0 + u]);
#pragma unroll
                    for (int u = 0; u < kAdjUnroll; ++u) {
                        if (t0 + u >= nb) break;
                        const int t = t0 + u;
                        const int64_t b = s_b[t];
                        while (cur < b) {  // control point `cur` is complete
                            if (cur >= c0) stp<T, VEC>(yq + M * cur, acc[0]);
#pragma unroll
                            for (int i = 0; i + 1 < DA; ++i) acc[i] = acc[i + 1];
#pragma unroll
                            for (int v = 0; v < VEC; ++v) acc[DA - 1].v[v] = T(0);
                            ++cur;
                        }
#pragma unroll
                        for (int i = 0; i < DA; ++i) {
                            if (i <= dd) {
                                const T bv = s_B[t * DA + i];
#pragma unroll
                                for (int v = 0; v < VEC; ++v) acc[i].v[v] += bv * xs[u].v[v];
                            }
                        }
                    }
                }
            }
        }
        if (active) {
            while (cur < c1) {
                if (cur >= c0) stp<T, VEC>(yq + M * cur, acc[0]);
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
// CTA = CT control points x QT columns q (CT*QT = 256 threads).  The samples whose
// supports meet the CTA's control points form one contiguous range of the sorted
// view; it is walked in batches of kAdj0Batch samples whose support starts, basis
// rows and X values (QT columns, coalesced along j) are staged in shared memory.
// Thread (c, q) sums the samples of its own support S(c) in view order: deterministic
// and without atomics.
// ---------------------------------------------------------------------------------
constexpr int kAdj0Batch = 128;
constexpr int kAdj0Threads = 256;

template <int D, typename T>
__global__ void __launch_bounds__(kAdj0Threads)
k_adj_axis0(const int32_t *__restrict__ idx, const int32_t *__restrict__ perm,
            const T *__restrict__ B, int64_t ns, int d, const T *__restrict__ X, int64_t n,
            int64_t Q, int QT, T *__restrict__ Y) {
    using DT = DegreeTraits<D>;
    constexpr int DA = DT::DA;
    const int dd = DT::deg(d);
    const int CT = kAdj0Threads / QT;
    __shared__ int64_t s_range[2];
    __shared__ int32_t s_bs[kAdj0Batch];
    __shared__ T s_B[kAdj0Batch * DA];
    extern __shared__ unsigned char s_dyn[];
    T *s_x = reinterpret_cast<T *>(s_dyn);  // [QT][kAdj0Batch]

    const int64_t c0 = (int64_t)blockIdx.x * CT;
    const int64_t c1 = (c0 + CT < n) ? c0 + CT : n;
    const int tc = threadIdx.x % CT, tq = threadIdx.x / CT;
    const int64_t c = c0 + tc;
    if (threadIdx.x == 0) {
        s_range[0] = view_lower_bound(idx, perm, ns, dd, n, c0 - dd);
        s_range[1] = view_lower_bound(idx, perm, ns, dd, n, c1);
    }
    __syncthreads();
    const int64_t s_lo = s_range[0], s_hi = s_range[1];
    // this thread's own support [my_lo, my_hi) within the CTA range
    int64_t my_lo = 0, my_hi = 0;
    if (c < c1) {
        my_lo = view_lower_bound(idx, perm, ns, dd, n, c - dd);
        my_hi = view_lower_bound(idx, perm, ns, dd, n, c + 1);
    }
    for (int64_t q0 = (int64_t)blockIdx.y * QT; q0 < Q; q0 += (int64_t)gridDim.y * QT) {
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
            for (int e = threadIdx.x; e < nb * QT; e += blockDim.x) {
                const int t = e % nb, qq = e / nb;
                const int64_t qg = q0 + qq;
                s_x[qq * kAdj0Batch + t] = (qg < Q) ? X[view_sample(perm, sb + t) + ns * qg] : T(0);
            }
            __syncthreads();
            if (c < c1 && q < Q) {
                const int64_t a = my_lo > sb ? my_lo : sb;
                const int64_t z = my_hi < sb + nb ? my_hi : sb + nb;
                for (int64_t sv = a; sv < z; ++sv) {
                    const int t = (int)(sv - sb);
                    const int i = (int)(c - s_bs[t]);
                    if (i >= 0 && i <= dd) acc += s_B[t * DA + i] * s_x[tq * kAdj0Batch + t];
                }
            }
        }
        if (c < c1 && q < Q) Y[c + n * q] = acc;
    }
}

}  // namespace sg
