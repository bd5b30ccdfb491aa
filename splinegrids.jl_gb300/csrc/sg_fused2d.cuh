// sg_fused2d.cuh -- evaluate! and evaluate_adjoint! of a grid with Nin = 2 in ONE pass
// over eval: both axes are contracted on chip, nothing intermediate goes to HBM.
//
// The separable form (sg_contract.cuh) applies eval = (B_0 (x) B_1) P one axis per
// pass: the axis-0 pass writes an intermediate Y[ns0, n1, nch] that the axis-1 pass
// reads back.  For Nin = 2 both contractions fit in one unit of work:
//
// Forward warp task = (channel, 128 consecutive axis-0 samples, a block of axis-1
//   rows).  Each lane keeps, for its four samples, the d1+1 values Y[s0, b1..b1+d1, c]
//   of the current axis-1 knot span in registers; a new column
//   Y[s0, r, c] = sum_i B0[s0, i] P[b0(s0)+i, r, c] is formed from control points
//   fetched one run of rows ahead; eval rows are written with streaming stores.  The
//   only HBM traffic is eval (written once) and the small control-point tensor.
// Adjoint tile = (channel group, a block of axis-0 control points, a block of axis-1
//   control points), axis 0 whole.  Phase A walks the axis-1 sample rows that touch the
//   block (the cotangent, read once, moved by bulk copies into a shared-memory ring)
//   with d1+1 rolling accumulators per (sample, channel) pair; a finished axis-1
//   control point leaves its column Z[., c1] in a shared-memory ring.  Every kF2Half
//   finished columns, phase B contracts them along axis 0: each output control point
//   sums its axis-0 samples in increasing order.
//
// Operation order.  Every value is the same chain of FMAs as in the separable passes:
// Y and eval (forward), Z and the gradient (adjoint) each start from zero and add their
// terms in increasing basis/sample order with one rounding per FMA (fma.rn.f32x2 for
// Float32 pairs rounds each half as one FFMA).  The fused results are therefore bitwise
// those of the separable passes (tested), deterministic, and without atomics.
//
// Requirements (checked by the host before choosing this path): degrees <= 3, element
// offsets of eval and control points below 2^31; the adjoint also needs sorted samples
// on both axes and axis 0's samples times one channel within one tile.
#pragma once

#include <type_traits>

#include "sg_contract.cuh"
#include "sg_mbar.cuh"

namespace sg {

constexpr int kF2Ring = 8;         // adjoint: finished axis-1 columns held in shared memory
constexpr int kF2Half = kF2Ring / 2;
constexpr int kF2Consumers = 8;    // adjoint: consumer warps (the producer warp is the 9th)
constexpr int kF2AdjThreads = 32 * (kF2Consumers + 1);
constexpr int kF2Rows = 4;         // adjoint: cotangent rows per stage
constexpr int kF2NS = 3;           // adjoint: stages in the ring
constexpr int kF2PhaseBPerStage = 1;  // adjoint: pending phase-B items a thread takes per stage
constexpr int kF2BarBytes = ((2 * kF2NS * 8 + 15) / 16) * 16;  // full + empty mbarriers
constexpr int kF2MaxG = 32;        // adjoint: channels per tile at most (one bulk copy each)

// Adjoint tiles: (sample, channel) pairs per tile; four pairs per consumer thread for
// Float32 (two register pairs), two for Float64.
template <typename T>
__host__ __device__ constexpr int f2_pairs() { return sizeof(T) == 4 ? 1024 : 512; }
template <typename T>
__host__ __device__ constexpr int f2_j() { return f2_pairs<T>() / (32 * kF2Consumers); }
// row stride of the Z ring: one value of padding keeps phase B's reads of neighbouring
// columns in different banks
template <typename T>
__host__ __device__ constexpr int f2_zstride() { return f2_pairs<T>() + 1; }
// one stage of the cotangent ring: per channel a segment of kF2Rows whole rows plus
// up to 16 bytes of alignment lead, rounded to 16 bytes
template <typename T>
__host__ __device__ constexpr int f2_stage_elems() {
    return kF2Rows * f2_pairs<T>() + kF2MaxG * 2 * (16 / (int)sizeof(T));
}
// segment capacity (elements, a 16-byte multiple) of a channel with ns0 samples per row
__host__ __device__ constexpr int f2_seg_elems(int ns0, int es) {
    return ((kF2Rows * ns0 * es + 16 + 15) / 16) * 16 / es;
}

// Two values as one register pair: Float32 pairs use fma.rn.f32x2.
template <typename T>
struct F2Pair;
template <>
struct F2Pair<float> {
    using V = float2;
    static __device__ __forceinline__ V zero() { return make_float2(0.f, 0.f); }
    static __device__ __forceinline__ V make(float a, float b) { return make_float2(a, b); }
    static __device__ __forceinline__ V fma(V b, V x, V c) { return __ffma2_rn(b, x, c); }
};
template <>
struct F2Pair<double> {
    using V = double2;
    static __device__ __forceinline__ V zero() { return make_double2(0.0, 0.0); }
    static __device__ __forceinline__ V make(double a, double b) { return make_double2(a, b); }
    static __device__ __forceinline__ V fma(V b, V x, V c) {
        return make_double2(::fma(b.x, x.x, c.x), ::fma(b.y, x.y, c.y));
    }
};

// What a fused unit of work reads of one grid and one derivative order.
struct F2Grid {
    const int32_t *idx0, *idx1;  // sample indices (1-based)
    const int32_t *lb0, *lb1;    // support tables lb[c + d] (adjoint)
    const int32_t *off0;         // adjoint: off0[c] = sum over c' < c of |S0(c')| (axis-0 weight list)
    const void *B0, *B1;         // basis blocks of the derivative order: B[s + ns*i]
    const void *X;               // forward: control points [n0, n1, nch]; adjoint: eval_bar
    void *Y;                     // forward: eval [ns0, ns1, nch]; adjoint: gradient
    int64_t ns0, ns1, n0, n1;
    int32_t d0, d1, nch, pad;
};

// One unit.  Forward: samples [a_lo, a_lo+a_len) of axis 0 x rows [b_lo, b_lo+b_len)
// of axis 1 in channel c_lo (G = 1); adjoint: control points [a_lo, ..) of axis 0 x
// [b_lo, ..) of axis 1, channels [c_lo, c_lo+G).
struct F2Tile {
    int32_t grid, kind;  // kind 0 forward warp task, 1 adjoint tile, 2 forward tile
    int32_t c_lo, G;
    int32_t a_lo, a_len;
    int32_t b_lo, b_len;
    int32_t cb, ncol;    // forward tile: first axis-1 column and column count (0: from the samples)
};

// Uniform blocking of one grid in one direction.  Adjoint unit i is (group, a block,
// b block) with the b block fastest: consecutive tiles are neighbours along axis 1 and
// share their halo rows in L2.  Forward unit i is (group, b block, a block) with the a
// block fastest: the warps of a CTA (consecutive units) write neighbouring 512-byte
// pieces of the same eval rows at about the same time, whole DRAM pages.
struct F2Tiling {
    int32_t G = 0, ngrp = 0;  // channels per group, groups
    int32_t ka = 0, nba = 0;  // block length and count along a
    int32_t kb = 0, nbb = 0;  // along b
    __host__ __device__ int64_t count() const { return (int64_t)ngrp * nba * nbb; }
    __host__ __device__ F2Tile tile(int64_t i, int kind, int nch, int64_t na, int64_t nb) const {
        F2Tile t;
        t.cb = t.ncol = 0;
        int64_t ia, ib;
        if (kind != 1) {  // forward (warp tasks: 0, tiles: 2)
            ia = i % nba;
            i /= nba;
            ib = i % nbb;
            i /= nbb;
        } else {
            ib = i % nbb;
            i /= nbb;
            ia = i % nba;
            i /= nba;
        }
        const int64_t grp = i;
        t.grid = 0;
        t.kind = kind;
        t.c_lo = (int32_t)(grp * G);
        t.G = (int32_t)((nch - t.c_lo) < G ? (nch - t.c_lo) : G);
        t.a_lo = (int32_t)(ia * ka);
        t.a_len = (int32_t)((na - t.a_lo) < ka ? (na - t.a_lo) : ka);
        t.b_lo = (int32_t)(ib * kb);
        t.b_len = (int32_t)((nb - t.b_lo) < kb ? (nb - t.b_lo) : kb);
        return t;
    }
};

// adjoint shared memory, in carving order
template <typename T>
__host__ __device__ constexpr int64_t f2_adj_hdr_bytes() {  // per stage: basis rows, starts, segment bases
    return align16((int64_t)kF2Rows * 4 * 2 * sizeof(T)) + align16(kF2Rows * 4) + align16(kF2MaxG * 4);
}
template <typename T>
__host__ __device__ constexpr int64_t f2_adj_smem() {
    return kF2BarBytes                                                 // full + empty barriers
           + 16                                                        // abort flag
           + kF2NS * f2_adj_hdr_bytes<T>()                             // stage headers
           + kF2NS * align16((int64_t)f2_stage_elems<T>() * sizeof(T))  // cotangent ring
           + align16((int64_t)kF2Ring * f2_zstride<T>() * sizeof(T))   // Z ring
           + (int64_t)f2_pairs<T>() * 4 * sizeof(T);                  // axis-0 weight list
}

// ---------------------------------------------------------------------------------
// Forward warp task: eval[s0, s1, c] = sum_k B1[s1, k] Y[s0, b1(s1)+k, c],
//                    Y[s0, r, c]     = sum_i B0[s0, i] P[b0(s0)+i, r, c],
// for the samples s0 in [a_lo, a_lo + a_len) (a_len <= 128) of one channel c and the
// rows s1 in [b_lo, b_lo + b_len).  Lane l owns s0 = a_lo + l + 32 v (v < 4): a row's
// four stores share one address (immediate offsets), and each store instruction of
// the warp covers 128 consecutive bytes of eval; or, for Float32 rows of 16-byte
// multiples (CT), s0 = a_lo + 4 l + v, stored as one 16-byte access (512 bytes per
// warp instruction).  The lane keeps the window
// Y[., b .. b+d1] of its four samples in registers (as two value pairs) and the control
// points of the column after it, fetched one run of rows ahead.  Axis-1 basis rows are
// staged 32 at a time in the warp's slice of shared memory; the warp never waits for
// another.  Index arithmetic is 32-bit (the host admits grids whose eval and control
// points have fewer than 2^31 elements).
// ---------------------------------------------------------------------------------
constexpr int kF2Lanes = 32;
constexpr int kF2LaneVals = 4;                       // samples per lane
constexpr int kF2WarpS0 = kF2Lanes * kF2LaneVals;    // samples per forward warp task
constexpr int kF2FwdWarps = 8;                       // warps (tasks) per forward CTA

template <typename T>
__host__ __device__ constexpr int64_t f2_fwd_warp_smem() {
    return (int64_t)kF2Lanes * 4 * 2 * sizeof(T)              // staged axis-1 rows (pairs)
           + (int64_t)kF2Lanes * 4                             // their support starts
           + (int64_t)kF2LaneVals * 4 * kF2Lanes * sizeof(T);  // axis-0 basis rows of the lanes
}
template <typename T>
__host__ __device__ constexpr int64_t f2_fwd_smem() { return kF2FwdWarps * f2_fwd_warp_smem<T>(); }

template <typename T, typename TX, int D1, bool CT = false>
__device__ __forceinline__ void f2_forward_warp(const F2Grid &g, const F2Tile &tl, unsigned char *wsm) {
    using PT = F2Pair<T>;
    using V = typename PT::V;
    constexpr int L = kF2Lanes;
    const int lane = threadIdx.x & (L - 1);
    const int d0 = g.d0;
    const int ns0 = (int)g.ns0, ns1 = (int)g.ns1, n0 = (int)g.n0, n1 = (int)g.n1;
    const int c = tl.c_lo;
    V *sB1 = reinterpret_cast<V *>(wsm);                      // [32][4], each value in both halves
    int32_t *sb1 = reinterpret_cast<int32_t *>(sB1 + L * 4);  // [32]
    V *sBw = reinterpret_cast<V *>(sb1 + L);                  // [2 jp][4 i][32 lanes]
    uint32_t pofs[4];
    {
        const T *__restrict__ B0 = (const T *)g.B0;
        T *w = reinterpret_cast<T *>(sBw);
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            const int sv = CT ? 4 * lane + v : lane + L * v;  // the lane's v-th sample in the task
            const bool ok = sv < tl.a_len;
            const int s0 = tl.a_lo + sv;
            const int b0 = ok ? (int)support_start(g.idx0[s0], d0, n0) : 0;
            pofs[v] = (uint32_t)b0 + (uint32_t)n0 * (uint32_t)n1 * (uint32_t)c;
#pragma unroll
            for (int i = 0; i < 4; ++i)
                w[2 * (((v >> 1) * 4 + i) * L + lane) + (v & 1)] = (ok && i <= d0) ? B0[s0 + ns0 * i] : T(0);
        }
    }
    const TX *__restrict__ P = (const TX *)g.X;
    auto col_raw = [&](V (&raw)[2][4], int r) {  // P[b0+i, r, c] of the lane's four samples
        const uint32_t ro = (uint32_t)n0 * (uint32_t)r;
#pragma unroll
        for (int jp = 0; jp < 2; ++jp)
#pragma unroll
            for (int i = 0; i < 4; ++i)
                if (i <= d0) {
                    raw[jp][i].x = (T)to_f(P[pofs[2 * jp] + ro + i]);
                    raw[jp][i].y = (T)to_f(P[pofs[2 * jp + 1] + ro + i]);
                }
    };
    auto col_dot = [&](const V (&raw)[2][4], V (&y)[2]) {  // from zero, increasing i
#pragma unroll
        for (int jp = 0; jp < 2; ++jp) {
            V a = PT::zero();
#pragma unroll
            for (int i = 0; i < 4; ++i)
                if (i <= d0) a = PT::fma(sBw[(jp * 4 + i) * L + lane], raw[jp][i], a);
            y[jp] = a;
        }
    };
    const bool st0 = (CT ? 4 * lane : lane) < tl.a_len, st1 = lane + L < tl.a_len,
               st2 = lane + 2 * L < tl.a_len, st3 = lane + 3 * L < tl.a_len;
    T *erow = (T *)g.Y + ((uint32_t)ns0 * ((uint32_t)ns1 * (uint32_t)c + (uint32_t)tl.b_lo) +
                          (uint32_t)(tl.a_lo + (CT ? 4 * lane : lane)));
    V win[D1][2];  // win[k] = Y[., b + k, c] for the current support start b
    V nxt[2][4];   // control points of column b + D1, fetched one run ahead
    int bprev = -2;
    const T *__restrict__ B1 = (const T *)g.B1;
    for (int tb = 0; tb < tl.b_len; tb += L) {
        const int nb = (tl.b_len - tb) < L ? (tl.b_len - tb) : L;
        __syncwarp();
        if (lane < nb) {
            const int s = tl.b_lo + tb + lane;
            sb1[lane] = (int32_t)support_start(g.idx1[s], D1 - 1, n1);
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const T bb = i < D1 ? B1[s + ns1 * i] : T(0);
                sB1[lane * 4 + i] = PT::make(bb, bb);
            }
        }
        __syncwarp();
        for (int t = 0; t < nb; ++t) {
            const int b = sb1[t];
            if (b != bprev) {
                if (b == bprev + 1) {  // the window moves by one column: the fetched one joins
#pragma unroll
                    for (int k = 0; k + 1 < D1; ++k)
#pragma unroll
                        for (int jp = 0; jp < 2; ++jp) win[k][jp] = win[k + 1][jp];
                    V y[2];
                    col_dot(nxt, y);
                    win[D1 - 1][0] = y[0];
                    win[D1 - 1][1] = y[1];
                } else {  // first row or a jump: the whole window, column by column
#pragma unroll
                    for (int k = 0; k < D1; ++k) {
                        V raw[2][4];
                        col_raw(raw, b + k);
                        col_dot(raw, win[k]);
                    }
                }
                bprev = b;
                if (b + D1 < n1) col_raw(nxt, b + D1);
            }
            V a0 = PT::zero(), a1 = PT::zero();
#pragma unroll
            for (int k = 0; k < D1; ++k) {
                const V bv = sB1[t * 4 + k];
                a0 = PT::fma(bv, win[k][0], a0);
                a1 = PT::fma(bv, win[k][1], a1);
            }
            if constexpr (CT) {  // four consecutive samples: one 16-byte store
                if (st0) __stcs(reinterpret_cast<float4 *>(erow), make_float4(a0.x, a0.y, a1.x, a1.y));
            } else {
                if (st0) __stcs(erow, a0.x);
                if (st1) __stcs(erow + L, a0.y);
                if (st2) __stcs(erow + 2 * L, a1.x);
                if (st3) __stcs(erow + 3 * L, a1.y);
            }
            erow += ns0;
        }
    }
}

// ---------------------------------------------------------------------------------
// Adjoint tile: grad[c0, c1, c] = sum_{s0 in S0(c0)} B0[s0, c0 - b0(s0)] Z[s0, c1, c],
//               Z[s0, c1, c]   = sum_{s1 in S1(c1)} B1[s1, c1 - b1(s1)] Ebar[s0, s1, c],
// S_k(c) = the samples whose support contains control point c, in increasing order.
// The tile spans axis 0 whole (all samples, all control points) for channels
// [c_lo, c_lo + G) and the axis-1 control points [b_lo, b_lo + b_len).
//
// Phase A streams the cotangent rows that touch the block through a ring of kF2NS
// stages of kF2Rows rows.  In a stage, a channel's rows are consecutive in memory, so
// the producer warp moves each channel's part with ONE bulk copy (cp.async.bulk, the
// untiled TMA form; its 16-byte-aligned superset) and its lanes stage the stage's
// axis-1 basis rows and the channels' segment offsets beside it.  Stages complete on
// `full` mbarriers (transaction bytes + the producer's arrival); each consumer warp
// releases a stage on an `empty` mbarrier.  Consumer thread t owns the (sample,
// channel) pairs t + 256 j and keeps d1+1 rolling accumulators per pair.
// Phase B (every kF2Half finished columns, consumers only, on a named barrier): one
// output (column, c0, channel) per thread and step, its axis-0 samples summed in
// increasing order: acc = fma(B0[s, c0 - b0(s)], Z[s, column, channel], acc) from zero.
// The weights B0[s, c0 - b0(s)] are staged once per tile as a list in c0-major order
// (off0[c0] + s - lb0[c0]), so a term is two consecutive shared-memory reads.
//
// Every wait is bounded (sg_mbar.cuh); a wait that gives up records SG_ERR_TIMEOUT in
// *status and sets the CTA's abort flag, after which every later wait returns at once,
// the tile's results are invalid, and the CTA drains its copies in flight and stops.
// gstage counts stages across the tiles a CTA runs (the barriers' phases continue).
// Returns false when the CTA must stop.
// ---------------------------------------------------------------------------------
template <typename T>
struct F2AdjSmem {
    uint64_t *full, *empty;
    volatile int *abort;
    unsigned char *hdr;  // [kF2NS][f2_adj_hdr_bytes]
    T *ring;             // [kF2NS][f2_stage_elems]
    T *Zs;               // [kF2Ring][zstride]
    T *W0;               // [4 NP]: the axis-0 weights B0[s, c0 - b0(s)], c0-major, s increasing
    __device__ explicit F2AdjSmem(unsigned char *smem) {
        full = reinterpret_cast<uint64_t *>(smem);
        empty = full + kF2NS;
        abort = reinterpret_cast<volatile int *>(smem + kF2BarBytes);
        hdr = smem + kF2BarBytes + 16;
        ring = reinterpret_cast<T *>(hdr + kF2NS * f2_adj_hdr_bytes<T>());
        Zs = ring + kF2NS * (align16((int64_t)f2_stage_elems<T>() * sizeof(T)) / (int64_t)sizeof(T));
        W0 = reinterpret_cast<T *>(reinterpret_cast<unsigned char *>(Zs) +
                                   align16((int64_t)kF2Ring * f2_zstride<T>() * sizeof(T)));
    }
    template <typename V>
    __device__ V *hB(int slot) { return reinterpret_cast<V *>(hdr + slot * f2_adj_hdr_bytes<T>()); }
    __device__ int32_t *hb(int slot) {
        return reinterpret_cast<int32_t *>(hdr + slot * f2_adj_hdr_bytes<T>() +
                                           align16((int64_t)kF2Rows * 4 * 2 * sizeof(T)));
    }
    __device__ int32_t *hseg(int slot) {
        return reinterpret_cast<int32_t *>(hdr + slot * f2_adj_hdr_bytes<T>() +
                                           align16((int64_t)kF2Rows * 4 * 2 * sizeof(T)) + align16(kF2Rows * 4));
    }
};

// once per CTA (thread 0, before a CTA barrier)
template <typename T>
__device__ __forceinline__ void f2_adj_init(unsigned char *smem) {
    F2AdjSmem<T> sm(smem);
    for (int i = 0; i < kF2NS; ++i) {
        mbar_init(&sm.full[i], 1);
        mbar_init(&sm.empty[i], kF2Consumers);
    }
    *sm.abort = 0;
    mbar_init_fence();
}

// Test hooks of the adjoint's bounded waits (set from the host, tests only): the
// consumers' wait budget in SM cycles, and a flag that makes the producer withhold its
// arrival on the first stage of every CTA, so that stage never completes and the
// consumers' waits run out.  One copy per translation unit; the kernels that read them
// are in sg_fused2d.cu, which also sets them.
static __device__ long long g_f2_wait_cycles = kMbarWaitCycles;
static __device__ int g_f2_withhold_first_stage = 0;

// consumer-only barrier (named barrier 1; the producer warp never takes part)
__device__ __forceinline__ void f2_consumer_sync() {
    asm volatile("bar.sync 1, %0;\n" ::"r"(32 * kF2Consumers) : "memory");
}

template <typename T, int D1>
__device__ __forceinline__ bool f2_adjoint_tile(const F2Grid &g, const F2Tile &tl, unsigned char *smem,
                                             uint32_t &gstage, int *status) {
    using PT = F2Pair<T>;
    using V = typename PT::V;
    constexpr int NC = 32 * kF2Consumers;
    constexpr int J = f2_j<T>();
    constexpr int JP = J / 2;
    constexpr int ZS = f2_zstride<T>();
    constexpr int R = kF2Ring;
    constexpr int H = kF2Half;
    constexpr int NS = kF2NS;
    constexpr int SR = kF2Rows;
    constexpr int ES = (int)sizeof(T);
    constexpr int64_t STAGE = align16((int64_t)f2_stage_elems<T>() * ES) / ES;
    constexpr int d1 = D1 - 1;
    static_assert(J % 2 == 0, "pairs per thread come in couples");
    F2AdjSmem<T> sm(smem);
    const int tid = threadIdx.x;
    const int warp = tid >> 5, lane = tid & 31;
    const int d0 = g.d0;
    const int ns0 = (int)g.ns0, ns1 = (int)g.ns1, n0 = (int)g.n0, n1 = (int)g.n1;
    const int C1a = tl.b_lo, K1 = tl.b_len, G = tl.G;
    const int s1lo = g.lb1[C1a], s1hi = g.lb1[C1a + K1 + d1];
    const int nst = (s1hi - s1lo + SR - 1) / SR;
    const int seg = f2_seg_elems(ns0, ES);  // elements per channel segment of a stage
    const T *__restrict__ X = (const T *)g.X;
    // axis-0 samples of the tile: those whose support meets [a_lo, a_lo + a_len).  The
    // whole axis: a channel's rows are consecutive, one copy per channel (any G).  A
    // chunk (G = 1; rows of 16-byte multiples): one copy per row, at row stride rs.
    const int C0a = tl.a_lo, K0 = tl.a_len;
    const int s0lo = g.lb0[C0a], w0 = g.lb0[C0a + K0 + d0] - s0lo;
    const bool chunk = w0 != ns0;
    const int rs = chunk ? ((w0 + 2 * (16 / ES) - 1) / (16 / ES)) * (16 / ES) : ns0;

    if (warp == kF2Consumers) {
        // ------------------------------------------------------------- producer
        const T *__restrict__ B1 = (const T *)g.B1;
        const uintptr_t lim = (uintptr_t)(X + (int64_t)ns0 * ns1 * g.nch) & ~(uintptr_t)15;
        const int withhold = g_f2_withhold_first_stage;
        uint32_t gs = gstage;
        int issued = 0;
        // Header rows (support start, basis values) come 32 at a time, one per lane: batch
        // k covers stages 8k .. 8k+7 and is fetched while batch k-1 is in use, so no
        // stage waits for a load of its header.
        constexpr int QB = 32 / SR;  // stages per header batch
        int32_t h_b = 0, n_b = 0;
        T h_v[D1], n_v[D1];
#pragma unroll
        for (int i = 0; i < D1; ++i) h_v[i] = n_v[i] = T(0);
        auto fetch = [&](int k, int32_t &fb, T (&fv)[D1]) {  // rows of batch k, row `lane`
            const int s = s1lo + k * 32 + lane;
            if (s < s1hi) {
                fb = (int32_t)support_start(g.idx1[s], d1, n1);
#pragma unroll
                for (int i = 0; i < D1; ++i) fv[i] = B1[s + ns1 * i];
            }
        };
        fetch(0, h_b, h_v);
        fetch(1, n_b, n_v);
        for (int q = 0; q < nst; ++q, ++gs) {
            const int slot = (int)(gs % NS);
            const uint32_t use = gs / NS;
            int ok = 1;
            if (lane == 0 && use > 0) ok = mbar_wait(&sm.empty[slot], (use - 1) & 1, sm.abort);
            ok = __shfl_sync(0xffffffffu, ok, 0);
            if (!ok) {
                if (lane == 0) {
                    atomicExch(status, SG_ERR_TIMEOUT);
                    *sm.abort = 1;
                }
                break;
            }
            const int r0 = s1lo + q * SR;
            const int nr = (s1hi - r0) < SR ? (s1hi - r0) : SR;
            T *dst = sm.ring + (int64_t)slot * STAGE;
            if (chunk) {  // one copy per row (lanes 0 .. nr-1), all with the row's 16-byte lead
                const uintptr_t a = (uintptr_t)(X + (uint32_t)ns0 * ((uint32_t)r0 + (uint32_t)ns1 *
                                                                     (uint32_t)tl.c_lo) + s0lo);
                const uintptr_t a0 = a & ~(uintptr_t)15;
                const unsigned bytes = (unsigned)(((a - a0) + (uintptr_t)w0 * ES + 15) & ~(uintptr_t)15);
                if (lane < nr) {  // each lane adds its row's bytes before issuing its copy
                    const uintptr_t ra0 = a0 + (uintptr_t)lane * ns0 * ES;
                    const uintptr_t re = ra0 + (a - a0) + (uintptr_t)w0 * ES;
                    uintptr_t re16 = ra0 + bytes;
                    T *d = dst + lane * rs;
                    if (re16 > lim) {  // the array's last bytes: past its last 16-byte boundary
                        re16 = lim > ra0 ? lim : ra0;
                        T *dt = d + (int)((re16 - ra0) / ES);
                        for (uintptr_t p = re16; p < re; p += ES) *dt++ = *reinterpret_cast<const T *>(p);
                    }
                    mbar_expect_tx(&sm.full[slot], (unsigned)(re16 - ra0));
                    if (re16 > ra0) bulk_g2s(d, (const void *)ra0, (unsigned)(re16 - ra0), &sm.full[slot]);
                }
                if (lane == 0) sm.hseg(slot)[0] = (int)((a - a0) / ES);
            } else if (lane < G) {  // the copies first: they are the long pole; one per lane
                const int c = lane;     // (channel c's rows are consecutive in memory)
                const uintptr_t a = (uintptr_t)(X + (uint32_t)ns0 * ((uint32_t)r0 + (uint32_t)ns1 *
                                                                     (uint32_t)(tl.c_lo + c)));
                const uintptr_t a0 = a & ~(uintptr_t)15;
                const uintptr_t e = a + (uintptr_t)nr * ns0 * ES;
                uintptr_t e16 = (e + 15) & ~(uintptr_t)15;
                if (e16 > lim) {  // the array's last bytes: past its last 16-byte boundary
                    e16 = lim > a0 ? lim : a0;
                    T *d = dst + c * seg + (int)((e16 - a0) / ES);
                    for (uintptr_t p = e16; p < e; p += ES) *d++ = *reinterpret_cast<const T *>(p);
                }
                mbar_expect_tx(&sm.full[slot], (unsigned)(e16 - a0));  // before the copy it counts
                if (e16 > a0) bulk_g2s(dst + c * seg, (const void *)a0, (unsigned)(e16 - a0), &sm.full[slot]);
            }
            {  // the stage's axis-1 basis rows and support starts: lanes 4(q % 8) .. + 3
                const int j = lane - SR * (q % QB);
                if (j >= 0 && j < nr) {
                    sm.hb(slot)[j] = h_b;
                    Pack<T, 4> hv;  // the row's basis values, one 16-byte (Float64: 32-byte) entry
#pragma unroll
                    for (int i = 0; i < 4; ++i) hv.v[i] = i < D1 ? h_v[i < D1 ? i : 0] : T(0);
                    stp<T, 4>(sm.template hB<T>(slot) + j * 4, hv);
                }
            }
            if (!chunk && lane < G) {  // channel `lane`: its segment's base (element of sample 0)
                const uintptr_t a = (uintptr_t)(X + (uint32_t)ns0 * ((uint32_t)r0 + (uint32_t)ns1 *
                                                                     (uint32_t)(tl.c_lo + lane)));
                sm.hseg(slot)[lane] = lane * seg + (int)((a & 15) / ES);
            }
            __syncwarp();
            // publishes the header with the data (a test hook can withhold the CTA's first
            // stage, which then never completes)
            if (lane == 0 && !(withhold && gs == 0)) mbar_arrive(&sm.full[slot]);
            if (q % QB == QB - 1) {  // the next batch becomes current; fetch the one after it
                h_b = n_b;
#pragma unroll
                for (int i = 0; i < D1; ++i) h_v[i] = n_v[i];
                fetch(q / QB + 2, n_b, n_v);
            }
            ++issued;
        }
        // drain: the copies of the last stages have landed before the shared memory is
        // reused (bounded by time alone: after an abort the consumers no longer wait)
        if (lane == 0) {
            for (int k = 0; k < issued && k < NS; ++k) {
                const uint32_t gk = gs - 1 - k;
                const long long t0 = clock64();
                while (!mbar_try_wait(&sm.full[gk % NS], (gk / NS) & 1) && clock64() - t0 < kMbarWaitCycles) {
                }
            }
        }
        gstage += nst;
        return *sm.abort == 0;
    }

    // ----------------------------------------------------------------- consumers
    const int32_t *__restrict__ lb0 = g.lb0;
    const int32_t *__restrict__ off0 = g.off0;
    const int ob = off0[C0a];
    {  // the weight list: control point c0's weights at off0[c0] - off0[a_lo] + (s - lb0[c0])
        const T *__restrict__ B0 = (const T *)g.B0;
        for (int s = s0lo + tid; s < s0lo + w0; s += NC) {
            const int b0 = (int)support_start(g.idx0[s], d0, n0);
            for (int i = 0; i <= d0; ++i) {
                const int c0 = b0 + i;
                if (c0 >= C0a && c0 < C0a + K0) sm.W0[off0[c0] - ob + (s - lb0[c0])] = B0[s + ns0 * i];
            }
        }
    }
    const int npairs = w0 * G;
    int pofs[J];  // sample (relative to the tile's first) + channel segment of each pair
    int pcl[J];
#pragma unroll
    for (int j = 0; j < J; ++j) {
        const int p = tid + NC * j;
        pcl[j] = p < npairs ? p / w0 : 0;
        pofs[j] = p < npairs ? p % w0 : 0;
    }
    // Phase B of a finished half (ring columns pb_col0 .. + pb_nc - 1) is pending from the
    // half's barrier until the next one: each consumer thread takes its items a few at
    // a time between the stages of the next half, so the ring keeps flowing, and
    // finishes them before that barrier (after it, the next half's flushes overwrite
    // the columns).  Work item: (column pair, c0, channel), the pair fastest; a pair's
    // two outputs share every weight load and run as one packed FMA chain (one output
    // when pb_nc is odd and the pair is the last).
    int pb_col0 = 0, pb_nc = 0, pb_np2 = 1, pb_o = 0, pb_n = 0;
    auto b_item = [&](int o) {
        const int slot0 = (pb_col0 - C1a) % R;
        const int hp = o % pb_np2;
        const int r2 = o / pb_np2;
        const int c0 = C0a + r2 % K0;
        const int cl = r2 / K0;
        const int sb = lb0[c0];
        const int m = lb0[c0 + 1 + d0] - sb;
        const int h = 2 * hp;
        const T *zc = sm.Zs + (slot0 + h) * ZS + w0 * cl + (sb - s0lo);
        const T *w = sm.W0 + (off0[c0] - ob);
        T *yo = (T *)g.Y + ((uint32_t)c0 + (uint32_t)n0 * ((uint32_t)(pb_col0 + h) + (uint32_t)n1 *
                                                            (uint32_t)(tl.c_lo + cl)));
        if (h + 1 < pb_nc) {
            V a = PT::zero();
            for (int k = 0; k < m; ++k) a = PT::fma(PT::make(w[k], w[k]), PT::make(zc[k], zc[k + ZS]), a);
            yo[0] = a.x;  // increasing s, from zero, for both columns
            yo[n0] = a.y;
        } else {
            T a = T(0);
            for (int k = 0; k < m; ++k) a = ::fma(w[k], zc[k], a);
            yo[0] = a;
        }
    };
    auto b_some = [&](int cnt) {
        for (int i = 0; i < cnt && pb_o < pb_n; ++i, pb_o += NC) b_item(pb_o);
    };
    V acc[D1][JP];  // acc[k]: axis-1 control point cur + k
#pragma unroll
    for (int k = 0; k < D1; ++k)
#pragma unroll
        for (int jp = 0; jp < JP; ++jp) acc[k][jp] = PT::zero();
    int cur = C1a - d1;
    const int cend = C1a + K1;
    // control point `cur` is complete: into the ring (when in the block), then phase B
    // once a half of the ring is full or the block ends
    auto flush = [&]() {
        if (cur >= C1a) {
            T *z = sm.Zs + ((cur - C1a) % R) * ZS + tid;
#pragma unroll
            for (int jp = 0; jp < JP; ++jp) {
                z[NC * (2 * jp)] = acc[0][jp].x;
                z[NC * (2 * jp + 1)] = acc[0][jp].y;
            }
        }
#pragma unroll
        for (int k = 0; k + 1 < D1; ++k)
#pragma unroll
            for (int jp = 0; jp < JP; ++jp) acc[k][jp] = acc[k + 1][jp];
#pragma unroll
        for (int jp = 0; jp < JP; ++jp) acc[D1 - 1][jp] = PT::zero();
        if (cur >= C1a && ((cur - C1a) % H == H - 1 || cur == cend - 1)) {
            b_some(1 << 30);  // the previous half: the rest of this thread's items
            f2_consumer_sync();
            pb_col0 = cur - (cur - C1a) % H;
            pb_nc = cur - pb_col0 + 1;
            pb_np2 = (pb_nc + 1) >> 1;
            pb_n = K0 * pb_np2 * G;
            pb_o = tid;
        }
        ++cur;
    };
    uint32_t gs = gstage;
    const long long budget = g_f2_wait_cycles;
    for (int q = 0; q < nst; ++q, ++gs) {
        const int slot = (int)(gs % NS);
        // A stage whose wait gave up is skipped whole by the warp (its header may never
        // have been written, so nothing of it is read); the flushes below catch up, so
        // every consumer warp still reaches the same number of named barriers and the
        // tile's writes stay inside its block.
        if (!__all_sync(0xffffffffu, mbar_wait_for(&sm.full[slot], (gs / NS) & 1, sm.abort, budget))) {
            if (lane == 0 && !*sm.abort) {
                atomicExch(status, SG_ERR_TIMEOUT);
                *sm.abort = 1;
            }
            continue;
        }
        const int r0 = s1lo + q * SR;
        const int nr = (s1hi - r0) < SR ? (s1hi - r0) : SR;
        const T *base = sm.ring + (int64_t)slot * STAGE;
        const int32_t *hseg = sm.hseg(slot);
        const T *xp[J];
#pragma unroll
        for (int j = 0; j < J; ++j) xp[j] = base + hseg[pcl[j]] + pofs[j];
        const T *hB = sm.template hB<T>(slot);
        const int32_t *hb = sm.hb(slot);
        for (int u = 0; u < nr; ++u) {
            const int b = hb[u];
            while (cur < b) flush();
            V x[JP];
#pragma unroll
            for (int jp = 0; jp < JP; ++jp) x[jp] = PT::make(xp[2 * jp][u * rs], xp[2 * jp + 1][u * rs]);
            const Pack<T, 4> hv = ldp<T, 4>(hB + u * 4);  // one load for the row's basis values
#pragma unroll
            for (int k = 0; k < D1; ++k) {
                const V bv = PT::make(hv.v[k], hv.v[k]);
#pragma unroll
                for (int jp = 0; jp < JP; ++jp) acc[k][jp] = PT::fma(bv, x[jp], acc[k][jp]);
            }
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&sm.empty[slot]);
        b_some(kF2PhaseBPerStage);
    }
    if (nst == 0) f2_consumer_sync();  // the staged axis-0 rows are complete before phase B
    while (cur < cend) flush();
    b_some(1 << 30);  // the last half
    gstage += nst;
    return *sm.abort == 0;
}

// ---------------------------------------------------------------------------------
// Forward tile (axis-1 samples sorted): one CTA computes eval[s0, s1, c] for 128
// samples s0 of axis 0 and a block of rows s1, in two phases.
//   Phase 1: Y[s0, r, c] = sum_i B0[s0, i] P[b0(s0)+i, r, c] for the block's columns
//            r in [b1(first row), b1(last row) + d1] into shared memory (one thread per
//            (sample, column), from zero in increasing i -- the separable axis-0 pass).
//   Phase 2: warp w takes a contiguous run of the block's rows; per row
//            eval = sum_k B1[s1, k] Y[s0, b1(s1)+k, c] from zero in increasing k (the
//            separable last pass), each lane four samples whose d1+1 Y columns it keeps
//            in registers (one column read from the tile per move of the support
//            start), stored as one 16-byte access (Float32 rows of 16-byte multiples,
//            CT) or as four 4-byte accesses of the warp-strided samples.
// So every value takes the separable passes' operations in their order (bitwise the
// same results), the intermediate never leaves shared memory, and a row costs the warp
// d1+1 shared loads per value group, the packed FMAs and one store.  The host sizes the
// row blocks so that their columns fit kF2TileCols<T>().
// ---------------------------------------------------------------------------------
constexpr int kF2TileS0 = 128;     // samples of axis 0 per forward tile
constexpr int kF2TileWarps = 8;    // warps (phase-2 row strides) per forward tile
constexpr int kF2TileRows = 512;   // rows of axis 1 per forward tile at most
template <typename T>
__host__ __device__ constexpr int kF2TileCols() { return sizeof(T) == 4 ? 64 : 32; }
template <typename T>
__host__ __device__ constexpr int64_t f2_tile_smem() {
    return (int64_t)kF2TileCols<T>() * kF2TileS0 * sizeof(T)  // Y tile
           + (int64_t)kF2TileRows * 4 * sizeof(T)             // the rows' axis-1 basis values
           + (int64_t)kF2TileRows * 4;                        // the rows' Y offsets
}

// Phase 1 of a forward tile for axis-0 degree D0 - 1: the Y tile's columns [cb, ce) of
// sample sl (stored at the lane-major position `pos` that phase 2 reads), four columns
// per step so that their loads are in flight together.
template <typename T, typename TX, int D0>
__device__ __forceinline__ void f2_tile_phase1(const F2Grid &g, const F2Tile &tl, T *Ys, int sl, int pos,
                                               int cb, int ce, int col0, int cstep) {
    const int ns0 = (int)g.ns0, n0 = (int)g.n0, n1 = (int)g.n1;
    const T *__restrict__ B0 = (const T *)g.B0;
    const TX *__restrict__ P = (const TX *)g.X;
    const int s0 = tl.a_lo + sl;
    const int b0 = (int)support_start(g.idx0[s0], D0 - 1, n0);
    T bw[D0];
#pragma unroll
    for (int i = 0; i < D0; ++i) bw[i] = B0[s0 + ns0 * i];
    const TX *pb = P + ((uint32_t)b0 + (uint32_t)n0 * (uint32_t)n1 * (uint32_t)tl.c_lo);
    for (int col = col0; col < ce; col += 4 * cstep) {
        T raw[4][D0];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int cu = col + cstep * u < ce ? col + cstep * u : col;  // (a repeat of col past the end)
            const TX *pc = pb + (uint32_t)n0 * (uint32_t)cu;
#pragma unroll
            for (int i = 0; i < D0; ++i) raw[u][i] = (T)to_f(pc[i]);
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            T a = T(0);
#pragma unroll
            for (int i = 0; i < D0; ++i) a = ::fma(bw[i], raw[u][i], a);
            const int cu = col + cstep * u;
            if (cu < ce) Ys[(cu - cb) * kF2TileS0 + pos] = a;
        }
    }
}

template <typename T, typename TX, int D1, bool CT>
__device__ __forceinline__ void f2_forward_tile(const F2Grid &g, const F2Tile &tl, unsigned char *smem) {
    using PT = F2Pair<T>;
    using V = typename PT::V;
    constexpr int L = kF2Lanes;
    constexpr int S = kF2TileS0;
    constexpr int NT = kF2TileWarps * 32;
    // Y tile [cols][S], lane-major: the value of the lane-l, v-th sample at col * S + 4 l + v
    // (samples 4 l + v when CT, else l + 32 v), so phase 2 reads a lane's four with one
    // 16-byte load either way
    T *Ys = reinterpret_cast<T *>(smem);
    T *hB1 = Ys + kF2TileCols<T>() * S;   // [rows][4]: B1[row, k]
    int32_t *hY = reinterpret_cast<int32_t *>(hB1 + kF2TileRows * 4);  // [rows]: (b1(row) - cb) * S
    const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
    const int ns0 = (int)g.ns0, ns1 = (int)g.ns1, n1 = (int)g.n1;
    const int c = tl.c_lo;
    // the block's columns: given by the unit list (the batch), else from the samples
    const int cb = tl.ncol > 0 ? tl.cb : (int)support_start(g.idx1[tl.b_lo], D1 - 1, n1);
    const int ce = tl.ncol > 0 ? tl.cb + tl.ncol
                               : (int)support_start(g.idx1[tl.b_lo + tl.b_len - 1], D1 - 1, n1) + D1;
    if (ce - cb > kF2TileCols<T>() || ce <= cb || tl.b_len > kF2TileRows) return;  // (ruled out by the host)
    {  // phase 1: the rows' headers, then the Y tile
        const T *__restrict__ B1 = (const T *)g.B1;
        for (int j = tid; j < tl.b_len; j += NT) {
            const int r = tl.b_lo + j;
            hY[j] = ((int32_t)support_start(g.idx1[r], D1 - 1, n1) - cb) * S;
#pragma unroll
            for (int k = 0; k < 4; ++k) hB1[j * 4 + k] = k < D1 ? B1[r + ns1 * k] : T(0);
        }
        const int sl = tid & (S - 1);
        if (sl < tl.a_len) {
            const int pos = CT ? sl : (sl & 31) * 4 + (sl >> 5);
            const int col0 = cb + tid / S;
            constexpr int CS = NT / S;
            switch (g.d0) {
                case 0: f2_tile_phase1<T, TX, 1>(g, tl, Ys, sl, pos, cb, ce, col0, CS); break;
                case 1: f2_tile_phase1<T, TX, 2>(g, tl, Ys, sl, pos, cb, ce, col0, CS); break;
                case 2: f2_tile_phase1<T, TX, 3>(g, tl, Ys, sl, pos, cb, ce, col0, CS); break;
                default: f2_tile_phase1<T, TX, 4>(g, tl, Ys, sl, pos, cb, ce, col0, CS); break;
            }
        }
    }
    __syncthreads();
    // phase 2: warp w takes a contiguous run of rows and keeps the Y columns of the
    // current support start (its lanes' four samples each) in registers, reading a
    // column from the tile only when the support start moves (shared-memory traffic
    // per row: the basis values and nothing else on most rows)
    const int kw = (tl.b_len + kF2TileWarps - 1) / kF2TileWarps;
    const int j0 = w * kw, j1 = (j0 + kw) < tl.b_len ? (j0 + kw) : tl.b_len;
    if (j0 >= j1) return;
    const bool st0 = (CT ? 4 * lane : lane) < tl.a_len, st1 = lane + L < tl.a_len,
               st2 = lane + 2 * L < tl.a_len, st3 = lane + 3 * L < tl.a_len;
    T *erow = (T *)g.Y + ((uint32_t)ns0 * ((uint32_t)ns1 * (uint32_t)c + (uint32_t)(tl.b_lo + j0)) +
                          (uint32_t)(tl.a_lo + (CT ? 4 * lane : lane)));
    const T *ylane = Ys + 4 * lane;
    V win[D1][2];  // win[k]: Y at column b + k of the lane's four samples (two pairs)
    int bcur = -2 * S;
    for (int j = j0; j < j1; ++j, erow += ns0) {
        const int bo = hY[j];
        if (bo != bcur) {
            if (bo == bcur + S) {  // the support start moved by one: one new column
#pragma unroll
                for (int k = 0; k + 1 < D1; ++k) {
                    win[k][0] = win[k + 1][0];
                    win[k][1] = win[k + 1][1];
                }
                const Pack<T, 4> y = ldp<T, 4>(ylane + bo + (D1 - 1) * S);
                win[D1 - 1][0] = PT::make(y.v[0], y.v[1]);
                win[D1 - 1][1] = PT::make(y.v[2], y.v[3]);
            } else {
#pragma unroll
                for (int k = 0; k < D1; ++k) {
                    const Pack<T, 4> y = ldp<T, 4>(ylane + bo + k * S);
                    win[k][0] = PT::make(y.v[0], y.v[1]);
                    win[k][1] = PT::make(y.v[2], y.v[3]);
                }
            }
            bcur = bo;
        }
        const T *bj = hB1 + j * 4;
        V a0 = PT::zero(), a1 = PT::zero();
#pragma unroll
        for (int k = 0; k < D1; ++k) {
            const V bv = PT::make(bj[k], bj[k]);
            a0 = PT::fma(bv, win[k][0], a0);
            a1 = PT::fma(bv, win[k][1], a1);
        }
        if constexpr (CT) {
            if (st0) __stcs(reinterpret_cast<float4 *>(erow), make_float4(a0.x, a0.y, a1.x, a1.y));
        } else {
            if (st0) __stcs(erow, a0.x);
            if (st1) __stcs(erow + L, a0.y);
            if (st2) __stcs(erow + 2 * L, a1.x);
            if (st3) __stcs(erow + 3 * L, a1.y);
        }
    }
}

template <typename T, typename TX>
__device__ __forceinline__ void f2_run_forward_tile(const F2Grid &g, const F2Tile &tl, unsigned char *smem) {
    bool ct = false;
    if constexpr (sizeof(T) == 4) ct = (g.ns0 & 3) == 0 && ((uintptr_t)g.Y & 15) == 0;
#define SG_F2_TILE(D)                                                   \
    if (ct) {                                                           \
        if constexpr (sizeof(T) == 4) f2_forward_tile<T, TX, D, true>(g, tl, smem); \
    } else {                                                            \
        f2_forward_tile<T, TX, D, false>(g, tl, smem);                  \
    }
    switch (g.d1) {
        case 0: SG_F2_TILE(1) break;
        case 1: SG_F2_TILE(2) break;
        case 2: SG_F2_TILE(3) break;
        default: SG_F2_TILE(4) break;
    }
#undef SG_F2_TILE
}

// Float64 warp tasks are compiled out of line (each degree with its own register
// allocation); Float32 ones inline, where the shared-memory accesses are known as such.
template <typename T, typename TX, int D1>
__device__ __noinline__ void f2_forward_warp_call(const F2Grid &g, const F2Tile &tl, unsigned char *wsm) {
    f2_forward_warp<T, TX, D1>(g, tl, wsm);
}
template <typename T, typename TX, int D1>
__device__ __forceinline__ void f2_forward_d(const F2Grid &g, const F2Tile &tl, unsigned char *wsm) {
    if constexpr (sizeof(T) == 8) f2_forward_warp_call<T, TX, D1>(g, tl, wsm);
    else f2_forward_warp<T, TX, D1>(g, tl, wsm);
}

// Dispatch by the axis-1 degree (the axis-0 degree is a runtime bound <= 3).
template <typename T, typename TX>
__device__ __forceinline__ void f2_run_forward(const F2Grid &g, const F2Tile &tl, unsigned char *wsm) {
    if constexpr (sizeof(T) == 4) {
        // rows of 16-byte multiples in a 16-byte aligned eval: lanes own four consecutive
        // samples and store them at once (tasks start at multiples of 128 samples)
        if ((g.ns0 & 3) == 0 && ((uintptr_t)g.Y & 15) == 0) {
            switch (g.d1) {
                case 0: f2_forward_warp<T, TX, 1, true>(g, tl, wsm); break;
                case 1: f2_forward_warp<T, TX, 2, true>(g, tl, wsm); break;
                case 2: f2_forward_warp<T, TX, 3, true>(g, tl, wsm); break;
                default: f2_forward_warp<T, TX, 4, true>(g, tl, wsm); break;
            }
            return;
        }
    }
    switch (g.d1) {
        case 0: f2_forward_d<T, TX, 1>(g, tl, wsm); break;
        case 1: f2_forward_d<T, TX, 2>(g, tl, wsm); break;
        case 2: f2_forward_d<T, TX, 3>(g, tl, wsm); break;
        default: f2_forward_d<T, TX, 4>(g, tl, wsm); break;
    }
}
template <typename T>
__device__ __forceinline__ bool f2_run_adjoint(const F2Grid &g, const F2Tile &tl, unsigned char *smem,
                                               uint32_t &gstage, int *status) {
    switch (g.d1) {
        case 0: return f2_adjoint_tile<T, 1>(g, tl, smem, gstage, status);
        case 1: return f2_adjoint_tile<T, 2>(g, tl, smem, gstage, status);
        case 2: return f2_adjoint_tile<T, 3>(g, tl, smem, gstage, status);
        default: return f2_adjoint_tile<T, 4>(g, tl, smem, gstage, status);
    }
}

}  // namespace sg
