// sg_passes.cuh -- host launchers of the separable passes (instantiated per value type
// in sg_passes_f32.cu / sg_passes_f64.cu so the translation units build in parallel).
#pragma once

#include <type_traits>

#include "sg_contract.cuh"
#include "sg_warp.cuh"
#include "sg_stream.cuh"

namespace sg {

// One contraction pass over one input axis (see sg_contract.cuh for the index maps).
struct AxisPass {
    const int32_t *idx = nullptr;   // sample indices of the axis (1-based)
    const int32_t *perm = nullptr;  // sorted view of the samples, or NULL when sorted
    const int32_t *lb = nullptr;    // support table of the axis (adjoint), or NULL
    const void *B = nullptr;        // basis table block of the derivative order: B[j + ns*i]
    int64_t ns = 0;                 // samples along the axis
    int d = 0;                      // degree
    int64_t n = 0;                  // control points along the axis
    int64_t M = 1;                  // product of the axes before this one
    int64_t Q = 1;                  // product of the axes after (axis-0 kHomog: without channels)
    const void *X = nullptr;
    void *Y = nullptr;
    const void *w = nullptr;        // NURBS weights (axis-0 forward pass only)
    int nch = 0;                    // output channels (Nout)
    int mode = kPlain;
    bool final_pass = false;        // writes eval
    int x_dtype = SG_F32;           // element type of X on the axis-0 forward pass
    int *status = nullptr;          // device status word of bounded waits
    int cc = 0;                     // adjoint stream: control points per chunk (0: heuristic)
};

int fwd_axis0_f32(const AxisPass &p, cudaStream_t s);
int fwd_axis0_f64(const AxisPass &p, cudaStream_t s);
int fwd_axis_f32(const AxisPass &p, cudaStream_t s);
int fwd_axis_f64(const AxisPass &p, cudaStream_t s);
int adj_axis_f32(const AxisPass &p, cudaStream_t s);
int adj_axis_f64(const AxisPass &p, cudaStream_t s);
int adj_axis0_f32(const AxisPass &p, cudaStream_t s);
int adj_axis0_f64(const AxisPass &p, cudaStream_t s);

constexpr int64_t kMaxGridYZ = 65535;
constexpr int64_t kNumSMs = 152;                 // GB300
constexpr int64_t kTargetCtas = kNumSMs * 8;     // grid size aimed at by sized launches

inline unsigned gdim(int64_t v, int64_t cap) { return (unsigned)(v < 1 ? 1 : (v > cap ? cap : v)); }

template <typename T>
inline int vec_width(const AxisPass &p) {
    // 16-byte accesses along m need M to be a multiple of the vector width and all
    // base pointers 16-byte aligned (every row start is then aligned too).
    constexpr int V = 16 / (int)sizeof(T);
    const bool ok = (p.M % V == 0) && ((uintptr_t)p.X % 16 == 0) && ((uintptr_t)p.Y % 16 == 0);
    return ok ? V : 1;
}

// ------------------------------------------------------------------ forward axis 0
template <typename T, typename TX, int D, int MODE>
inline void launch_fwd_axis0_t(const AxisPass &p, cudaStream_t s) {
    const unsigned gx = (unsigned)((p.ns + kThreads - 1) / kThreads);
    int64_t Qy = (MODE == kHomog) ? p.Q * (p.nch + 1) : (MODE == kRational ? 1 : p.Q * p.nch);
    // each thread walks Qy/gridDim.y columns with its basis values in registers; size
    // grid.y for ~32 CTAs per SM (a few columns per thread: more loads in flight per SM)
    // rather than one output per thread
    const int64_t want_y = (kTargetCtas * 4 + gx - 1) / gx;
    dim3 grid(gx, gdim(Qy < want_y ? Qy : want_y, kMaxGridYZ));
    k_fwd_axis0<D, TX, T, MODE><<<grid, kThreads, 0, s>>>(
        p.idx, (const T *)p.B, p.ns, p.d, (const TX *)p.X, (const T *)p.w, p.n, p.Q, p.nch,
        (T *)p.Y);
}

template <typename T, typename TX, int MODE>
inline void launch_fwd_axis0_d(const AxisPass &p, cudaStream_t s) {
    switch (p.d) {
        case 0: launch_fwd_axis0_t<T, TX, 1, MODE>(p, s); break;
        case 1: launch_fwd_axis0_t<T, TX, 2, MODE>(p, s); break;
        case 2: launch_fwd_axis0_t<T, TX, 3, MODE>(p, s); break;
        case 3: launch_fwd_axis0_t<T, TX, 4, MODE>(p, s); break;
        default: launch_fwd_axis0_t<T, TX, 0, MODE>(p, s); break;
    }
}

// Warp tasks of the axis-0 passes: enough for ~16 warps per SM.
constexpr int64_t kAxis0Tasks = (int64_t)kNumSMs * 16;

// kPlain, degrees <= 3, same-type input: warp tasks of 32 columns x a chunk of samples
// (sg_warp.cuh); few columns get short chunks (at least 32 samples) so the tasks still
// fill the GPU
template <typename T, int D>
inline void launch_fwd0_warp(const AxisPass &p, cudaStream_t s) {
    const int64_t Qy = p.Q * p.nch;
    const int64_t groups = (Qy + 31) / 32;
    if (groups == 0 || p.ns == 0) return;
    const int64_t want = (kAxis0Tasks + groups - 1) / groups;  // sample chunks wanted
    int64_t SC = (p.ns + want - 1) / want;
    SC = SC < 32 ? 32 : SC;
    const int64_t tasks = groups * ((p.ns + SC - 1) / SC);
    const int64_t blocks = (tasks + kWarpsPerBlock - 1) / kWarpsPerBlock;
    k_fwd0_warp<D, T><<<(unsigned)blocks, 32 * kWarpsPerBlock, 0, s>>>(
        p.idx, (const T *)p.B, p.ns, p.d, (const T *)p.X, p.n, Qy, SC, (T *)p.Y);
}

template <typename T, typename TX>
inline void launch_fwd_axis0_m(const AxisPass &p, cudaStream_t s) {
    if constexpr (std::is_same<T, TX>::value) {
        // warp tasks when their columns alone fill the GPU; fewer columns run faster as
        // the CTA kernel (each thread keeps one sample's basis row for many columns)
        if (p.mode == kPlain && p.d <= 3 && (p.Q * p.nch + 31) / 32 >= kAxis0Tasks) {
            switch (p.d) {
                case 0: launch_fwd0_warp<T, 1>(p, s); return;
                case 1: launch_fwd0_warp<T, 2>(p, s); return;
                case 2: launch_fwd0_warp<T, 3>(p, s); return;
                default: launch_fwd0_warp<T, 4>(p, s); return;
            }
        }
    }
    if (p.mode == kPlain) launch_fwd_axis0_d<T, TX, kPlain>(p, s);
    else if (p.mode == kHomog) launch_fwd_axis0_d<T, TX, kHomog>(p, s);
    else launch_fwd_axis0_d<T, TX, kRational>(p, s);
}

// ------------------------------------------------------------------ forward axis k
template <typename T, int D, int VEC, int MODE, int NC, bool FINAL, bool ST>
inline void launch_fwd_axis_t(const AxisPass &p, cudaStream_t s) {
    const int64_t per_cta = (int64_t)kThreads * VEC;
    const unsigned gx = (unsigned)((p.M + per_cta - 1) / per_cta);
    const int64_t chunks = (p.ns + kChunk - 1) / kChunk;
    // grid.y addresses sample chunks; an axis longer than 65535 chunks is launched in
    // slices, each on bases shifted by the slice's first sample.
    for (int64_t c0 = 0; c0 < chunks; c0 += kMaxGridYZ) {
        const int64_t cn = (chunks - c0 < kMaxGridYZ) ? chunks - c0 : kMaxGridYZ;
        const int64_t jb = c0 * kChunk;
        const int64_t jcount = (p.ns - jb < cn * kChunk) ? p.ns - jb : cn * kChunk;
        dim3 grid(gx, (unsigned)cn, MODE == kRational ? 1u : gdim(p.Q, kMaxGridYZ));
        k_fwd_axis<D, T, VEC, MODE, NC, FINAL, ST><<<grid, kThreads, 0, s>>>(
            p.idx + jb, (const T *)p.B + jb, p.ns, jcount, p.d, (const T *)p.X, p.M, p.n, p.Q,
            p.nch, (T *)p.Y + p.M * jb);
    }
}

// kPlain passes of degree <= 3 run as warp tasks (sg_warp.cuh)
template <typename T, int D, bool ST, bool FINAL>
inline void launch_fwd_warp(const AxisPass &p, cudaStream_t s) {
    const int64_t gxw = (p.M + warp_width<T>() - 1) / warp_width<T>();
    const int64_t tasks = gxw * ((p.ns + kFwdGridRows - 1) / kFwdGridRows) * p.Q;
    const int64_t blocks = (tasks + kWarpsPerBlock - 1) / kWarpsPerBlock;
    if (blocks == 0) return;
    k_fwd_warp<D, T, ST, FINAL><<<(unsigned)blocks, 32 * kWarpsPerBlock, 0, s>>>(
        p.idx, (const T *)p.B, p.ns, p.d, (const T *)p.X, p.M, p.n, p.Q, gxw, (T *)p.Y);
}

template <typename T, int D, int VEC, bool ST>
inline void launch_fwd_axis_v(const AxisPass &p, cudaStream_t s) {
    if (p.mode == kRational) {
        if (p.nch + 1 <= 2) launch_fwd_axis_t<T, D, VEC, kRational, 2, true, ST>(p, s);
        else launch_fwd_axis_t<T, D, VEC, kRational, 4, true, ST>(p, s);
    } else if (p.final_pass) {
        launch_fwd_warp<T, D, ST, true>(p, s);
    } else {
        launch_fwd_warp<T, D, ST, false>(p, s);
    }
}

// aligned rows: contiguous 16-byte accesses; otherwise the same VEC values per thread
// strided by the block width
template <typename T, int D>
inline void launch_fwd_axis_d(const AxisPass &p, cudaStream_t s) {
    constexpr int V = 16 / (int)sizeof(T);
    if (vec_width<T>(p) == V) launch_fwd_axis_v<T, D, V, false>(p, s);
    else launch_fwd_axis_v<T, D, V, true>(p, s);
}

template <typename T>
inline void launch_fwd_axis(const AxisPass &p, cudaStream_t s) {
    if (p.mode == kRational && (p.nch + 1 > 4 || p.d > 3)) {
        dim3 grid((unsigned)((p.M + kThreads - 1) / kThreads), gdim(p.ns, kMaxGridYZ));
        k_fwd_axis_rational_generic<T><<<grid, kThreads, 0, s>>>(
            p.idx, (const T *)p.B, p.ns, p.d, (const T *)p.X, p.M, p.n, p.nch, (T *)p.Y);
        return;
    }
    switch (p.d) {
        case 0: launch_fwd_axis_d<T, 1>(p, s); break;
        case 1: launch_fwd_axis_d<T, 2>(p, s); break;
        case 2: launch_fwd_axis_d<T, 3>(p, s); break;
        case 3: launch_fwd_axis_d<T, 4>(p, s); break;
        default:  // any degree: runtime-degree kernel, scalar accesses
            if (p.final_pass) launch_fwd_axis_t<T, 0, 1, kPlain, 1, true, false>(p, s);
            else launch_fwd_axis_t<T, 0, 1, kPlain, 1, false, false>(p, s);
    }
}

// ------------------------------------------------------------------ adjoint axis k
template <typename T, int D, int VEC, bool ST>
inline void launch_adj_axis_t(const AxisPass &p, cudaStream_t s) {
    // Control points per CTA: as wide as possible (the halo of d knot spans shared
    // with the neighbour chunk is re-read) while the grid still gives every SM ~4 CTAs.
    const int64_t per_cta = (int64_t)kThreads * VEC;
    const unsigned gx = (unsigned)((p.M + per_cta - 1) / per_cta);
    const int64_t gz = p.Q < kMaxGridYZ ? p.Q : kMaxGridYZ;
    const int64_t want_chunks = (kNumSMs * 4 + gx * gz - 1) / (gx * gz);
    int64_t CC = (p.n + want_chunks - 1) / want_chunks;
    CC = CC < 8 ? 8 : (CC > 64 ? 64 : CC);
    if ((p.n + CC - 1) / CC > kMaxGridYZ) CC = (p.n + kMaxGridYZ - 1) / kMaxGridYZ;
    const int64_t chunks = (p.n + CC - 1) / CC;
    dim3 grid(gx, (unsigned)chunks, (unsigned)gz);
    const int smem = (int)adj_axis_smem_bytes<D, T, VEC>(kThreads);
    static bool attr_set = false;  // one instance per template instantiation
    if (!attr_set) {
        cudaFuncSetAttribute(k_adj_axis<D, T, VEC, ST>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             smem);
        attr_set = true;
    }
    k_adj_axis<D, T, VEC, ST><<<grid, kThreads, smem, s>>>(p.idx, p.perm, p.lb, (const T *)p.B, p.ns,
                                                     p.d, (const T *)p.X, p.M, p.n, p.Q, (int)CC,
                                                     (T *)p.Y);
}

// Warp tasks (sg_warp.cuh): chunks of CC control points, CC as wide as possible (the
// halo of d knot spans shared with the neighbour chunk is re-read) while the tasks
// still fill every SM with ~32 warps.
template <typename T, int D, bool ST>
inline void launch_adj_warp(const AxisPass &p, cudaStream_t s) {
    const int64_t gxw = (p.M + warp_width<T>() - 1) / warp_width<T>();
    const int64_t per_chunk = gxw * p.Q;  // tasks per chunk
    const int64_t want_chunks = (kNumSMs * 32 * 2 + per_chunk - 1) / per_chunk;
    int64_t CC = (p.n + want_chunks - 1) / want_chunks;
    CC = CC < 8 ? 8 : (CC > 64 ? 64 : CC);
    const int64_t chunks = (p.n + CC - 1) / CC;
    const int64_t blocks = (per_chunk * chunks + kWarpsPerBlock - 1) / kWarpsPerBlock;
    if (blocks == 0) return;
    k_adj_warp<D, T, ST><<<(unsigned)blocks, 32 * kWarpsPerBlock, 0, s>>>(
        p.idx, p.perm, p.lb, (const T *)p.B, p.ns, p.d, (const T *)p.X, p.M, p.n, p.Q, (int)CC, gxw,
        chunks, (T *)p.Y);
}

// Bulk-copy stream (sg_stream.cuh): tiles of up to stream_width<T>() values of m (all
// of M when it fits) x CC control points x one column; CC as wide as possible while
// the tiles still give every SM ~2 waves of resident CTAs.
// Stream tiles of an adjoint pass: m blocks x chunks of CC control points x columns.
// CC (8..64) is the largest chunk that still gives enough tiles: about 2.5 per SM when
// a chunk has few tiles (few columns: longer chunks re-read fewer halo rows), two per
// CTA slot when it has many (long m).
template <typename T>
inline int64_t stream_tiles(const AxisPass &p, int64_t &CC, int64_t &chunks) {
    constexpr int64_t W = stream_width<T>();
    const int64_t per_chunk = ((p.M + W - 1) / W) * p.Q;
    const int64_t target = per_chunk <= 64 ? 384 : kNumSMs * 3 * 2;
    const int64_t min_chunks = (target + per_chunk - 1) / per_chunk;
    CC = p.n / min_chunks;
    CC = CC < 8 ? 8 : (CC > 64 ? 64 : CC);
    if (p.cc > 0) CC = p.cc;  // measured by sg_grid_plan_tune
    chunks = (p.n + CC - 1) / CC;
    return per_chunk * chunks;
}

template <typename T, int D>
inline void launch_adj_stream(const AxisPass &p, cudaStream_t s) {
    constexpr int64_t W = stream_width<T>();
    const int64_t nmb = (p.M + W - 1) / W;
    const int64_t L = p.M < W ? p.M : W;
    int64_t CC = 0, chunks = 0;
    const int64_t tiles = stream_tiles<T>(p, CC, chunks);
    const int smem = (int)stream_smem_bytes<D, T>();
    static bool attr_set = false;  // one instance per template instantiation
    if (!attr_set) {
        cudaFuncSetAttribute(k_adj_stream<D, T>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        attr_set = true;
    }
    if (tiles == 0) return;
    k_adj_stream<D, T><<<(unsigned)tiles, kStreamThreads, smem, s>>>(
        p.idx, p.perm, p.lb, (const T *)p.B, p.ns, p.d, (const T *)p.X, p.M, p.n, p.Q, (int)CC, nmb,
        chunks, stream_rows_per_stage(L, (int)sizeof(T)), (T *)p.Y, p.status);
}

template <typename T, int D>
inline void launch_adj_axis_d(const AxisPass &p, cudaStream_t s) {
    constexpr int V = 16 / (int)sizeof(T);
    if constexpr (D == 0) {
        launch_adj_axis_t<T, D, 1, false>(p, s);  // runtime degree: one value a thread
    } else {
        // the stream needs a 16-byte aligned source; with fewer tiles than SMs (few
        // long columns, e.g. Nout = 1 on a large grid) the warp tasks spread wider
        int64_t CC = 0, chunks = 0;
        if ((uintptr_t)p.X % 16 == 0 && stream_tiles<T>(p, CC, chunks) >= kNumSMs)
            launch_adj_stream<T, D>(p, s);
        else if (vec_width<T>(p) == V) launch_adj_warp<T, D, false>(p, s);
        else launch_adj_warp<T, D, true>(p, s);
    }
}

template <typename T>
inline void launch_adj_axis(const AxisPass &p, cudaStream_t s) {
    switch (p.d) {
        case 0: launch_adj_axis_d<T, 1>(p, s); break;
        case 1: launch_adj_axis_d<T, 2>(p, s); break;
        case 2: launch_adj_axis_d<T, 3>(p, s); break;
        case 3: launch_adj_axis_d<T, 4>(p, s); break;
        default: launch_adj_axis_d<T, 0>(p, s); break;
    }
}

template <typename T, int D>
inline void launch_adj_axis0_t(const AxisPass &p, cudaStream_t s) {
    // QT columns x CT control points per CTA; few columns -> more control points
    const int QT = p.Q >= 32 ? 32 : (p.Q >= 16 ? 16 : (p.Q >= 8 ? 8 : (p.Q >= 4 ? 4 : (p.Q >= 2 ? 2 : 1))));
    const int CT = kAdj0Threads / QT;
    const int64_t gy = (p.Q + QT - 1) / QT;
    dim3 grid((unsigned)((p.n + CT - 1) / CT), gdim(gy, kMaxGridYZ));
    const size_t smem = (size_t)adj_axis0_smem_bytes<D, T>(QT);
    static bool attr_set = false;  // one instance per template instantiation
    if (!attr_set) {
        cudaFuncSetAttribute(k_adj_axis0<D, T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)adj_axis0_smem_bytes<D, T>(32));
        attr_set = true;
    }
    k_adj_axis0<D, T><<<grid, kAdj0Threads, smem, s>>>(p.idx, p.perm, p.lb, (const T *)p.B,
                                                       p.ns, p.d, (const T *)p.X, p.n, p.Q, QT,
                                                       (T *)p.Y);
}

// degrees <= 3: warp tasks of 32 columns x a chunk of control points (sg_warp.cuh);
// few columns get short chunks (at least 4 control points) so the tasks fill the GPU
template <typename T, int D>
inline void launch_adj0_warp(const AxisPass &p, cudaStream_t s) {
    const int64_t groups = (p.Q + 31) / 32;
    if (groups == 0 || p.n == 0) return;
    const int64_t want = (kAxis0Tasks + groups - 1) / groups;  // chunks wanted
    int64_t CC = (p.n + want - 1) / want;
    CC = CC < 4 ? 4 : CC;
    const int64_t tasks = groups * ((p.n + CC - 1) / CC);
    const int64_t blocks = (tasks + kWarpsPerBlock - 1) / kWarpsPerBlock;
    const int smem = kWarpsPerBlock * warp_adj0_smem<D, T>();
    static bool attr_set = false;  // one instance per template instantiation
    if (!attr_set) {
        cudaFuncSetAttribute(k_adj0_warp<D, T>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        attr_set = true;
    }
    if (blocks == 0) return;
    k_adj0_warp<D, T><<<(unsigned)blocks, 32 * kWarpsPerBlock, smem, s>>>(
        p.idx, p.perm, p.lb, (const T *)p.B, p.ns, p.d, (const T *)p.X, p.n, p.Q, CC, (T *)p.Y);
}

// Degrees <= 3 run as warp tasks; other degrees (runtime-degree path) as CTA tiles.
template <typename T>
inline void launch_adj_axis0(const AxisPass &p, cudaStream_t s) {
    switch (p.d) {
        case 0: launch_adj0_warp<T, 1>(p, s); break;
        case 1: launch_adj0_warp<T, 2>(p, s); break;
        case 2: launch_adj0_warp<T, 3>(p, s); break;
        case 3: launch_adj0_warp<T, 4>(p, s); break;
        default: launch_adj_axis0_t<T, 0>(p, s); break;
    }
}

}  // namespace sg
