// sg_fused2d.cu -- kernels, tiling and launchers of the fused Nin = 2 path
// (sg_fused2d.cuh): one launch per evaluate! / evaluate_adjoint! of a 2D grid, and the
// batch kernels that run the fused units of many 2D grids.
#include <algorithm>
#include <cmath>

#include "sg_fused2d_host.h"

namespace sg {

static int64_t cdiv(int64_t a, int64_t b) { return (a + b - 1) / b; }

// ------------------------------------------------------------------ kernels
// One grid, forward: warp w of block x runs warp task 8x + w of the uniform tiling.
template <typename T, typename TX>
__global__ void __launch_bounds__(kF2Lanes * kF2FwdWarps, 3)
k_f2_fwd_grid(F2Grid g, F2Tiling tiling) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ F2Grid s_g;
    if (threadIdx.x == 0) s_g = g;
    __syncthreads();
    const int w = threadIdx.x / kF2Lanes;
    const int64_t task = (int64_t)blockIdx.x * kF2FwdWarps + w;
    if (task >= tiling.count()) return;
    const F2Tile tl = tiling.tile(task, 0, g.nch, g.ns0, g.ns1);
    f2_run_forward<T, TX>(s_g, tl, smem + w * f2_fwd_warp_smem<T>());
}

// One grid, forward over sorted axis-1 samples: blockIdx.x is the tile.
template <typename T, typename TX>
__global__ void __launch_bounds__(kF2TileWarps * 32)
k_f2_fwdt_grid(F2Grid g, F2Tiling tiling) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ F2Grid s_g;
    __shared__ F2Tile s_t;
    if (threadIdx.x == 0) {
        s_g = g;
        s_t = tiling.tile((int64_t)blockIdx.x, 2, g.nch, g.ns0, g.ns1);
    }
    __syncthreads();
    f2_run_forward_tile<T, TX>(s_g, s_t, smem);
}

// Batch forward tiles: block x runs tile x of the list.
template <typename T>
__global__ void __launch_bounds__(kF2TileWarps * 32)
k_f2_fwdt_batch(const F2Grid *__restrict__ grids, const F2Tile *__restrict__ tiles) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ F2Grid s_g;
    __shared__ F2Tile s_t;
    static_assert(sizeof(F2Grid) % 4 == 0 && sizeof(F2Grid) / 4 <= kF2TileWarps * 32, "descriptor copy");
    if (threadIdx.x == 0) s_t = tiles[blockIdx.x];
    __syncthreads();
    if (threadIdx.x < sizeof(F2Grid) / 4)
        reinterpret_cast<int32_t *>(&s_g)[threadIdx.x] = reinterpret_cast<const int32_t *>(grids + s_t.grid)[threadIdx.x];
    __syncthreads();
    f2_run_forward_tile<T, T>(s_g, s_t, smem);
}

// One grid, adjoint: blockIdx.x is the tile.
template <typename T>
__global__ void __launch_bounds__(kF2AdjThreads, 2)
k_f2_adj_grid(F2Grid g, F2Tiling tiling, int *status) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ F2Grid s_g;
    __shared__ F2Tile s_t;
    if (threadIdx.x == 0) {
        s_g = g;
        s_t = tiling.tile((int64_t)blockIdx.x, 1, g.nch, g.n0, g.n1);
        f2_adj_init<T>(smem);
    }
    __syncthreads();
    uint32_t gstage = 0;
    f2_run_adjoint<T>(s_g, s_t, smem, gstage, status);
}

// Batch forward: warp w of block x runs unit 8x + w of the list (units are
// independent; the hardware hands out the blocks).
template <typename T>
__global__ void __launch_bounds__(kF2Lanes * kF2FwdWarps, 3)
k_f2_fwd_batch(const F2Grid *__restrict__ grids, const F2Tile *__restrict__ tiles, int64_t n_tiles) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ F2Grid s_g[kF2FwdWarps];
    static_assert(sizeof(F2Grid) % 4 == 0 && sizeof(F2Grid) / 4 <= kF2Lanes, "descriptor copy");
    const int w = threadIdx.x / kF2Lanes, lane = threadIdx.x % kF2Lanes;
    const int64_t task = (int64_t)blockIdx.x * kF2FwdWarps + w;
    if (task >= n_tiles) return;
    const F2Tile tl = tiles[task];
    if (lane < (int)(sizeof(F2Grid) / 4))
        reinterpret_cast<int32_t *>(&s_g[w])[lane] = reinterpret_cast<const int32_t *>(grids + tl.grid)[lane];
    __syncwarp();
    f2_run_forward<T, T>(s_g[w], tl, smem + w * f2_fwd_warp_smem<T>());
}

// Batch adjoint, persistent: every CTA takes the next tile of the list with one
// atomicAdd until the list is exhausted (or a bounded wait gave up).  Tiles do not
// depend on each other, so no CTA ever waits for another.
template <typename T>
__global__ void __launch_bounds__(kF2AdjThreads, 2)
k_f2_adj_batch(const F2Grid *__restrict__ grids, const F2Tile *__restrict__ tiles, int64_t n_tiles,
               unsigned long long *head, int *status) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ F2Grid s_g;
    __shared__ F2Tile s_t;
    __shared__ int64_t s_it;
    static_assert(sizeof(F2Grid) % 4 == 0 && sizeof(F2Grid) / 4 <= kF2AdjThreads, "descriptor copy");
    if (threadIdx.x == 0) f2_adj_init<T>(smem);
    uint32_t gstage = 0;  // stages consumed so far: the ring barriers' phases continue
    for (;;) {
        if (threadIdx.x == 0) {
            const int64_t it = (int64_t)atomicAdd(head, 1ull);
            s_it = it;
            if (it < n_tiles) s_t = tiles[it];
        }
        __syncthreads();
        if (s_it >= n_tiles) break;
        if (threadIdx.x < sizeof(F2Grid) / 4)
            reinterpret_cast<int32_t *>(&s_g)[threadIdx.x] =
                reinterpret_cast<const int32_t *>(grids + s_t.grid)[threadIdx.x];
        __syncthreads();
        f2_run_adjoint<T>(s_g, s_t, smem, gstage, status);
        __syncthreads();  // shared memory and the descriptors are free for the next tile
        if (*F2AdjSmem<T>(smem).abort) break;
    }
}

// ------------------------------------------------------------------ tiling
// Values a unit's set-up is worth (staging, first window): the per-grid tilings weigh
// it against wave quantization.
constexpr double kF2TileOverhead = 8192.0;
constexpr double kF2WarpTaskOverhead = 2048.0;

// Number of blocks along b: with slots > 0 (one grid alone on the GPU) the count whose
// waves of `base * nb` units finish first, counting a set-up per unit; otherwise the
// one closest to `target` values per unit.  values(nb): values of one unit.
template <typename F>
static int64_t pick_blocks(int64_t nb_lo, int64_t nb_hi, int64_t base, int slots, int64_t target,
                           double overhead, F values) {
    nb_hi = std::max(nb_lo, nb_hi);
    int64_t best = nb_lo;
    double best_cost = 1e300;
    for (int64_t nb = nb_lo; nb <= nb_hi; ++nb) {
        const double v = values(nb);
        double cost;
        if (slots > 0) {
            const double waves = (double)cdiv(base * nb, slots);
            cost = waves * (v + overhead);
        } else {
            cost = std::fabs(v - (double)target);
        }
        if (cost < best_cost) {
            best_cost = cost;
            best = nb;
        }
    }
    return best;
}

// Forward: warp tasks of 128 consecutive samples of axis 0 in one channel x a block of
// axis-1 rows (slots = resident warps).
bool f2_forward_tiling(int64_t ns0, int64_t ns1, int nch, int64_t target, int slots, F2Tiling &t) {
    if (ns0 < 1 || ns1 < 1 || nch < 1) return false;
    const int64_t nba = cdiv(ns0, kF2WarpS0);
    const int64_t per_row = std::min<int64_t>(ns0, kF2WarpS0);
    const int64_t nb_lo = cdiv(ns1, 2048);
    const int64_t nb_hi = std::max(nb_lo, std::min<int64_t>(cdiv(ns1, 16), 4096));
    const int64_t nbb0 = pick_blocks(nb_lo, nb_hi, (int64_t)nch * nba, slots, target, kF2WarpTaskOverhead,
                                     [&](int64_t nb) { return (double)per_row * (double)cdiv(ns1, nb); });
    const int64_t rows = cdiv(ns1, nbb0);
    t.G = 1;
    t.ngrp = nch;
    t.ka = kF2WarpS0;
    t.nba = (int32_t)nba;
    t.kb = (int32_t)rows;
    t.nbb = (int32_t)cdiv(ns1, rows);
    return true;
}

// Adjoint: tiles span axis 0 whole (its ns0 samples times the tile's channels fit one
// tile) and a block of axis-1 control points.  lb0: the axis-0 support table
// (lb0[c + d0] = first sample whose support start is >= c, n0 + d0 + 1 entries).
// target <= 0 and slots == 0: one axis-1 block (the whole axis, no cotangent row is
// read twice).
// Support start of row r of a sorted axis from its support table lb[c + d] (the first
// row whose support start is >= c): the largest c with lb[c + d] <= r.
static int64_t support_of_row(const int32_t *lb, int64_t n, int d, int64_t r) {
    int64_t lo = 0, hi = std::max<int64_t>(0, n - d - 1);
    while (lo < hi) {
        const int64_t mid = (lo + hi + 1) / 2;
        if (lb[mid + d] <= r) lo = mid; else hi = mid - 1;
    }
    return lo;
}

void f2_tile_columns(const int32_t *lb1, int64_t n1, int d1, int64_t b_lo, int64_t b_len, int32_t &cb,
                     int32_t &ncol) {
    cb = (int32_t)support_of_row(lb1, n1, d1, b_lo);
    ncol = (int32_t)(support_of_row(lb1, n1, d1, b_lo + b_len - 1) + d1 + 1 - cb);
}

bool f2_forward_tile_tiling(const int32_t *lb1, int64_t n1, int d1, int64_t ns0, int64_t ns1, int nch,
                            int cols, int64_t target, int slots, F2Tiling &t) {
    if (ns0 < 1 || ns1 < 1 || nch < 1 || n1 < 1 || !lb1 || cols < d1 + 1) return false;
    const int64_t nba = cdiv(ns0, kF2TileS0);
    const int64_t per_row = std::min<int64_t>(ns0, kF2TileS0);
    // widest column span of a uniform blocking into rows of kb
    auto fits = [&](int64_t kb) {
        for (int64_t r0 = 0; r0 < ns1; r0 += kb) {
            const int64_t r1 = std::min(ns1, r0 + kb) - 1;
            if (support_of_row(lb1, n1, d1, r1) + d1 + 1 - support_of_row(lb1, n1, d1, r0) > cols) return false;
        }
        return true;
    };
    int64_t nbb = 1;
    if (slots > 0) {  // at most kF2TileRows rows per tile
        nbb = pick_blocks(cdiv(ns1, kF2TileRows), std::max<int64_t>(cdiv(ns1, kF2TileRows), std::min<int64_t>(ns1, 4096)),
                          (int64_t)nch * nba, slots, 0, kF2TileOverhead,
                          [&](int64_t nb) { return (double)per_row * (double)cdiv(ns1, nb); });
    } else {
        nbb = cdiv(ns1, std::max<int64_t>(1, (target > 0 ? target : 16384) / per_row));
    }
    int64_t kb = std::min<int64_t>(cdiv(ns1, nbb), kF2TileRows);
    while (kb > 1 && !fits(kb)) kb = std::max<int64_t>(1, kb - std::max<int64_t>(1, kb / 8));
    if (!fits(kb)) return false;
    t.G = 1;
    t.ngrp = nch;
    t.ka = kF2TileS0;
    t.nba = (int32_t)nba;
    t.kb = (int32_t)kb;
    t.nbb = (int32_t)cdiv(ns1, kb);
    return true;
}

bool f2_adjoint_tiling(const int32_t *lb0, int64_t n0, int d0, int64_t ns0, int64_t n1, int d1,
                       int64_t ns1, int nch, int np, int align, int64_t target, int slots, F2Tiling &t) {
    if (n0 < 1 || n1 < 1 || nch < 1 || np < 1 || align < 1 || !lb0 || ns0 < 1) return false;
    if ((int64_t)lb0[n0 + d0] - lb0[0] != ns0) return false;  // every sample in some support
    int64_t G = 1, ngrp = nch, ka = n0, nba = 1, w0 = ns0;
    if (ns0 <= np) {  // axis 0 whole, channel groups
        const int64_t gmax = std::max<int64_t>(1, std::min<int64_t>(np / ns0, kF2MaxG));
        ngrp = cdiv(nch, std::min<int64_t>(gmax, nch));
        G = cdiv(nch, ngrp);
    } else {
        // chunks of control points, one channel per tile: a chunk reads the samples of its
        // supports (its last d0 knot spans again in the next chunk), one row copy each,
        // so a row must be a 16-byte multiple and a chunk's samples (plus the copy's
        // lead) must fit the stage
        if (ns0 % align != 0) return false;
        const int64_t wmax = np - 2 * align;
        auto widest = [&](int64_t k) {
            int64_t w = 0;
            for (int64_t a = 0; a < n0; a += k)
                w = std::max<int64_t>(w, lb0[std::min(a + k, n0) + d0] - lb0[a]);
            return w;
        };
        nba = std::max<int64_t>(2, ns0 / wmax);
        for (;; ++nba) {
            if (nba > n0) return false;  // one control point's support is too wide
            ka = cdiv(n0, nba);
            if (widest(ka) <= wmax) break;
        }
        nba = cdiv(n0, ka);
        w0 = widest(ka);
    }
    const int64_t pairs = w0 * G;
    int64_t nbb = 1;
    if (target > 0 || slots > 0) {
        // cotangent rows a block of kb control points reads: its d1 knot spans of halo
        const double rows_per_cp = (double)ns1 / (double)n1;
        nbb = pick_blocks(1, std::min<int64_t>(n1, 4096), ngrp * nba, slots, target, kF2TileOverhead,
                          [&](int64_t nb) {
                              const double kb = (double)cdiv(n1, nb);
                              return (double)pairs * std::min((double)ns1, (kb + d1) * rows_per_cp);
                          });
    }
    const int64_t kb = cdiv(n1, nbb);
    t.G = (int32_t)G;
    t.ngrp = (int32_t)cdiv(nch, G);
    t.ka = (int32_t)ka;
    t.nba = (int32_t)nba;
    t.kb = (int32_t)kb;
    t.nbb = (int32_t)cdiv(n1, kb);
    return true;
}

// ------------------------------------------------------------------ launchers
template <typename K>
static void set_smem(K kernel, int64_t bytes) {
    cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

template <typename T, typename TX>
static int launch_grid_t(const F2Grid &g, const F2Tiling &t, int kind, int *status, cudaStream_t s) {
    const int64_t n = t.count();
    if (n == 0) return SG_OK;
    static bool attr = false;  // one instance per template instantiation
    if (!attr) {
        set_smem(k_f2_fwd_grid<T, TX>, f2_fwd_smem<T>());
        set_smem(k_f2_fwdt_grid<T, TX>, f2_tile_smem<T>());
        if constexpr (std::is_same<T, TX>::value) set_smem(k_f2_adj_grid<T>, f2_adj_smem<T>());
        attr = true;
    }
    if (kind == 2) {
        if (n > 0x7fffffffLL) return set_error(SG_ERR_UNSUPPORTED, "fused 2D: too many tiles");
        k_f2_fwdt_grid<T, TX><<<(unsigned)n, kF2TileWarps * 32, (size_t)f2_tile_smem<T>(), s>>>(g, t);
    } else if (kind == 0) {
        const int64_t blocks = cdiv(n, kF2FwdWarps);
        if (blocks > 0x7fffffffLL) return set_error(SG_ERR_UNSUPPORTED, "fused 2D: too many units");
        k_f2_fwd_grid<T, TX><<<(unsigned)blocks, kF2Lanes * kF2FwdWarps, (size_t)f2_fwd_smem<T>(), s>>>(g, t);
    } else if constexpr (std::is_same<T, TX>::value) {
        if (n > 0x7fffffffLL) return set_error(SG_ERR_UNSUPPORTED, "fused 2D: too many tiles");
        k_f2_adj_grid<T><<<(unsigned)n, kF2AdjThreads, (size_t)f2_adj_smem<T>(), s>>>(g, t, status);
    }
    return cuda_check(cudaGetLastError(), "fused 2D launch");
}

int f2_launch_grid(int dtype, const F2Grid &g, const F2Tiling &t, int kind, int *status, cudaStream_t s) {
    if (dtype == SG_F64) return launch_grid_t<double, double>(g, t, kind, status, s);
    if (dtype == SG_BF16_F32 && kind != 1) return launch_grid_t<float, __nv_bfloat16>(g, t, kind, status, s);
    return launch_grid_t<float, float>(g, t, kind, status, s);
}

// resident forward warps and adjoint CTAs on this device (the persistent grid and the
// per-grid wave model)
template <typename T>
struct F2Occupancy {
    int fwd = 0, adj = 0, tile = 0;
    F2Occupancy() {
        set_smem(k_f2_fwd_batch<T>, f2_fwd_smem<T>());
        set_smem(k_f2_fwdt_batch<T>, f2_tile_smem<T>());
        set_smem(k_f2_adj_batch<T>, f2_adj_smem<T>());
        int dev = 0, sms = 0, pf = 0, pa = 0, pt = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&pf, k_f2_fwd_batch<T>, kF2Lanes * kF2FwdWarps,
                                                      (size_t)f2_fwd_smem<T>());
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&pa, k_f2_adj_batch<T>, kF2AdjThreads,
                                                      (size_t)f2_adj_smem<T>());
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&pt, k_f2_fwdt_batch<T>, kF2TileWarps * 32,
                                                      (size_t)f2_tile_smem<T>());
        fwd = std::max(1, sms * std::max(1, pf) * kF2FwdWarps);
        adj = std::max(1, sms * std::max(1, pa));
        tile = std::max(1, sms * std::max(1, pt));
    }
};

template <typename T>
static const F2Occupancy<T> &occupancy() {
    static F2Occupancy<T> o;  // first use, on the device current then
    return o;
}

int f2_slots(int dtype, int kind) {
    if (dtype == SG_F64) return kind == 0 ? occupancy<double>().fwd : kind == 1 ? occupancy<double>().adj
                                                                              : occupancy<double>().tile;
    return kind == 0 ? occupancy<float>().fwd : kind == 1 ? occupancy<float>().adj : occupancy<float>().tile;
}

int f2_launch_batch(int dtype, int kind, const F2Grid *grids, const F2Tile *tiles, int64_t n_tiles,
                    unsigned long long *head, int *status, cudaStream_t s) {
    if (n_tiles == 0) return SG_OK;
    if (kind == 2) {  // forward tiles, one per CTA
        if (n_tiles > 0x7fffffffLL) return set_error(SG_ERR_UNSUPPORTED, "fused 2D: too many units");
        if (dtype == SG_F64) {
            (void)occupancy<double>();
            k_f2_fwdt_batch<double><<<(unsigned)n_tiles, kF2TileWarps * 32, (size_t)f2_tile_smem<double>(), s>>>(
                grids, tiles);
        } else {
            (void)occupancy<float>();
            k_f2_fwdt_batch<float><<<(unsigned)n_tiles, kF2TileWarps * 32, (size_t)f2_tile_smem<float>(), s>>>(
                grids, tiles);
        }
    } else if (kind == 0) {  // independent warp tasks, one per warp
        const int64_t blocks = cdiv(n_tiles, kF2FwdWarps);
        if (blocks > 0x7fffffffLL) return set_error(SG_ERR_UNSUPPORTED, "fused 2D: too many units");
        if (dtype == SG_F64) {
            (void)occupancy<double>();
            k_f2_fwd_batch<double><<<(unsigned)blocks, kF2Lanes * kF2FwdWarps, (size_t)f2_fwd_smem<double>(), s>>>(
                grids, tiles, n_tiles);
        } else {
            (void)occupancy<float>();
            k_f2_fwd_batch<float><<<(unsigned)blocks, kF2Lanes * kF2FwdWarps, (size_t)f2_fwd_smem<float>(), s>>>(
                grids, tiles, n_tiles);
        }
    } else {  // persistent CTAs over the tile list
        const unsigned ctas = (unsigned)std::min<int64_t>(f2_slots(dtype, 1), n_tiles);
        if (dtype == SG_F64)
            k_f2_adj_batch<double><<<ctas, kF2AdjThreads, (size_t)f2_adj_smem<double>(), s>>>(
                grids, tiles, n_tiles, head, status);
        else
            k_f2_adj_batch<float><<<ctas, kF2AdjThreads, (size_t)f2_adj_smem<float>(), s>>>(
                grids, tiles, n_tiles, head, status);
    }
    return cuda_check(cudaGetLastError(), "fused 2D batch launch");
}

int64_t f2_pairs_per_tile(int dtype) { return dtype == SG_F64 ? f2_pairs<double>() : f2_pairs<float>(); }

int f2_set_wait_cycles(int64_t cycles) {
    const long long v = cycles > 0 ? (long long)cycles : kMbarWaitCycles;
    return cuda_check(cudaMemcpyToSymbol(g_f2_wait_cycles, &v, sizeof(v)), "fused 2D: wait budget");
}

int f2_set_withhold_first_stage(bool on) {
    const int v = on ? 1 : 0;
    return cuda_check(cudaMemcpyToSymbol(g_f2_withhold_first_stage, &v, sizeof(v)), "fused 2D: test hook");
}

}  // namespace sg
