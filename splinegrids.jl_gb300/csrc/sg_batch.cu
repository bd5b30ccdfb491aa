// sg_batch.cu -- many grids of uneven sizes, forward and adjoint, in one persistent
// launch fed by a device-side work queue.
//
// A batch plan turns every grid's separable passes (sg_contract.cuh) into a list of
// passes in queue order: for each grid, its forward passes then its adjoint passes.
// Every pass is cut into tiles; the queue is the concatenation of all passes' tiles,
// and persistent CTAs (as many as fit on the GPU at once) take the next tile with one
// atomicAdd on a device counter.  A pass that reads the output of an earlier pass of
// the same grid waits, before its first tile, until that pass's completion counter
// reaches its tile count.  All tiles of the earlier pass were dequeued before the
// waiting tile (queue order) by CTAs that are running and depend on nothing later, so
// the wait always ends; it is nevertheless bounded (kSpinLimit polls), and on timeout
// the CTA records SG_ERR_TIMEOUT in the plan's status word and skips the tile, so the
// kernel always terminates and the host reports the error (sg_batch_check).
//
// Because each grid's passes are close in the queue, the intermediate tensor of a grid
// is produced and consumed while it is still in L2, and the whole batch (all grids,
// forward and adjoint) is one launch: no per-grid launch overhead and no tails between
// passes.  Memory ordering: producers fence their writes before counting a tile done;
// the consumer's ld.acquire.gpu of the counter (which also invalidates the SM's L1)
// and the following barrier order every later load of the CTA after those writes.  An
// intermediate is read only after its producer completed, so no SM can hold a stale
// L1 copy of it, and ordinary (L1-cached) loads are used.
#include <algorithm>
#include <array>
#include <cstring>
#include <numeric>
#include <vector>

#include "sg_passes.cuh"
#include "sg_fused2d_host.h"

namespace sg {

enum PassKind : int32_t {
    kFwdAxis0 = 0,   // forward, axis 0: warp tasks of 32 columns
    kFwdAxis = 1,    // forward, axis k >= 1: warp tasks
    kAdjAxis = 2,    // adjoint, axis k >= 1, input not 16-byte aligned: warp tasks
    kAdjAxis0 = 3,   // adjoint, axis 0: warp tasks of 32 columns x 32 control points
    kAdjStream = 4,  // adjoint, axis k >= 1: bulk-copy stream tiles (sg_stream.cuh)
};

constexpr int kBatchThreads = kStreamThreads;     // the stream's consumer warps + its producer
// Warp tasks per queue item: every warp of the block (stream tiles use 8 consumer
// warps and the producer warp; warp-task items give each of the 9 warps a task).
constexpr int kBatchWarpTasks = kBatchThreads / 32;
__host__ __device__ constexpr int tasks_per_item(int32_t) { return kBatchWarpTasks; }

// shared memory of one warp task (the larger of the forward and adjoint layouts)
template <typename T>
__host__ __device__ constexpr int batch_warp_smem() {
    return warp_adj_smem<4, T>() > warp_fwd_smem<4, T>() ? warp_adj_smem<4, T>() : warp_fwd_smem<4, T>();
}
constexpr unsigned kSpinLimit = 1u << 22;  // ~0.5 s of polling with 100 ns sleeps

// Test hooks of the bounded waits (sg_test_set_wait_limits, sg_test_block_waits): the
// poll limit of a dependency wait, and extra completed tiles a wait asks for (nonzero:
// no dependency can ever complete, so every wait runs out).
static unsigned g_batch_spin_limit = kSpinLimit;
static int g_batch_dep_extra = 0;

// One pass of one grid in the queue.
struct BatchPass {
    int32_t kind, D, vec, final_pass;
    int32_t dep;      // index of the pass whose output this pass reads, or -1
    int32_t cc_qt;    // adjoint axis: control points per task; axis-0 adjoint: QT
    int32_t d, nch;
    int32_t rows;     // stream tiles: rows per stage
    int32_t unused;
    int64_t gx, gy, gz;
    int64_t first;    // first queue index of this pass's tiles
    int64_t tiles;    // queue items: gx*gy*gz tiles (axis 0) or ceil(gx*gy*gz / 4) warp tasks
    const int32_t *idx, *perm, *lb;
    const void *B;
    int64_t ns, n, M, Q;
    const void *X;
    void *Y;
};

// tile of pass p for queue index `it`
__device__ __forceinline__ Tile batch_tile(const BatchPass &p, int64_t it) {
    int64_t r = it - p.first;
    Tile t;
    t.bx = r % p.gx;
    r /= p.gx;
    t.by = r % p.gy;
    t.bz = r / p.gy;
    t.gy = p.gy;
    t.gz = p.gz;
    return t;
}

// One out-of-line entry per tile variant: each is register-allocated on its own, so
// the persistent kernel's register budget is the largest variant's, not their union.
// axis-0 forward: warp task = 32 columns x kFwd0Samples samples (gx = column groups,
// gy = sample chunks)
constexpr int kFwd0Samples = 128;
template <typename T, int D>
__device__ __noinline__ void b_fwd_axis0(const BatchPass &p, int64_t task, unsigned char *sm) {
    const int64_t cg = task % p.gx, sc = task / p.gx;
    const int64_t s0 = sc * kFwd0Samples;
    const int64_t s1 = (s0 + kFwd0Samples < p.ns) ? s0 + kFwd0Samples : p.ns;
    fwd0_warp<D, T>(cg * 32, s0, s1, threadIdx.x & 31, sm, p.idx, (const T *)p.B, p.ns, p.d,
                    (const T *)p.X, p.n, p.Q * p.nch, (T *)p.Y);
}

// Axes k >= 1: a queue item is kBatchWarpTasks warp tasks (sg_warp.cuh), numbered
// m-fastest (gx = warp tiles along m, gy = chunks, gz = columns).
template <typename T, int D, bool ST, bool FINAL>
__device__ __noinline__ void b_fwd_axis(const BatchPass &p, int64_t task, unsigned char *sm) {
    const int64_t mw = task % p.gx, r = task / p.gx;
    fwd_axis_warp<D, T, ST, FINAL>(mw, r % p.gy, kFwdTaskRows, r / p.gy, threadIdx.x & 31, sm, p.idx,
                                   (const T *)p.B, p.ns, p.d, (const T *)p.X, p.M, p.n, (T *)p.Y);
}

template <typename T, int D, bool ST>
__device__ __noinline__ void b_adj_axis(const BatchPass &p, int64_t task, unsigned char *sm) {
    const int64_t mw = task % p.gx, r = task / p.gx;
    adj_axis_warp<D, T, ST>(mw, r % p.gy, r / p.gy, threadIdx.x & 31, sm, p.idx, p.perm, p.lb,
                            (const T *)p.B, p.ns, p.d, (const T *)p.X, p.M, p.n, p.cc_qt, (T *)p.Y);
}

// stream tile (gx = m blocks, gy = chunks, gz = columns)
template <typename T, int D>
__device__ __noinline__ void b_adj_stream(const BatchPass &p, Tile tl, unsigned char *sm,
                                          int *status) {
    constexpr int64_t W = stream_width<T>();
    const int64_t m_lo = tl.bx * W;
    const int64_t L = (p.M - m_lo) < W ? (p.M - m_lo) : W;
    adj_stream_tile<D, T>(m_lo, L, tl.by, tl.bz, p.rows, sm, p.idx, p.perm, p.lb, (const T *)p.B,
                          p.ns, p.d, (const T *)p.X, p.M, p.n, p.cc_qt, (T *)p.Y, status);
}

// axis-0 adjoint: warp task = 32 columns x kAdj0Chunk control points (gx = column groups,
// gy = chunks); shorter tasks than whole columns balance the queue's tail
constexpr int kAdj0Chunk = 32;
template <typename T, int D>
__device__ __noinline__ void b_adj_axis0(const BatchPass &p, int64_t task, unsigned char *sm) {
    const int64_t cg = task % p.gx, c_lo = (task / p.gx) * kAdj0Chunk;
    const int64_t c_hi = c_lo + kAdj0Chunk < p.n ? c_lo + kAdj0Chunk : p.n;
    adj0_warp<D, T>(cg * 32, c_lo, c_hi, threadIdx.x & 31, sm, p.idx, p.perm, p.lb, (const T *)p.B,
                    p.ns, p.d, (const T *)p.X, p.n, p.Q, (T *)p.Y);
}

template <typename T, int D>
__device__ __forceinline__ void run_tile_d(const BatchPass &p, int64_t it, unsigned char *sm,
                                           int *status) {
    constexpr int V = 16 / (int)sizeof(T);
    if (p.kind == kAdjStream) {
        b_adj_stream<T, D>(p, batch_tile(p, it), sm, status);
    } else {
        const int w = threadIdx.x >> 5;
        const int per_item = tasks_per_item(p.kind);
        const int64_t task = (it - p.first) * per_item + w;
        if (task >= p.gx * p.gy * p.gz) return;
        if (p.kind == kAdjAxis0) {
            b_adj_axis0<T, D>(p, task, sm + w * warp_adj0_smem<4, T>());
            return;
        }
        if (p.kind == kFwdAxis0) {
            b_fwd_axis0<T, D>(p, task, sm + w * warp_fwd0_smem<4, T>());
            return;
        }
        unsigned char *wsm = sm + w * batch_warp_smem<T>();
        // vec == V: aligned rows, contiguous lanes; otherwise strided lanes
        if (p.kind == kFwdAxis) {
            if (p.vec == V) {
                if (p.final_pass) b_fwd_axis<T, D, false, true>(p, task, wsm);
                else b_fwd_axis<T, D, false, false>(p, task, wsm);
            } else {
                if (p.final_pass) b_fwd_axis<T, D, true, true>(p, task, wsm);
                else b_fwd_axis<T, D, true, false>(p, task, wsm);
            }
        } else {
            if (p.vec == V) b_adj_axis<T, D, false>(p, task, wsm);
            else b_adj_axis<T, D, true>(p, task, wsm);
        }
    }
}

__device__ __forceinline__ int ld_acquire(const int *p) {
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

template <typename T>
__global__ void __launch_bounds__(kBatchThreads, 3)
k_batch(const BatchPass *__restrict__ passes, int32_t n_passes, int64_t n_items,
        unsigned long long *head, int *done, int *status, unsigned long long *prof,
        unsigned spin_limit, int dep_extra) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ int64_t s_item;
    __shared__ int32_t s_pass;
    __shared__ int32_t s_skip;
    __shared__ BatchPass s_P;
    // Queue indices a CTA takes only grow, so its pass index only moves forward: the
    // lookup walks from the previous pass (usually 0-2 steps) and the descriptor is
    // copied to shared memory only when the pass changes.
    int32_t cur_pass = -1;
    long long t_take = 0, t_work = 0;  // profile: item taken, dependency met (thread 0)
    for (;;) {
        if (threadIdx.x == 0) {
            if (prof) t_take = clock64();
            const int64_t it = (int64_t)atomicAdd(head, 1ull);
            s_item = it;
            int32_t p = cur_pass < 0 ? 0 : cur_pass;
            s_skip = 0;
            if (it < n_items) {
                if (cur_pass < 0) {  // first item of this CTA: binary search
                    int32_t lo = 0, hi = n_passes - 1;  // last pass with first <= it
                    while (lo < hi) {
                        const int32_t mid = (lo + hi + 1) >> 1;
                        if (passes[mid].first <= it) lo = mid; else hi = mid - 1;
                    }
                    p = lo;
                } else {
                    while (p + 1 < n_passes && passes[p + 1].first <= it) ++p;
                }
                const int32_t dep = passes[p].dep;
                if (dep >= 0) {
                    const int need = (int)passes[dep].tiles + dep_extra;
                    unsigned spins = 0;
                    while (ld_acquire(done + dep) < need) {
                        // gives up after spin_limit polls, or at once when another CTA
                        // already gave up (the launch's results are invalid then)
                        if (++spins > spin_limit || ld_acquire(status) != 0) {
                            atomicExch(status, SG_ERR_TIMEOUT);
                            s_skip = 1;
                            break;
                        }
                        __nanosleep(100);
                    }
                }
            }
            if (it < n_items && p != cur_pass) s_P = passes[p];
            s_pass = p;
            cur_pass = p;
            if (prof) t_work = clock64();
        }
        __syncthreads();
        const int64_t it = s_item;
        if (it >= n_items) break;
        const BatchPass &P = s_P;
        if (!s_skip) {
            switch (P.D) {
                case 1: run_tile_d<T, 1>(P, it, smem, status); break;
                case 2: run_tile_d<T, 2>(P, it, smem, status); break;
                case 3: run_tile_d<T, 3>(P, it, smem, status); break;
                default: run_tile_d<T, 4>(P, it, smem, status); break;
            }
        }
        __threadfence();  // this thread's writes are visible GPU-wide before the count
        __syncthreads();
        if (threadIdx.x == 0) {
            atomicAdd(done + s_pass, 1);
            if (prof) {
                unsigned long long *pk = prof + 3 * P.kind;
                atomicAdd(pk, (unsigned long long)(t_work - t_take));
                atomicAdd(pk + 1, (unsigned long long)(clock64() - t_work));
                atomicAdd(pk + 2, 1ull);
            }
        }
    }
}

template <typename T>
constexpr int64_t batch_smem_bytes() {
    int64_t m = (int64_t)kBatchWarpTasks * batch_warp_smem<T>();
    m = std::max<int64_t>(m, (int64_t)kBatchWarpTasks * warp_adj0_smem<4, T>());
    m = std::max<int64_t>(m, (int64_t)kBatchWarpTasks * warp_fwd0_smem<4, T>());
    m = std::max<int64_t>(m, stream_smem_bytes<4, T>());
    return m;
}

}  // namespace sg

using namespace sg;

struct sg_batch_plan {
    int32_t n_grids = 0;
    int32_t dtype = SG_F32;
    std::vector<sg_grid_desc> desc;
    std::vector<std::array<int32_t, SG_MAX_NIN>> orders;
    std::vector<std::vector<int32_t *>> perm, lb;  // device, per grid per axis
    std::vector<int32_t *> off0;                   // device, per grid: fused adjoint weight offsets
    std::vector<void *> fwd_scratch, adj_scratch;  // device, per grid (ping-pong x2)
    std::vector<int64_t> scratch_elems;
    // host copies of the pass tables for the three run modes; device copies below
    std::vector<BatchPass> host_passes[4];
    BatchPass *dev_passes[4] = {};
    int64_t n_items[4] = {};
    int *done = nullptr;  // per pass of the largest table
    unsigned long long *head = nullptr;
    int *status = nullptr;
    unsigned long long *prof = nullptr;  // per pass kind: take+wait cycles, work cycles, items
    bool profile = false;
    bool arrays_set = false;
    int grid_ctas = 0;
    std::vector<void *> allocs;
    // fused Nin = 2 grids (sg_fused2d.cuh): a forward unit list and an adjoint tile
    // list; these grids need no intermediates and are not in the pass queue
    int32_t strategy = SG_STRATEGY_AUTO;
    int64_t f2_fwd_target = kF2BatchFwdTarget;   // eval values per forward unit
    int64_t f2_adj_target = kF2BatchAdjTarget;   // cotangent values per adjoint tile (0: axis 1 whole)
    std::vector<char> f2_ok;                     // per grid: eligible for the fused path
    std::vector<sg::F2Tiling> f2_fwd, f2_adj;    // per grid
    std::vector<char> scratch_done;              // per grid: separable intermediates allocated
    std::vector<std::vector<int32_t>> lb0_host, lb1_host;  // per grid: support tables
    std::vector<sg::F2Tile> f2_tiles[2];         // host copies: forward units, adjoint tiles
    sg::F2Tile *dev_f2_tiles[2] = {};
    int64_t n_f2[2] = {};
    sg::F2Grid *dev_f2_grids = nullptr;          // [2 * n_grids]: forward, adjoint descriptors
    unsigned long long *f2_head = nullptr;       // queue head of the adjoint tile list
    // the arrays of the last sg_batch_set_arrays (rebuilt when the strategy changes)
    std::vector<const void *> a_cp, a_ebar;
    std::vector<void *> a_ev, a_cpbar;
    bool has_fwd = false, has_adj = false;
};

static void batch_free(sg_batch_plan *p) {
    for (void *a : p->allocs) dev_free(a);  // everything but the work lists
    for (int m = 0; m < 4; ++m)
        dev_free(p->dev_passes[m]);
    for (int k = 0; k < 2; ++k)
        dev_free(p->dev_f2_tiles[k]);
    delete p;
}

static bool grid_fused(const sg_batch_plan *p, int g) {
    return p->f2_ok[g] && p->strategy != SG_STRATEGY_SEPARABLE;
}

static int batch_alloc(sg_batch_plan *p, void **out, size_t bytes, const char *what) {
    int rc = dev_alloc(out, bytes, what);
    if (!rc) p->allocs.push_back(*out);
    return rc;
}

// The separable passes' intermediates of grid g, forward and adjoint separately (both
// may be in flight in one launch); allocated once, when the grid first needs them.
static int batch_scratch(sg_batch_plan *p, int g) {
    if (p->scratch_done[g]) return SG_OK;
    const sg_grid_desc &d = p->desc[g];
    const size_t es = p->dtype == SG_F64 ? 8 : 4;
    const int64_t best = p->scratch_elems[g];
    const int nbuf = d.nin >= 3 ? 2 : (d.nin == 2 ? 1 : 0);
    int rc = SG_OK;
    for (int b = 0; b < nbuf && !rc; ++b) {
        rc = batch_alloc(p, &p->fwd_scratch[2 * g + b], best * es, "batch: forward scratch");
        if (!rc) rc = batch_alloc(p, &p->adj_scratch[2 * g + b], best * es, "batch: adjoint scratch");
    }
    if (!rc) p->scratch_done[g] = 1;
    return rc;
}

extern "C" int sg_batch_plan_create(int32_t n_grids, const sg_grid_desc *grids,
                                    const int32_t *derivative_orders, sg_stream_t stream,
                                    sg_batch_plan **out) {
    if (!out) return set_error(SG_ERR_INVALID_ARGUMENT, "batch: output pointer is NULL");
    *out = nullptr;
    if (n_grids < 1 || !grids || !derivative_orders)
        return set_error(SG_ERR_INVALID_ARGUMENT, "batch: need n_grids >= 1, grids and orders");
    sg_batch_plan *p = new sg_batch_plan();
    p->n_grids = n_grids;
    p->dtype = grids[0].dtype;
    p->desc.assign(grids, grids + n_grids);
    p->orders.resize(n_grids);
    p->perm.assign(n_grids, std::vector<int32_t *>(SG_MAX_NIN, nullptr));
    p->lb.assign(n_grids, std::vector<int32_t *>(SG_MAX_NIN, nullptr));
    p->off0.assign(n_grids, nullptr);
    p->fwd_scratch.assign(2 * n_grids, nullptr);
    p->adj_scratch.assign(2 * n_grids, nullptr);
    p->scratch_elems.assign(n_grids, 0);
    p->f2_ok.assign(n_grids, 0);
    p->f2_fwd.assign(n_grids, F2Tiling());
    p->f2_adj.assign(n_grids, F2Tiling());
    p->scratch_done.assign(n_grids, 0);
    p->lb0_host.assign(n_grids, {});
    p->lb1_host.assign(n_grids, {});
    cudaStream_t s = (cudaStream_t)stream;
    int rc = SG_OK;
    const size_t es = p->dtype == SG_F64 ? 8 : 4;
    for (int g = 0; g < n_grids && !rc; ++g) {
        const sg_grid_desc &d = p->desc[g];
        if (d.dtype != p->dtype || (d.dtype != SG_F32 && d.dtype != SG_F64)) {
            rc = set_error(SG_ERR_UNSUPPORTED, "batch: grid %d: all grids must be F32 or all F64", g);
            break;
        }
        if (d.has_weights) {
            rc = set_error(SG_ERR_UNSUPPORTED, "batch: grid %d: NURBS grids use sg_evaluate", g);
            break;
        }
        if (d.nin < 1 || d.nin > SG_MAX_NIN || d.nout < 1) {
            rc = set_error(SG_ERR_INVALID_ARGUMENT, "batch: grid %d: bad nin/nout", g);
            break;
        }
        for (int k = 0; k < d.nin && !rc; ++k) {
            const int o = derivative_orders[g * SG_MAX_NIN + k];
            p->orders[g][k] = o;
            if (d.degree[k] < 0 || d.degree[k] > 3)
                rc = set_error(SG_ERR_UNSUPPORTED, "batch: grid %d: degree %d > 3 (use sg_evaluate)",
                               g, d.degree[k]);
            else if (d.n_basis[k] < d.degree[k] + 1 || d.n_samples[k] < 1 ||
                     d.n_samples[k] > INT32_MAX || !d.sample_indices[k] || !d.basis_eval[k])
                rc = set_error(SG_ERR_INVALID_ARGUMENT, "batch: grid %d: bad dimension %d", g, k + 1);
            else if (o < 0 || o > d.max_derivative_order[k])
                rc = set_error(SG_ERR_INVALID_ARGUMENT,
                               "batch: grid %d: derivative order %d not available in dimension %d",
                               g, o, k + 1);
        }
        if (rc) break;
        // sample indices: range check, sorted view, support tables (as a grid plan)
        bool sorted_all = true;
        for (int k = 0; k < d.nin && !rc; ++k) {
            const int64_t ns = d.n_samples[k], n = d.n_basis[k];
            const int dk = d.degree[k];
            std::vector<int32_t> h(ns);
            rc = cuda_check(cudaMemcpyAsync(h.data(), d.sample_indices[k], ns * 4,
                                            cudaMemcpyDeviceToHost, s), "batch: read indices");
            if (!rc) rc = cuda_check(cudaStreamSynchronize(s), "batch: sync");
            if (rc) break;
            bool sorted = true;
            for (int64_t j = 0; j < ns; ++j) {
                if (h[j] < dk + 1 || h[j] > n) {
                    rc = set_error(SG_ERR_INVALID_ARGUMENT, "batch: grid %d dim %d: sample index "
                                   "%d out of range", g, k + 1, h[j]);
                    break;
                }
                if (j && h[j] < h[j - 1]) sorted = false;
            }
            if (rc) break;
            std::vector<int32_t> perm(ns);
            std::iota(perm.begin(), perm.end(), 0);
            if (!sorted) {
                std::stable_sort(perm.begin(), perm.end(), [&](int32_t a, int32_t b) { return h[a] < h[b]; });
                void *dp;
                rc = batch_alloc(p, &dp, ns * 4, "batch: perm");
                if (!rc) rc = cuda_check(cudaMemcpy(dp, perm.data(), ns * 4, cudaMemcpyHostToDevice), "batch: perm");
                p->perm[g][k] = (int32_t *)dp;
                if (rc) break;
            }
            std::vector<int32_t> lb(n + dk + 1);
            int64_t sp = 0;
            for (int64_t i = 0; i <= n + dk; ++i) {
                while (sp < ns && (int64_t)h[perm[sp]] - dk - 1 < i - dk) ++sp;
                lb[i] = (int32_t)sp;
            }
            void *dl;
            rc = batch_alloc(p, &dl, lb.size() * 4, "batch: support table");
            if (!rc) rc = cuda_check(cudaMemcpy(dl, lb.data(), lb.size() * 4, cudaMemcpyHostToDevice), "batch: lb");
            p->lb[g][k] = (int32_t *)dl;
            sorted_all = sorted_all && sorted;
            if (k == 0) {  // the fused adjoint's weight-list offsets
                p->lb0_host[g] = lb;
                const std::vector<int32_t> off = f2_weight_offsets(lb.data(), n, dk);
                void *doff;
                rc = batch_alloc(p, &doff, off.size() * 4, "batch: weight offsets");
                if (!rc) rc = cuda_check(cudaMemcpy(doff, off.data(), off.size() * 4, cudaMemcpyHostToDevice),
                                         "batch: weight offsets");
                p->off0[g] = (int32_t *)doff;
                if (rc) break;
            }
            if (k == 1) p->lb1_host[g] = lb;
        }
        if (rc) break;
        // largest intermediate of the separable passes
        int64_t best = 0;
        for (int k = 1; k < d.nin; ++k) {
            int64_t e = d.nout;
            for (int i = 0; i < d.nin; ++i) e *= (i < k) ? d.n_samples[i] : d.n_basis[i];
            best = std::max(best, e);
        }
        p->scratch_elems[g] = best;
        // the fused Nin = 2 path: sorted samples, 32-bit offsets, tiles that fit
        if (d.nin == 2 && sorted_all && d.n_samples[0] > 0 && d.n_samples[1] > 0 &&
            f2_offsets_fit(d.n_samples[0], d.n_samples[1], d.n_basis[0], d.n_basis[1], d.nout)) {
            const int np = (int)f2_pairs_per_tile(p->dtype);
            p->f2_ok[g] = f2_forward_tile_tiling(p->lb1_host[g].data(), d.n_basis[1], d.degree[1], d.n_samples[0],
                                                 d.n_samples[1], d.nout, f2_tile_cols(p->dtype), kF2BatchFwdTarget,
                                                 0, p->f2_fwd[g]) &&
                          f2_adjoint_tiling(p->lb0_host[g].data(), d.n_basis[0], d.degree[0], d.n_samples[0],
                                            d.n_basis[1], d.degree[1], d.n_samples[1], d.nout, np,
                                            f2_align_elems(p->dtype), kF2BatchAdjTarget, 0, p->f2_adj[g]);
        }
        if (!p->f2_ok[g]) rc = batch_scratch(p, g);
    }
    if (!rc) rc = batch_alloc(p, (void **)&p->head, sizeof(unsigned long long), "batch: queue head");
    if (!rc) rc = batch_alloc(p, (void **)&p->f2_head, sizeof(unsigned long long), "batch: fused queue head");
    if (!rc) rc = batch_alloc(p, (void **)&p->dev_f2_grids, 2 * (size_t)n_grids * sizeof(F2Grid),
                              "batch: fused descriptors");
    if (!rc) rc = batch_alloc(p, (void **)&p->status, sizeof(int), "batch: status");
    if (!rc) rc = cuda_check(cudaMemset(p->status, 0, sizeof(int)), "batch: status");
    if (!rc) {
        const int64_t max_passes = 2LL * SG_MAX_NIN * n_grids;
        rc = batch_alloc(p, (void **)&p->done, max_passes * sizeof(int), "batch: counters");
    }
    if (!rc) {
        int dev = 0, sms = 0, per_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        const size_t smem = (size_t)(p->dtype == SG_F64 ? batch_smem_bytes<double>() : batch_smem_bytes<float>());
        if (p->dtype == SG_F64)
            cudaFuncSetAttribute(k_batch<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        else
            cudaFuncSetAttribute(k_batch<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (p->dtype == SG_F64)
            rc = cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch<double>, kBatchThreads, smem), "batch: occupancy");
        else
            rc = cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch<float>, kBatchThreads, smem), "batch: occupancy");
        p->grid_ctas = std::max(1, sms * std::max(1, per_sm));
    }
    if (rc) {
        batch_free(p);
        return rc;
    }
    *out = p;
    return SG_OK;
}

// Pass tables for mode 1 (forward), 2 (adjoint), 3 (both).  Queue order: a stream
// over the grids in which level l (a grid's (l+1)-th forward pass and (l+1)-th adjoint
// pass) of grid g is emitted together with level 0 of grid g + l*kLag.  A pass's
// producer therefore sits kLag grids of work earlier in the queue and is normally
// finished when the consumer is dequeued (no CTA idles in a dependency wait), while
// the intermediates alive at once (~2*kLag grids) still fit in L2.
constexpr int kLag = 16;

static void build_passes(sg_batch_plan *p, const void *const *cps, void *const *evals,
                         const void *const *ebars, void *const *cpbars) {
    const bool f64 = p->dtype == SG_F64;
    const int V = f64 ? 2 : 4;
    const int64_t W = f64 ? warp_width<double>() : warp_width<float>();  // values per warp task
    const size_t es = f64 ? 8 : 4;
    for (int mode = 1; mode <= 3; ++mode) {
        std::vector<BatchPass> &out = p->host_passes[mode];
        out.clear();
        int64_t first = 0;
        std::vector<int32_t> last_fwd(p->n_grids, -1), last_adj(p->n_grids, -1);
        std::vector<const void *> fwd_x(p->n_grids), adj_x(p->n_grids);
        std::vector<int> adj_buf(p->n_grids, 0);
        auto base = [&](int g, int k) {
            const sg_grid_desc &d = p->desc[g];
            BatchPass b;
            memset(&b, 0, sizeof(b));
            b.idx = d.sample_indices[k];
            b.perm = p->perm[g][k];
            b.lb = p->lb[g][k];
            b.ns = d.n_samples[k];
            b.d = d.degree[k];
            b.D = d.degree[k] + 1;
            b.n = d.n_basis[k];
            b.nch = d.nout;
            b.B = (const char *)d.basis_eval[k] + es * (size_t)(b.ns * (b.d + 1) * (int64_t)p->orders[g][k]);
            b.dep = -1;
            return b;
        };
        auto push = [&](BatchPass b) {
            const int64_t units = b.gx * b.gy * b.gz;
            const bool warp = b.kind != kAdjStream;  // all other kinds are warp tasks
            b.tiles = warp ? (units + tasks_per_item(b.kind) - 1) / tasks_per_item(b.kind) : units;
            b.first = first;
            first += b.tiles;
            out.push_back(b);
            return (int32_t)out.size() - 1;
        };
        auto fwd_pass = [&](int g, int k) {
            const sg_grid_desc &d = p->desc[g];
            BatchPass b = base(g, k);
            const bool last = k == d.nin - 1;
            b.X = k == 0 ? cps[g] : fwd_x[g];
            b.Y = last ? evals[g] : p->fwd_scratch[2 * g + (k % 2)];
            b.final_pass = last;
            b.dep = k > 0 ? last_fwd[g] : -1;
            if (k == 0) {
                int64_t Qr = 1;
                for (int i = 1; i < d.nin; ++i) Qr *= d.n_basis[i];
                b.kind = kFwdAxis0;
                b.M = 1;
                b.Q = Qr;
                b.gx = (Qr * d.nout + 31) / 32;  // warp tasks of 32 columns
                b.gy = (b.ns + kFwd0Samples - 1) / kFwd0Samples;  // x sample chunks
                b.gz = 1;
            } else {
                int64_t M = 1, Q = d.nout;
                for (int i = 0; i < k; ++i) M *= d.n_samples[i];
                for (int i = k + 1; i < d.nin; ++i) Q *= d.n_basis[i];
                b.kind = kFwdAxis;
                b.M = M;
                b.Q = Q;
                b.vec = (M % V == 0 && (uintptr_t)b.X % 16 == 0 && (uintptr_t)b.Y % 16 == 0) ? V : 1;
                b.gx = (M + W - 1) / W;
                b.gy = (b.ns + kFwdTaskRows - 1) / kFwdTaskRows;
                b.gz = Q;
            }
            last_fwd[g] = push(b);
            fwd_x[g] = b.Y;
        };
        auto adj_pass = [&](int g, int k) {
            const sg_grid_desc &d = p->desc[g];
            BatchPass b = base(g, k);
            b.X = k == d.nin - 1 ? ebars[g] : adj_x[g];
            b.Y = k == 0 ? cpbars[g] : p->adj_scratch[2 * g + adj_buf[g]];
            adj_buf[g] ^= 1;
            b.dep = k < d.nin - 1 ? last_adj[g] : -1;
            int64_t M = 1, Q = d.nout;
            for (int i = 0; i < k; ++i) M *= d.n_samples[i];
            for (int i = k + 1; i < d.nin; ++i) Q *= d.n_basis[i];
            b.M = M;
            b.Q = Q;
            if (k > 0) {
                b.cc_qt = 32;
                b.gy = (b.n + b.cc_qt - 1) / b.cc_qt;
                b.gz = Q;
                if ((uintptr_t)b.X % 16 == 0) {  // bulk copies need a 16-byte aligned source
                    const int64_t SW = f64 ? stream_width<double>() : stream_width<float>();
                    b.kind = kAdjStream;
                    b.gx = (M + SW - 1) / SW;
                    b.rows = stream_rows_per_stage(M < SW ? M : SW, (int)es);
                } else {
                    b.kind = kAdjAxis;
                    b.vec = 1;  // X unaligned: strided lanes
                    b.gx = (M + W - 1) / W;
                }
            } else {
                b.kind = kAdjAxis0;
                b.gx = (Q + 31) / 32;  // warp tasks of 32 columns
                b.gy = (b.n + kAdj0Chunk - 1) / kAdj0Chunk;  // x chunks of control points
                b.gz = 1;
            }
            last_adj[g] = push(b);
            adj_x[g] = b.Y;
        };
        const bool do_fwd = (mode & 1) && cps && evals;
        const bool do_adj = (mode & 2) && ebars && cpbars;
        int max_levels = 0;
        for (int g = 0; g < p->n_grids; ++g) max_levels = std::max(max_levels, (int)p->desc[g].nin);
        for (int t = 0; t < p->n_grids + (max_levels - 1) * kLag; ++t) {
            for (int level = max_levels - 1; level >= 0; --level) {
                const int g = t - level * kLag;
                if (g < 0 || g >= p->n_grids || level >= p->desc[g].nin) continue;
                if (grid_fused(p, g)) continue;  // in the fused lists instead
                if (do_fwd && cps[g] && evals[g]) fwd_pass(g, level);
                if (do_adj && ebars[g] && cpbars[g]) adj_pass(g, p->desc[g].nin - 1 - level);
            }
        }
        p->n_items[mode] = first;
    }
}

extern "C" int sg_batch_run(sg_batch_plan *p, int32_t what, sg_stream_t stream);
extern "C" int sg_batch_check(sg_batch_plan *p, sg_stream_t stream);

// Tilings of the fused grids for the plan's unit sizes.
static void batch_retile(sg_batch_plan *p) {
    const int np = (int)f2_pairs_per_tile(p->dtype);
    for (int g = 0; g < p->n_grids; ++g) {
        if (!p->f2_ok[g]) continue;
        const sg_grid_desc &d = p->desc[g];
        f2_forward_tile_tiling(p->lb1_host[g].data(), d.n_basis[1], d.degree[1], d.n_samples[0], d.n_samples[1],
                               d.nout, f2_tile_cols(p->dtype), p->f2_fwd_target, 0, p->f2_fwd[g]);
        f2_adjoint_tiling(p->lb0_host[g].data(), d.n_basis[0], d.degree[0], d.n_samples[0], d.n_basis[1],
                          d.degree[1], d.n_samples[1], d.nout, np, f2_align_elems(p->dtype), p->f2_adj_target, 0,
                          p->f2_adj[g]);
    }
}

// Fused unit lists (forward, adjoint) and the per-grid descriptors (2g: forward,
// 2g+1: adjoint).  Each list runs its largest units first (the tail of a launch is
// made of the smallest ones).
static void build_fused(sg_batch_plan *p, const void *const *cps, void *const *evals,
                        const void *const *ebars, void *const *cpbars, std::vector<F2Grid> &descs) {
    const size_t es = p->dtype == SG_F64 ? 8 : 4;
    descs.assign(2 * (size_t)p->n_grids, F2Grid());
    std::vector<std::pair<int64_t, F2Tile>> lists[2];
    for (int g = 0; g < p->n_grids; ++g) {
        if (!grid_fused(p, g)) continue;
        const sg_grid_desc &d = p->desc[g];
        F2Grid b;
        memset(&b, 0, sizeof(b));
        b.idx0 = d.sample_indices[0];
        b.idx1 = d.sample_indices[1];
        b.lb0 = p->lb[g][0];
        b.lb1 = p->lb[g][1];
        b.off0 = p->off0[g];
        b.B0 = (const char *)d.basis_eval[0] + es * (size_t)(d.n_samples[0] * (d.degree[0] + 1) * (int64_t)p->orders[g][0]);
        b.B1 = (const char *)d.basis_eval[1] + es * (size_t)(d.n_samples[1] * (d.degree[1] + 1) * (int64_t)p->orders[g][1]);
        b.ns0 = d.n_samples[0];
        b.ns1 = d.n_samples[1];
        b.n0 = d.n_basis[0];
        b.n1 = d.n_basis[1];
        b.d0 = d.degree[0];
        b.d1 = d.degree[1];
        b.nch = d.nout;
        F2Grid f = b, a = b;
        if (cps && evals && cps[g] && evals[g]) {
            f.X = cps[g];
            f.Y = evals[g];
            for (int64_t i = 0; i < p->f2_fwd[g].count(); ++i) {
                F2Tile t = p->f2_fwd[g].tile(i, 2, d.nout, d.n_samples[0], d.n_samples[1]);
                t.grid = 2 * g;
                f2_tile_columns(p->lb1_host[g].data(), d.n_basis[1], d.degree[1], t.b_lo, t.b_len, t.cb, t.ncol);
                lists[0].push_back({(int64_t)t.a_len * t.G * t.b_len, t});
            }
        }
        if (ebars && cpbars && ebars[g] && cpbars[g]) {
            a.X = ebars[g];
            a.Y = cpbars[g];
            const int32_t *lb0 = p->lb0_host[g].data(), *lb1 = p->lb1_host[g].data();
            for (int64_t i = 0; i < p->f2_adj[g].count(); ++i) {
                F2Tile t = p->f2_adj[g].tile(i, 1, d.nout, d.n_basis[0], d.n_basis[1]);
                t.grid = 2 * g + 1;
                const int64_t s0 = lb0[t.a_lo + t.a_len + d.degree[0]] - lb0[t.a_lo];
                const int64_t s1 = lb1[t.b_lo + t.b_len + d.degree[1]] - lb1[t.b_lo];
                lists[1].push_back({s0 * t.G * s1, t});
            }
        }
        descs[2 * (size_t)g] = f;
        descs[2 * (size_t)g + 1] = a;
    }
    for (int k = 0; k < 2; ++k) {
        std::stable_sort(lists[k].begin(), lists[k].end(),
                         [](const std::pair<int64_t, F2Tile> &x, const std::pair<int64_t, F2Tile> &y) {
                             return x.first > y.first;
                         });
        p->f2_tiles[k].clear();
        for (const auto &e : lists[k]) p->f2_tiles[k].push_back(e.second);
        p->n_f2[k] = (int64_t)p->f2_tiles[k].size();
    }
}

template <typename E>
static int upload(E **dev, const std::vector<E> &h, const char *what) {
    dev_free(*dev);
    *dev = nullptr;
    if (h.empty()) return SG_OK;
    int rc = dev_alloc((void **)dev, h.size() * sizeof(E), what);
    if (!rc) rc = cuda_check(cudaMemcpy(*dev, h.data(), h.size() * sizeof(E), cudaMemcpyHostToDevice), what);
    return rc;
}

static int batch_build(sg_batch_plan *p) {
    const void *const *cps = p->has_fwd ? p->a_cp.data() : nullptr;
    void *const *evals = p->has_fwd ? p->a_ev.data() : nullptr;
    const void *const *ebars = p->has_adj ? p->a_ebar.data() : nullptr;
    void *const *cpbars = p->has_adj ? p->a_cpbar.data() : nullptr;
    build_passes(p, cps, evals, ebars, cpbars);
    std::vector<F2Grid> descs;
    build_fused(p, cps, evals, ebars, cpbars, descs);
    int rc = cuda_check(cudaMemcpy(p->dev_f2_grids, descs.data(), descs.size() * sizeof(F2Grid),
                                   cudaMemcpyHostToDevice), "batch: fused descriptors");
    for (int mode = 1; mode <= 3 && !rc; ++mode)
        rc = upload(&p->dev_passes[mode], p->host_passes[mode], "batch: pass table");
    for (int k = 0; k < 2 && !rc; ++k)
        rc = upload(&p->dev_f2_tiles[k], p->f2_tiles[k], "batch: fused unit list");
    return rc;
}

extern "C" int sg_batch_set_arrays(sg_batch_plan *p, const void *const *control_points,
                                   void *const *evals, const void *const *eval_bars,
                                   void *const *control_points_bars) {
    if (!p) return set_error(SG_ERR_INVALID_ARGUMENT, "batch: plan is NULL");
    const size_t n = (size_t)p->n_grids;
    p->has_fwd = control_points && evals;
    p->has_adj = eval_bars && control_points_bars;
    p->a_cp.assign(n, nullptr);
    p->a_ev.assign(n, nullptr);
    p->a_ebar.assign(n, nullptr);
    p->a_cpbar.assign(n, nullptr);
    for (size_t g = 0; g < n; ++g) {
        if (p->has_fwd) {
            p->a_cp[g] = control_points[g];
            p->a_ev[g] = evals[g];
        }
        if (p->has_adj) {
            p->a_ebar[g] = eval_bars[g];
            p->a_cpbar[g] = control_points_bars[g];
        }
    }
    const int rc = batch_build(p);
    if (rc) return rc;
    p->arrays_set = true;
    return SG_OK;
}

extern "C" int sg_batch_set_strategy(sg_batch_plan *p, int32_t strategy) {
    if (!p) return set_error(SG_ERR_INVALID_ARGUMENT, "batch: plan is NULL");
    if (strategy != SG_STRATEGY_AUTO && strategy != SG_STRATEGY_SEPARABLE && strategy != SG_STRATEGY_FUSED)
        return set_error(SG_ERR_INVALID_ARGUMENT, "batch: unknown strategy %d", strategy);
    p->strategy = strategy;
    for (int g = 0; g < p->n_grids; ++g)
        if (!grid_fused(p, g)) {
            const int rc = batch_scratch(p, g);
            if (rc) return rc;
        }
    return p->arrays_set ? batch_build(p) : SG_OK;
}

// Measured choice of the fused unit sizes: each candidate runs three times on the plan's
// own arrays (forward-only for the forward units, adjoint-only for the adjoint tiles);
// the fastest median is kept.  The arithmetic of every value is the same whatever the
// unit size, so the results do not change, only the time.
extern "C" int sg_batch_tune(sg_batch_plan *p, sg_stream_t stream, int64_t *chosen) {
    if (!p) return set_error(SG_ERR_INVALID_ARGUMENT, "batch: plan is NULL");
    if (!p->arrays_set) return set_error(SG_ERR_INVALID_ARGUMENT, "batch: sg_batch_set_arrays first");
    cudaStream_t s = (cudaStream_t)stream;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int rc = cuda_check(cudaEventCreate(&e0), "batch tune: event");
    if (!rc) rc = cuda_check(cudaEventCreate(&e1), "batch tune: event");
    static const int64_t kFwd[] = {1 << 13, 1 << 14, 1 << 15, 1 << 16, 1 << 17};
    static const int64_t kAdj[] = {0, 1 << 16, 1 << 17, 1 << 18, 1 << 19};
    for (int kind = 0; kind < 2 && !rc; ++kind) {
        const int what = kind == 0 ? SG_BATCH_FORWARD : SG_BATCH_ADJOINT;
        if ((kind == 0 && !p->has_fwd) || (kind == 1 && !p->has_adj)) continue;
        const int64_t *cand = kind == 0 ? kFwd : kAdj;
        float best = 3.4e38f;
        int64_t best_t = kind == 0 ? p->f2_fwd_target : p->f2_adj_target;
        for (int c = 0; c < 5 && !rc; ++c) {
            (kind == 0 ? p->f2_fwd_target : p->f2_adj_target) = cand[c];
            batch_retile(p);
            rc = batch_build(p);
            float ms[3];
            for (int r = 0; r < 3 && !rc; ++r) {
                rc = cuda_check(cudaEventRecord(e0, s), "batch tune: record");
                if (!rc) rc = sg_batch_run(p, what, stream);
                if (!rc) rc = cuda_check(cudaEventRecord(e1, s), "batch tune: record");
                if (!rc) rc = cuda_check(cudaEventSynchronize(e1), "batch tune: sync");
                if (!rc) rc = cuda_check(cudaEventElapsedTime(&ms[r], e0, e1), "batch tune: time");
            }
            if (rc) break;
            std::sort(ms, ms + 3);
            if (ms[1] < best) {
                best = ms[1];
                best_t = cand[c];
            }
        }
        (kind == 0 ? p->f2_fwd_target : p->f2_adj_target) = best_t;
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    batch_retile(p);
    if (!rc) rc = batch_build(p);
    if (!rc) rc = sg_batch_check(p, stream);
    if (chosen) {
        chosen[0] = p->f2_fwd_target;
        chosen[1] = p->f2_adj_target;
    }
    return rc;
}

// Back to the built-in unit sizes (or explicit ones: a target <= 0 keeps the default).
extern "C" int sg_batch_set_unit_sizes(sg_batch_plan *p, int64_t fwd_values, int64_t adj_values) {
    if (!p) return set_error(SG_ERR_INVALID_ARGUMENT, "batch: plan is NULL");
    p->f2_fwd_target = fwd_values > 0 ? fwd_values : kF2BatchFwdTarget;
    p->f2_adj_target = adj_values > 0 ? adj_values : kF2BatchAdjTarget;
    batch_retile(p);
    return p->arrays_set ? batch_build(p) : SG_OK;
}

extern "C" int64_t sg_batch_fused_grids(const sg_batch_plan *p) {
    if (!p) return 0;
    int64_t c = 0;
    for (int g = 0; g < p->n_grids; ++g) c += grid_fused(p, g) ? 1 : 0;
    return c;
}

extern "C" int sg_batch_run(sg_batch_plan *p, int32_t what, sg_stream_t stream) {
    if (!p) return set_error(SG_ERR_INVALID_ARGUMENT, "batch: plan is NULL");
    if (what < 1 || what > 3) return set_error(SG_ERR_INVALID_ARGUMENT, "batch: what must be 1, 2 or 3");
    if (!p->arrays_set) return set_error(SG_ERR_INVALID_ARGUMENT, "batch: sg_batch_set_arrays first");
    const auto &h = p->host_passes[what];
    const int64_t nf = (what & 1) ? p->n_f2[0] : 0, na = (what & 2) ? p->n_f2[1] : 0;
    if (h.empty() && nf == 0 && na == 0)
        return set_error(SG_ERR_INVALID_ARGUMENT, "batch: no arrays for this mode");
    cudaStream_t s = (cudaStream_t)stream;
    int rc = cuda_check(cudaMemsetAsync(p->status, 0, sizeof(int), s), "batch: reset");
    // the fused Nin = 2 grids: one launch per direction
    if (!rc && nf)
        rc = f2_launch_batch(p->dtype, 2, p->dev_f2_grids, p->dev_f2_tiles[0], nf, nullptr, p->status, s);
    if (!rc && na) {
        rc = cuda_check(cudaMemsetAsync(p->f2_head, 0, sizeof(unsigned long long), s), "batch: reset");
        if (!rc)
            rc = f2_launch_batch(p->dtype, 1, p->dev_f2_grids, p->dev_f2_tiles[1], na, p->f2_head, p->status, s);
    }
    if (rc || h.empty()) return rc;
    rc = cuda_check(cudaMemsetAsync(p->done, 0, h.size() * sizeof(int), s), "batch: reset");
    if (!rc) rc = cuda_check(cudaMemsetAsync(p->head, 0, sizeof(unsigned long long), s), "batch: reset");
    if (rc) return rc;
    const int64_t items = p->n_items[what];
    const unsigned grid = (unsigned)std::min<int64_t>(p->grid_ctas, std::max<int64_t>(1, items));
    if (p->dtype == SG_F64)
        k_batch<double><<<grid, kBatchThreads, batch_smem_bytes<double>(), s>>>(
            p->dev_passes[what], (int32_t)h.size(), items, p->head, p->done, p->status,
            p->profile ? p->prof : nullptr, g_batch_spin_limit, g_batch_dep_extra);
    else
        k_batch<float><<<grid, kBatchThreads, batch_smem_bytes<float>(), s>>>(
            p->dev_passes[what], (int32_t)h.size(), items, p->head, p->done, p->status,
            p->profile ? p->prof : nullptr, g_batch_spin_limit, g_batch_dep_extra);
    return cuda_check(cudaGetLastError(), "k_batch launch");
}

extern "C" int sg_batch_enable_profile(sg_batch_plan *p, int32_t enable) {
    if (!p) return set_error(SG_ERR_INVALID_ARGUMENT, "batch: plan is NULL");
    if (enable && !p->prof) {
        int rc = batch_alloc(p, (void **)&p->prof, SG_BATCH_PROFILE_WORDS * sizeof(unsigned long long),
                             "batch: profile");
        if (!rc) rc = cuda_check(cudaMemset(p->prof, 0, SG_BATCH_PROFILE_WORDS * sizeof(unsigned long long)),
                                 "batch: profile");
        if (rc) return rc;
    }
    p->profile = enable != 0;
    return SG_OK;
}

extern "C" int sg_batch_profile(sg_batch_plan *p, sg_stream_t stream, int64_t *out) {
    if (!p || !out) return set_error(SG_ERR_INVALID_ARGUMENT, "batch: plan or out is NULL");
    if (!p->prof) return set_error(SG_ERR_INVALID_ARGUMENT, "batch: profiling was never enabled");
    cudaStream_t s = (cudaStream_t)stream;
    int rc = cuda_check(cudaMemcpyAsync(out, p->prof, SG_BATCH_PROFILE_WORDS * sizeof(int64_t),
                                        cudaMemcpyDeviceToHost, s), "batch: read profile");
    if (!rc) rc = cuda_check(cudaStreamSynchronize(s), "batch: sync");
    if (!rc) rc = cuda_check(cudaMemsetAsync(p->prof, 0, SG_BATCH_PROFILE_WORDS * sizeof(int64_t), s),
                             "batch: reset profile");
    return rc;
}

extern "C" int sg_batch_check(sg_batch_plan *p, sg_stream_t stream) {
    if (!p) return set_error(SG_ERR_INVALID_ARGUMENT, "batch: plan is NULL");
    int st = 0;
    int rc = cuda_check(cudaMemcpyAsync(&st, p->status, sizeof(int), cudaMemcpyDeviceToHost,
                                        (cudaStream_t)stream), "batch: read status");
    if (!rc) rc = cuda_check(cudaStreamSynchronize((cudaStream_t)stream), "batch: sync");
    if (rc) return rc;
    if (st == SG_ERR_TIMEOUT)
        return set_error(SG_ERR_TIMEOUT, "batch: a dependency wait of the persistent kernel gave up");
    return SG_OK;
}

extern "C" void sg_batch_plan_destroy(sg_batch_plan *p) {
    if (p) batch_free(p);
}

extern "C" int64_t sg_batch_plan_workspace_bytes(const sg_batch_plan *p) {
    if (!p) return 0;
    int64_t tot = 0;
    const int64_t es = p->dtype == SG_F64 ? 8 : 4;
    for (int g = 0; g < p->n_grids; ++g) {
        if (!p->scratch_done[g]) continue;  // fused grids have no intermediates
        const int nbuf = p->desc[g].nin >= 3 ? 2 : (p->desc[g].nin == 2 ? 1 : 0);
        tot += 2 * nbuf * p->scratch_elems[g] * es;
    }
    return tot;
}

extern "C" int64_t sg_batch_items(const sg_batch_plan *p, int32_t what) {
    if (!p || what < 1 || what > 3) return 0;
    return p->n_items[what] + ((what & 1) ? p->n_f2[0] : 0) + ((what & 2) ? p->n_f2[1] : 0);
}

// One cudaMemcpyAsync per entry, issued from here so that a host-data step of many grids
// costs one call per direction instead of one per array.
extern "C" int sg_copy_list(int64_t n, void *const *dst, const void *const *src,
                            const int64_t *bytes, sg_stream_t stream) {
    if (n < 0 || (n > 0 && (!dst || !src || !bytes)))
        return set_error(SG_ERR_INVALID_ARGUMENT, "sg_copy_list: bad arguments");
    for (int64_t i = 0; i < n; ++i) {
        if (bytes[i] < 0 || (bytes[i] > 0 && (!dst[i] || !src[i])))
            return set_error(SG_ERR_INVALID_ARGUMENT, "sg_copy_list: entry %lld", (long long)i);
        if (bytes[i] == 0) continue;
        const int rc = cuda_check(cudaMemcpyAsync(dst[i], src[i], (size_t)bytes[i], cudaMemcpyDefault,
                                                  (cudaStream_t)stream),
                                  "sg_copy_list: copy");
        if (rc) return rc;
    }
    return SG_OK;
}

extern "C" int sg_test_set_wait_limits(int64_t batch_spin_limit, int64_t mbar_wait_cycles) {
    g_batch_spin_limit = batch_spin_limit > 0 ? (unsigned)std::min<int64_t>(batch_spin_limit, 0xffffffffLL)
                                              : kSpinLimit;
    return f2_set_wait_cycles(mbar_wait_cycles);
}

extern "C" int sg_test_block_waits(int32_t batch_dependency, int32_t fused_first_stage) {
    g_batch_dep_extra = batch_dependency ? 1 : 0;
    return f2_set_withhold_first_stage(fused_first_stage != 0);
}
