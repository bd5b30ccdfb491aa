// sg_api.cu -- C ABI entry points for grid plans, evaluate! and evaluate_adjoint!.
//
// A plan holds what one SplineGrid hands to its kernels (src/spline_grid.jl:211-214)
// plus the device scratch of the separable passes.  evaluate! runs Nin passes
// (axis 0 first, the last pass writes eval); evaluate_adjoint! runs them in reverse
// (the first pass reads the cotangent).  See sg_contract.cuh for the passes.
#include <algorithm>
#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <numeric>
#include <vector>

#include "sg_passes.cuh"
#include "sg_fused2d_host.h"

namespace sg {

static thread_local char g_err[1024] = "";

int set_error(int code, const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    return code;
}

int cuda_check(cudaError_t e, const char *what) {
    if (e == cudaSuccess) return SG_OK;
    return set_error(e == cudaErrorMemoryAllocation ? SG_ERR_OUT_OF_MEMORY : SG_ERR_CUDA,
                     "%s: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
}

static size_t elem_size(int dtype) { return dtype == SG_F64 ? 8 : 4; }

// Device allocations of plans and handles.  A test hook can make every allocation after
// the next `after` ones fail, as cudaMalloc does when the device is full; the count of
// live allocations shows that a failed create released what it had taken.
static std::atomic<int64_t> g_alloc_budget{-1};  // < 0: no injected failures
static std::atomic<int64_t> g_live_allocs{0};

int dev_alloc(void **out, size_t bytes, const char *what) {
    *out = nullptr;
    int64_t b = g_alloc_budget.load();
    while (b >= 0) {
        if (b == 0)
            return set_error(SG_ERR_OUT_OF_MEMORY, "%s: cudaErrorMemoryAllocation (injected by the "
                                                   "allocation-failure test hook)", what);
        if (g_alloc_budget.compare_exchange_weak(b, b - 1)) break;
    }
    const int rc = cuda_check(cudaMalloc(out, bytes ? bytes : 16), what);
    if (!rc) g_live_allocs.fetch_add(1);
    else *out = nullptr;
    return rc;
}

void dev_free(void *p) {
    if (!p) return;
    cudaFree(p);
    g_live_allocs.fetch_sub(1);
}

}  // namespace sg

extern "C" int sg_test_fail_allocations(int64_t after) {
    sg::g_alloc_budget.store(after < 0 ? -1 : after);
    return SG_OK;
}

extern "C" int64_t sg_test_live_allocations(void) { return sg::g_live_allocs.load(); }

struct sg_grid_plan {
    sg_grid_desc desc;
    int device = 0;
    void *scratch[2] = {nullptr, nullptr};
    int64_t scratch_elems = 0;
    int32_t *perm[SG_MAX_NIN] = {};  // device; NULL when the axis is sorted
    // device support tables: lb[k][c + d] = first position of the sorted sample view
    // whose support start is >= c, for c in [-d, n] (adjoint sample ranges)
    int32_t *lb[SG_MAX_NIN] = {};
    // axis 0: off0[c] = number of (sample, control point) incidences of control points
    // below c (offsets of the fused adjoint's weight list); device, n_basis[0] + 1 values
    int32_t *off0 = nullptr;
    // device status word: SG_ERR_TIMEOUT when a bounded wait of a streaming pass gave up
    int *status = nullptr;
    // adjoint stream chunk size per axis chosen by sg_grid_plan_tune (0: heuristic)
    int32_t tuned_cc[SG_MAX_NIN] = {};
    // Nin = 2: the fused single-launch path (sg_fused2d.cuh) when the grid fits it
    int32_t strategy = SG_STRATEGY_AUTO;
    bool f2_fwd_ok = false, f2_adj_ok = false;
    sg::F2Tiling f2_fwd, f2_adj;
    int64_t f2_adj_target = 0;      // cotangent values per adjoint tile (0: the wave model)
    std::vector<int32_t> lb0_host;  // axis-0 support table (host copy, for re-tiling)
    std::vector<int32_t> lb1_host;  // axis-1 support table (host copy, forward tiles)
    bool sorted_all = true, sorted1 = true;
    int32_t f2_fwd_kind = 0;        // fused forward: 0 warp tasks, 2 tiles (sorted axis 1)
    // optional per-pass timing: events[2*i], events[2*i+1] bracket pass i
    bool timing = false;
    cudaEvent_t events[2 * SG_MAX_NIN] = {};
    int n_timed = 0;
};

namespace {
struct PassTimer {
    sg_grid_plan *p;
    cudaStream_t s;
    int i = 0;
    PassTimer(sg_grid_plan *p_, cudaStream_t s_) : p(p_), s(s_) { p->n_timed = 0; }
    void begin() {
        if (p->timing && i < SG_MAX_NIN) cudaEventRecord(p->events[2 * i], s);
    }
    void end() {
        if (p->timing && i < SG_MAX_NIN) {
            cudaEventRecord(p->events[2 * i + 1], s);
            p->n_timed = ++i;
        }
    }
};
}  // namespace

using namespace sg;

extern "C" int sg_version(void) { return 100; }

extern "C" const char *sg_last_error(void) { return g_err; }

static int validate_desc(const sg_grid_desc *d) {
    if (!d) return set_error(SG_ERR_INVALID_ARGUMENT, "grid descriptor is NULL");
    if (d->nin < 1 || d->nin > SG_MAX_NIN)
        return set_error(SG_ERR_INVALID_ARGUMENT, "nin=%d outside 1..%d", d->nin, SG_MAX_NIN);
    if (d->nout < 1) return set_error(SG_ERR_INVALID_ARGUMENT, "nout=%d must be >= 1", d->nout);
    if (d->dtype != SG_F32 && d->dtype != SG_F64 && d->dtype != SG_BF16_F32)
        return set_error(SG_ERR_INVALID_ARGUMENT, "unknown dtype %d", d->dtype);
    for (int k = 0; k < d->nin; ++k) {
        if (d->degree[k] < 0 || d->degree[k] > SG_MAX_DEGREE)
            return set_error(SG_ERR_UNSUPPORTED, "dimension %d: degree %d outside 0..%d", k + 1,
                             d->degree[k], SG_MAX_DEGREE);
        if (d->n_basis[k] < d->degree[k] + 1)
            return set_error(SG_ERR_INVALID_ARGUMENT,
                             "dimension %d: %lld basis functions for degree %d "
                             "(src/knot_vector.jl:84 needs n_basis - degree >= 1)",
                             k + 1, (long long)d->n_basis[k], d->degree[k]);
        if (d->max_derivative_order[k] < 0 || d->max_derivative_order[k] > d->degree[k])
            return set_error(SG_ERR_INVALID_ARGUMENT,
                             "dimension %d: max_derivative_order %d outside 0..degree", k + 1,
                             d->max_derivative_order[k]);
        if (d->n_samples[k] < 0)
            return set_error(SG_ERR_INVALID_ARGUMENT, "dimension %d: negative sample count", k + 1);
        if (d->n_samples[k] > 0 && (!d->sample_indices[k] || !d->basis_eval[k]))
            return set_error(SG_ERR_INVALID_ARGUMENT, "dimension %d: NULL indices or basis", k + 1);
        if (d->n_samples[k] > INT32_MAX)
            return set_error(SG_ERR_UNSUPPORTED, "dimension %d: more than 2^31-1 samples", k + 1);
        if (d->n_basis[k] > INT32_MAX)
            return set_error(SG_ERR_UNSUPPORTED, "dimension %d: more than 2^31-1 control points",
                             k + 1);
    }
    return SG_OK;
}

// Reads the sample indices of every axis, checks that they address a valid support
// (1-based idx in [degree+1, n_basis], the clamp range of src/util_kernels.jl:43-47),
// and builds the sorted view of any unsorted axis.
// Whether (and how) the fused Nin = 2 path takes this grid: degrees <= 3, 32-bit
// element offsets, no weights; the adjoint also needs sorted samples on both axes and
// axis-0 supports that fit a tile.  The grid runs alone, so the tilings are sized for
// whole waves of the resident units.
static void plan_fused_tilings(sg_grid_plan *p) {
    const sg_grid_desc &d = p->desc;
    p->f2_fwd_ok = p->f2_adj_ok = false;
    if (d.nin != 2 || d.has_weights || d.degree[0] > 3 || d.degree[1] > 3) return;
    if (d.n_samples[0] < 1 || d.n_samples[1] < 1) return;
    if (!f2_offsets_fit(d.n_samples[0], d.n_samples[1], d.n_basis[0], d.n_basis[1], d.nout)) return;
    const int dt = d.dtype == SG_F64 ? SG_F64 : SG_F32;
    const int np = (int)f2_pairs_per_tile(dt);
    p->f2_fwd_kind = 0;
    if (p->sorted1 && !p->lb1_host.empty() &&
        f2_forward_tile_tiling(p->lb1_host.data(), d.n_basis[1], d.degree[1], d.n_samples[0], d.n_samples[1],
                               d.nout, f2_tile_cols(dt), 0, f2_slots(dt, 2), p->f2_fwd)) {
        p->f2_fwd_ok = true;
        p->f2_fwd_kind = 2;
    } else {
        p->f2_fwd_ok = f2_forward_tiling(d.n_samples[0], d.n_samples[1], d.nout, 0, f2_slots(dt, 0),
                                         p->f2_fwd);
    }
    if (p->sorted_all && !p->lb0_host.empty())
        p->f2_adj_ok = f2_adjoint_tiling(p->lb0_host.data(), d.n_basis[0], d.degree[0], d.n_samples[0],
                                         d.n_basis[1], d.degree[1], d.n_samples[1], d.nout, np,
                                         f2_align_elems(dt), p->f2_adj_target,
                                         p->f2_adj_target > 0 ? 0 : f2_slots(dt, 1),
                                         p->f2_adj);
}

static int plan_scan_indices(sg_grid_plan *p, cudaStream_t s) {
    const sg_grid_desc &d = p->desc;
    p->lb0_host.clear();
    p->sorted_all = true;
    p->sorted1 = true;
    p->lb1_host.clear();
    for (int k = 0; k < d.nin; ++k) {
        if (p->perm[k]) {
            dev_free(p->perm[k]);
            p->perm[k] = nullptr;
        }
        if (p->lb[k]) {
            dev_free(p->lb[k]);
            p->lb[k] = nullptr;
        }
        const int64_t ns = d.n_samples[k];
        if (ns == 0) continue;
        std::vector<int32_t> h(ns);
        int rc = cuda_check(cudaMemcpyAsync(h.data(), d.sample_indices[k], ns * sizeof(int32_t),
                                            cudaMemcpyDeviceToHost, s),
                            "plan: read sample indices");
        if (!rc) rc = cuda_check(cudaStreamSynchronize(s), "plan: sync");
        if (rc) return rc;
        bool sorted = true;
        for (int64_t j = 0; j < ns; ++j) {
            if (h[j] < d.degree[k] + 1 || h[j] > d.n_basis[k])
                return set_error(SG_ERR_INVALID_ARGUMENT,
                                 "dimension %d: sample index %d at sample %lld outside [%d, %lld]",
                                 k + 1, h[j], (long long)(j + 1), d.degree[k] + 1,
                                 (long long)d.n_basis[k]);
            if (j > 0 && h[j] < h[j - 1]) sorted = false;
        }
        std::vector<int32_t> perm(ns);
        std::iota(perm.begin(), perm.end(), 0);
        if (!sorted) {
            std::stable_sort(perm.begin(), perm.end(),
                             [&](int32_t a, int32_t b) { return h[a] < h[b]; });
            rc = dev_alloc((void **)&p->perm[k], ns * sizeof(int32_t), "plan: perm");
            if (!rc)
                rc = cuda_check(cudaMemcpy(p->perm[k], perm.data(), ns * sizeof(int32_t),
                                           cudaMemcpyHostToDevice),
                                "plan: upload perm");
            if (rc) return rc;
        }
        // support table: support start of view position s is h[perm[s]] - d - 1
        const int dk = d.degree[k];
        const int64_t n = d.n_basis[k];
        std::vector<int32_t> lb(n + dk + 1);
        int64_t s_pos = 0;
        for (int64_t i = 0; i <= n + dk; ++i) {
            const int64_t c = i - dk;
            while (s_pos < ns && (int64_t)h[perm[s_pos]] - dk - 1 < c) ++s_pos;
            lb[i] = (int32_t)s_pos;
        }
        rc = dev_alloc((void **)&p->lb[k], lb.size() * sizeof(int32_t), "plan: lb");
        if (!rc)
            rc = cuda_check(cudaMemcpy(p->lb[k], lb.data(), lb.size() * sizeof(int32_t),
                                       cudaMemcpyHostToDevice),
                            "plan: upload support table");
        if (rc) return rc;
        p->sorted_all = p->sorted_all && sorted;
        if (k == 1) {
            p->sorted1 = sorted;
            p->lb1_host = lb;
        }
        if (k == 0) {
            const std::vector<int32_t> off = f2_weight_offsets(lb.data(), n, dk);
            dev_free(p->off0);
            p->off0 = nullptr;
            rc = dev_alloc((void **)&p->off0, off.size() * sizeof(int32_t), "plan: weight offsets");
            if (!rc)
                rc = cuda_check(cudaMemcpy(p->off0, off.data(), off.size() * sizeof(int32_t),
                                           cudaMemcpyHostToDevice),
                                "plan: upload weight offsets");
            if (rc) return rc;
            p->lb0_host.swap(lb);
        }
    }
    plan_fused_tilings(p);
    return SG_OK;
}

// Largest intermediate tensor of the separable passes: after contracting axes
// 0..k-1 the tensor is [ns_0..ns_{k-1}, n_k..n_{nin-1}, channels].
static int64_t scratch_elems_for(const sg_grid_desc &d) {
    const int64_t ch = d.nout + (d.has_weights ? 1 : 0);
    int64_t best = 0;
    for (int k = 1; k < d.nin; ++k) {
        int64_t e = ch;
        for (int i = 0; i < d.nin; ++i) e *= (i < k) ? d.n_samples[i] : d.n_basis[i];
        best = std::max(best, e);
    }
    return best;
}

extern "C" int sg_grid_plan_create(const sg_grid_desc *desc, sg_stream_t stream,
                                   sg_grid_plan **out) {
    if (!out) return set_error(SG_ERR_INVALID_ARGUMENT, "plan output pointer is NULL");
    *out = nullptr;
    int rc = validate_desc(desc);
    if (rc) return rc;
    sg_grid_plan *p = new (std::nothrow) sg_grid_plan();
    if (!p) return set_error(SG_ERR_OUT_OF_MEMORY, "plan: host allocation failed");
    p->desc = *desc;
    cudaGetDevice(&p->device);
    cudaStream_t s = (cudaStream_t)stream;
    rc = plan_scan_indices(p, s);
    if (!rc) {
        p->scratch_elems = scratch_elems_for(p->desc);
        const int nbuf = p->desc.nin >= 3 ? 2 : (p->desc.nin == 2 ? 1 : 0);
        const size_t es = (p->desc.dtype == SG_F64) ? 8 : 4;
        for (int b = 0; b < nbuf && !rc; ++b)
            rc = dev_alloc(&p->scratch[b], (size_t)p->scratch_elems * es, "plan: scratch allocation");
    }
    if (!rc) rc = dev_alloc((void **)&p->status, sizeof(int), "plan: status");
    if (!rc) rc = cuda_check(cudaMemsetAsync(p->status, 0, sizeof(int), s), "plan: status");
    if (rc) {
        sg_grid_plan_destroy(p);
        return rc;
    }
    *out = p;
    return SG_OK;
}

extern "C" int sg_grid_plan_refresh(sg_grid_plan *p, sg_stream_t stream) {
    if (!p) return set_error(SG_ERR_INVALID_ARGUMENT, "plan is NULL");
    return plan_scan_indices(p, (cudaStream_t)stream);
}

extern "C" int sg_grid_plan_enable_timing(sg_grid_plan *p, int32_t enable) {
    if (!p) return set_error(SG_ERR_INVALID_ARGUMENT, "plan is NULL");
    if (enable && !p->events[0]) {
        for (int i = 0; i < 2 * SG_MAX_NIN; ++i) {
            int rc = cuda_check(cudaEventCreate(&p->events[i]), "timing: event create");
            if (rc) return rc;
        }
    }
    p->timing = enable != 0;
    p->n_timed = 0;
    return SG_OK;
}

extern "C" int sg_grid_plan_pass_times(sg_grid_plan *p, float *ms, int32_t *n_passes) {
    if (!p || !n_passes) return set_error(SG_ERR_INVALID_ARGUMENT, "plan or n_passes is NULL");
    const int cap = *n_passes;
    *n_passes = p->n_timed;
    for (int i = 0; i < p->n_timed && i < cap; ++i) {
        int rc = cuda_check(cudaEventSynchronize(p->events[2 * i + 1]), "timing: sync");
        if (!rc) rc = cuda_check(cudaEventElapsedTime(&ms[i], p->events[2 * i],
                                                      p->events[2 * i + 1]), "timing: elapsed");
        if (rc) return rc;
    }
    return SG_OK;
}

extern "C" int sg_grid_plan_check(sg_grid_plan *p, sg_stream_t stream) {
    if (!p) return set_error(SG_ERR_INVALID_ARGUMENT, "plan is NULL");
    int st = 0;
    int rc = cuda_check(cudaMemcpyAsync(&st, p->status, sizeof(int), cudaMemcpyDeviceToHost,
                                        (cudaStream_t)stream), "plan: read status");
    if (!rc) rc = cuda_check(cudaStreamSynchronize((cudaStream_t)stream), "plan: sync");
    if (rc) return rc;
    if (st == SG_OK) return SG_OK;
    rc = cuda_check(cudaMemset(p->status, 0, sizeof(int)), "plan: reset status");
    if (rc) return rc;
    return set_error(SG_ERR_TIMEOUT, "a bounded wait of an adjoint pass gave up; its results are invalid");
}

extern "C" void sg_grid_plan_destroy(sg_grid_plan *p) {
    if (!p) return;
    dev_free(p->status);
    for (int i = 0; i < 2 * SG_MAX_NIN; ++i)
        if (p->events[i]) cudaEventDestroy(p->events[i]);
    for (int b = 0; b < 2; ++b)
        dev_free(p->scratch[b]);
    for (int k = 0; k < SG_MAX_NIN; ++k) {
        dev_free(p->perm[k]);
        dev_free(p->lb[k]);
    }
    dev_free(p->off0);
    delete p;
}

extern "C" int64_t sg_grid_plan_workspace_bytes(const sg_grid_plan *p) {
    if (!p) return 0;
    const int nbuf = p->desc.nin >= 3 ? 2 : (p->desc.nin == 2 ? 1 : 0);
    return nbuf * p->scratch_elems * (p->desc.dtype == SG_F64 ? 8 : 4);
}

// derivative_order checks of src/validation.jl:52-88 with the reference's messages.
// The derivative orders a call asks for, checked as the reference's
// validate_partial_derivatives does (src/validation.jl:76-102): NURBS grids take none,
// and an order above the dimension's max_derivative_order is refused with its message.
// Shared with sg_evaluate_noalloc.
int sg::check_orders(const sg_grid_desc &d, const int32_t *ord) {
    if (!ord) return set_error(SG_ERR_INVALID_ARGUMENT, "derivative_order is NULL");
    if (d.has_weights) {
        for (int k = 0; k < d.nin; ++k)
            if (ord[k] != 0)
                return set_error(SG_ERR_UNSUPPORTED,
                                 "Computing derivatives of NURBS is currently not supported.");
    }
    for (int k = 0; k < d.nin; ++k) {
        if (ord[k] < 0 || ord[k] > d.max_derivative_order[k])
            return set_error(
                SG_ERR_INVALID_ARGUMENT,
                "The maximum derivative order available for spline dimension %d is %d, got %d. "
                "Invalid derivative order(s) supplied. If you want to evaluate (higher order) "
                "derivatives, specify this at construction as "
                "SplineDimension(...; max_derivative_order).",
                k + 1, d.max_derivative_order[k], ord[k]);
    }
    return SG_OK;
}

static AxisPass axis_pass(const sg_grid_desc &d, const sg_grid_plan *p, int k,
                          const int32_t *ord) {
    AxisPass a;
    a.idx = d.sample_indices[k];
    a.perm = p->perm[k];
    a.lb = p->lb[k];
    a.status = p->status;
    a.ns = d.n_samples[k];
    a.d = d.degree[k];
    a.n = d.n_basis[k];
    const size_t bes = (d.dtype == SG_F64) ? 8 : 4;  // basis tables are F32 in BF16 mode
    a.B = (const char *)d.basis_eval[k] + bes * (size_t)(a.ns * (a.d + 1) * (int64_t)ord[k]);
    a.cc = p->tuned_cc[k];
    return a;
}

// The fused Nin = 2 path's view of the grid for one derivative order.
static F2Grid f2_grid(const sg_grid_plan *p, const int32_t *ord, const void *X, void *Y) {
    const sg_grid_desc &d = p->desc;
    F2Grid g;
    memset(&g, 0, sizeof(g));
    const size_t bes = (d.dtype == SG_F64) ? 8 : 4;  // basis tables are F32 in BF16 mode
    g.idx0 = d.sample_indices[0];
    g.idx1 = d.sample_indices[1];
    g.lb0 = p->lb[0];
    g.lb1 = p->lb[1];
    g.off0 = p->off0;
    g.B0 = (const char *)d.basis_eval[0] + bes * (size_t)(d.n_samples[0] * (d.degree[0] + 1) * (int64_t)ord[0]);
    g.B1 = (const char *)d.basis_eval[1] + bes * (size_t)(d.n_samples[1] * (d.degree[1] + 1) * (int64_t)ord[1]);
    g.X = X;
    g.Y = Y;
    g.ns0 = d.n_samples[0];
    g.ns1 = d.n_samples[1];
    g.n0 = d.n_basis[0];
    g.n1 = d.n_basis[1];
    g.d0 = d.degree[0];
    g.d1 = d.degree[1];
    g.nch = d.nout;
    return g;
}

static bool use_fused(const sg_grid_plan *p, bool ok) {
    return ok && p->strategy != SG_STRATEGY_SEPARABLE;
}

// Forward pass k (contract axis k) of one derivative order: X -> Y.  Only order[k] is
// read; the last pass writes eval (NURBS: and divides).
static int forward_pass(sg_grid_plan *p, int k, const int32_t *order, const void *X, void *Y,
                        const void *weights, cudaStream_t s, PassTimer &timer) {
    const sg_grid_desc &d = p->desc;
    const bool f64 = d.dtype == SG_F64;
    const bool nurbs = d.has_weights != 0;
    const int64_t ch = d.nout + (nurbs ? 1 : 0);
    AxisPass a = axis_pass(d, p, k, order);
    const bool last = (k == d.nin - 1);
    a.X = X;
    a.Y = Y;
    a.nch = d.nout;
    a.final_pass = last;
    int rc;
    if (k == 0) {
        a.M = 1;
        int64_t Qr = 1;
        for (int i = 1; i < d.nin; ++i) Qr *= d.n_basis[i];
        a.Q = Qr;  // kPlain multiplies by nch itself; kHomog by nch+1
        a.w = weights;
        a.mode = !nurbs ? kPlain : (last ? kRational : kHomog);
        a.x_dtype = d.dtype;
        timer.begin();
        rc = f64 ? fwd_axis0_f64(a, s) : fwd_axis0_f32(a, s);
        timer.end();
    } else {
        int64_t M = 1, Q = ch;
        for (int i = 0; i < k; ++i) M *= d.n_samples[i];
        for (int i = k + 1; i < d.nin; ++i) Q *= d.n_basis[i];
        a.M = M;
        a.Q = Q;
        a.mode = (nurbs && last) ? kRational : kPlain;
        timer.begin();
        rc = f64 ? fwd_axis_f64(a, s) : fwd_axis_f32(a, s);
        timer.end();
    }
    return rc;
}

static int forward_checks(sg_grid_plan *p, const void *control_points, const void *weights,
                          int64_t &V) {
    if (!p) return set_error(SG_ERR_INVALID_ARGUMENT, "plan is NULL");
    const sg_grid_desc &d = p->desc;
    if (d.has_weights && !weights)
        return set_error(SG_ERR_INVALID_ARGUMENT, "NURBS grid evaluated without weights");
    if (!d.has_weights && weights)
        return set_error(SG_ERR_INVALID_ARGUMENT, "weights given for a non-NURBS grid");
    V = 1;
    for (int k = 0; k < d.nin; ++k) V *= d.n_samples[k];
    if (V > 0 && !control_points) return set_error(SG_ERR_INVALID_ARGUMENT, "control_points is NULL");
    return SG_OK;
}

extern "C" int sg_evaluate(sg_grid_plan *p, const int32_t *derivative_order,
                           const void *control_points, const void *weights, void *eval,
                           sg_stream_t stream) {
    int64_t V = 0;
    int rc = forward_checks(p, control_points, weights, V);
    if (rc) return rc;
    const sg_grid_desc &d = p->desc;
    rc = check_orders(d, derivative_order);
    if (rc) return rc;
    if (V == 0) return SG_OK;
    if (!eval) return set_error(SG_ERR_INVALID_ARGUMENT, "control_points or eval is NULL");
    cudaStream_t s = (cudaStream_t)stream;
    PassTimer timer(p, s);
    if (use_fused(p, p->f2_fwd_ok)) {  // Nin = 2: both axes in one launch
        timer.begin();
        rc = f2_launch_grid(d.dtype, f2_grid(p, derivative_order, control_points, eval), p->f2_fwd,
                            p->f2_fwd_kind, p->status, s);
        timer.end();
        return rc;
    }
    const void *X = control_points;
    for (int k = 0; k < d.nin; ++k) {
        void *Y = (k == d.nin - 1) ? eval : p->scratch[k % 2];
        rc = forward_pass(p, k, derivative_order, X, Y, weights, s, timer);
        if (rc) return rc;
        X = Y;
    }
    return SG_OK;
}

// Depth-first walk of the prefix tree of the requested orders: the intermediate after
// axes 0..k depends only on orders[.][0..k], so every distinct prefix is contracted
// once.  `ix[lo, hi)` are order indices sorted lexicographically, sharing the prefix of
// length k; X is that prefix's intermediate.  Level k's output lives in scratch[k % 2],
// which is free again once the subtree below it is done (Nin <= 3).
static int forward_tree(sg_grid_plan *p, const int32_t *orders, const int *ix, int lo, int hi,
                        int k, const void *X, const void *weights, void *const *evals,
                        cudaStream_t s, PassTimer &timer) {
    const int nin = p->desc.nin;
    if (k == nin - 1) {
        for (int i = lo; i < hi; ++i) {
            const int rc = forward_pass(p, k, orders + (size_t)ix[i] * nin, X, evals[ix[i]],
                                        weights, s, timer);
            if (rc) return rc;
        }
        return SG_OK;
    }
    void *Y = p->scratch[k % 2];
    for (int a = lo; a < hi;) {
        int b = a + 1;
        while (b < hi && orders[(size_t)ix[b] * nin + k] == orders[(size_t)ix[a] * nin + k]) ++b;
        int rc = forward_pass(p, k, orders + (size_t)ix[a] * nin, X, Y, weights, s, timer);
        if (!rc) rc = forward_tree(p, orders, ix, a, b, k + 1, Y, weights, evals, s, timer);
        if (rc) return rc;
        a = b;
    }
    return SG_OK;
}

extern "C" int sg_evaluate_multi(sg_grid_plan *p, int32_t n_orders, const int32_t *orders,
                                 const void *control_points, const void *weights,
                                 void *const *evals, sg_stream_t stream) {
    int64_t V = 0;
    int rc = forward_checks(p, control_points, weights, V);
    if (rc) return rc;
    const sg_grid_desc &d = p->desc;
    if (n_orders < 0 || (n_orders > 0 && (!orders || !evals)))
        return set_error(SG_ERR_INVALID_ARGUMENT, "sg_evaluate_multi: bad order list");
    for (int i = 0; i < n_orders; ++i) {
        rc = check_orders(d, orders + (size_t)i * d.nin);
        if (rc) return rc;
        if (V > 0 && !evals[i])
            return set_error(SG_ERR_INVALID_ARGUMENT, "sg_evaluate_multi: eval %d is NULL", i);
    }
    if (V == 0 || n_orders == 0) return SG_OK;
    cudaStream_t s = (cudaStream_t)stream;
    if (d.nin == 1 || d.nin > 3 || use_fused(p, p->f2_fwd_ok)) {
        // one pass per order (Nin = 1), more live intermediates than the plan holds, or
        // the fused Nin = 2 path (no intermediate to share: one launch per order)
        for (int i = 0; i < n_orders; ++i) {
            rc = sg_evaluate(p, orders + (size_t)i * d.nin, control_points, weights, evals[i],
                             stream);
            if (rc) return rc;
        }
        return SG_OK;
    }
    std::vector<int> ix(n_orders);
    std::iota(ix.begin(), ix.end(), 0);
    const int nin = d.nin;
    std::stable_sort(ix.begin(), ix.end(), [&](int a, int b) {
        return std::lexicographical_compare(orders + (size_t)a * nin, orders + (size_t)a * nin + nin,
                                            orders + (size_t)b * nin, orders + (size_t)b * nin + nin);
    });
    PassTimer timer(p, s);
    return forward_tree(p, orders, ix.data(), 0, n_orders, 0, control_points, weights, evals, s,
                        timer);
}

extern "C" int sg_evaluate_adjoint(sg_grid_plan *p, const int32_t *derivative_order,
                                   const void *eval_bar, void *control_points_bar,
                                   sg_stream_t stream) {
    if (!p) return set_error(SG_ERR_INVALID_ARGUMENT, "plan is NULL");
    const sg_grid_desc &d = p->desc;
    if (d.has_weights)
        return set_error(SG_ERR_UNSUPPORTED, "Adjoint evaluation not supported for NURBS.");
    int rc = check_orders(d, derivative_order);
    if (rc) return rc;
    if (!control_points_bar)
        return set_error(SG_ERR_INVALID_ARGUMENT, "control_points_bar is NULL");
    cudaStream_t s = (cudaStream_t)stream;
    // SG_BF16_F32 grids take a Float32 cotangent and return a Float32 gradient.
    const bool f64 = d.dtype == SG_F64;
    int64_t V = 1, NCP = 1;
    for (int k = 0; k < d.nin; ++k) {
        V *= d.n_samples[k];
        NCP *= d.n_basis[k];
    }
    if (V == 0)  // no samples: M' * eval_bar is zero (src/adjoint.jl:61)
        return cuda_check(cudaMemsetAsync(control_points_bar, 0,
                                          (size_t)(NCP * d.nout) * elem_size(d.dtype), s),
                          "adjoint: zero output");
    if (!eval_bar) return set_error(SG_ERR_INVALID_ARGUMENT, "eval_bar is NULL");

    PassTimer timer(p, s);
    if (use_fused(p, p->f2_adj_ok)) {  // Nin = 2: both axes in one launch
        timer.begin();
        rc = f2_launch_grid(d.dtype == SG_F64 ? SG_F64 : SG_F32,
                            f2_grid(p, derivative_order, eval_bar, control_points_bar), p->f2_adj, 1,
                            p->status, s);
        timer.end();
        return rc;
    }
    const void *X = eval_bar;
    int buf = 0;
    for (int k = d.nin - 1; k >= 0; --k) {
        AxisPass a = axis_pass(d, p, k, derivative_order);
        a.X = X;
        a.Y = (k == 0) ? control_points_bar : p->scratch[buf];
        buf ^= 1;
        int64_t M = 1, Q = d.nout;
        for (int i = 0; i < k; ++i) M *= d.n_samples[i];
        for (int i = k + 1; i < d.nin; ++i) Q *= d.n_basis[i];
        a.M = M;
        a.Q = Q;
        timer.begin();
        if (k > 0) rc = f64 ? adj_axis_f64(a, s) : adj_axis_f32(a, s);
        else rc = f64 ? adj_axis0_f64(a, s) : adj_axis0_f32(a, s);
        timer.end();
        if (rc) return rc;
        X = a.Y;
    }
    return SG_OK;
}

// Measured choice of the adjoint stream's chunk size per axis k >= 1: each candidate
// runs the pass three times on the caller's arrays (events on `stream`), the fastest
// median wins.  The results do not depend on the chunk size (every control point sums
// its samples in the same order), only the time does.
// Fused path: the adjoint tile size (which sets the axis-1 block) is timed over the
// wave model's tiling and fixed sizes; the fastest tiling is kept.
static int tune_fused_adjoint(sg_grid_plan *p, const int32_t *ord, const void *eval_bar,
                              void *control_points_bar, cudaStream_t s, cudaEvent_t e0,
                              cudaEvent_t e1, int32_t *chosen) {
    const sg_grid_desc &d = p->desc;
    const int dt = d.dtype == SG_F64 ? SG_F64 : SG_F32;
    const int np = (int)f2_pairs_per_tile(dt);
    const F2Grid g = f2_grid(p, ord, eval_bar, control_points_bar);
    // 0: the wave model's tiling; otherwise cotangent values per tile
    static const int64_t kTargets[] = {0, 1 << 15, 1 << 16, 1 << 17, 1 << 18, 1 << 19, 1 << 20};
    float best = 3.4e38f;
    int64_t best_target = -1;
    F2Tiling best_t = p->f2_adj;
    int rc = SG_OK;
    for (int64_t target : kTargets) {
        F2Tiling t;
        if (!f2_adjoint_tiling(p->lb0_host.data(), d.n_basis[0], d.degree[0], d.n_samples[0], d.n_basis[1],
                               d.degree[1], d.n_samples[1], d.nout, np, f2_align_elems(dt), target,
                               target > 0 ? 0 : f2_slots(dt, 1), t))
            continue;
        float ms[3];
        for (int r = 0; r < 3 && !rc; ++r) {
            rc = cuda_check(cudaEventRecord(e0, s), "tune: record");
            if (!rc) rc = f2_launch_grid(dt, g, t, 1, p->status, s);
            if (!rc) rc = cuda_check(cudaEventRecord(e1, s), "tune: record");
            if (!rc) rc = cuda_check(cudaEventSynchronize(e1), "tune: sync");
            if (!rc) rc = cuda_check(cudaEventElapsedTime(&ms[r], e0, e1), "tune: time");
        }
        if (rc) return rc;
        std::sort(ms, ms + 3);
        if (ms[1] < best) {
            best = ms[1];
            best_target = target;
            best_t = t;
        }
    }
    if (best_target >= 0) {
        p->f2_adj_target = best_target;
        p->f2_adj = best_t;
    }
    if (chosen) {
        for (int k = 0; k < SG_MAX_NIN; ++k) chosen[k] = 0;
        chosen[1] = p->f2_adj.kb;  // axis-1 control points per tile
    }
    return cuda_check(cudaStreamSynchronize(s), "tune: sync");
}

extern "C" int sg_grid_plan_tune(sg_grid_plan *p, const int32_t *derivative_order,
                                 const void *eval_bar, void *control_points_bar,
                                 sg_stream_t stream, int32_t *chosen) {
    if (!p) return set_error(SG_ERR_INVALID_ARGUMENT, "plan is NULL");
    const sg_grid_desc &d = p->desc;
    if (d.has_weights) return set_error(SG_ERR_UNSUPPORTED, "Adjoint evaluation not supported for NURBS.");
    int rc = check_orders(d, derivative_order);
    if (rc) return rc;
    if (!eval_bar || !control_points_bar)
        return set_error(SG_ERR_INVALID_ARGUMENT, "sg_grid_plan_tune: NULL array");
    cudaStream_t s = (cudaStream_t)stream;
    const bool f64 = d.dtype == SG_F64;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    rc = cuda_check(cudaEventCreate(&e0), "tune: event");
    if (!rc) rc = cuda_check(cudaEventCreate(&e1), "tune: event");
    if (!rc && use_fused(p, p->f2_adj_ok)) {
        rc = tune_fused_adjoint(p, derivative_order, eval_bar, control_points_bar, s, e0, e1, chosen);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        return rc;
    }
    const void *X = eval_bar;
    int buf = 0;
    static const int kCand[] = {8, 12, 16, 24, 32, 48, 64};
    for (int k = d.nin - 1; k >= 0 && !rc; --k) {
        AxisPass a = axis_pass(d, p, k, derivative_order);
        a.X = X;
        a.Y = (k == 0) ? control_points_bar : p->scratch[buf];
        buf ^= 1;
        int64_t M = 1, Q = d.nout;
        for (int i = 0; i < k; ++i) M *= d.n_samples[i];
        for (int i = k + 1; i < d.nin; ++i) Q *= d.n_basis[i];
        a.M = M;
        a.Q = Q;
        if (k > 0 && a.n >= 8) {
            float best = 3.4e38f;
            int best_cc = 0;
            for (int c = 0; c < (int)(sizeof(kCand) / sizeof(kCand[0])) && !rc; ++c) {
                if (kCand[c] > a.n && c > 0) break;
                a.cc = kCand[c];
                float ms[3];
                for (int r = 0; r < 3 && !rc; ++r) {
                    rc = cuda_check(cudaEventRecord(e0, s), "tune: record");
                    if (!rc) rc = f64 ? adj_axis_f64(a, s) : adj_axis_f32(a, s);
                    if (!rc) rc = cuda_check(cudaEventRecord(e1, s), "tune: record");
                    if (!rc) rc = cuda_check(cudaEventSynchronize(e1), "tune: sync");
                    if (!rc) rc = cuda_check(cudaEventElapsedTime(&ms[r], e0, e1), "tune: time");
                }
                if (rc) break;
                std::sort(ms, ms + 3);
                if (ms[1] < best) {
                    best = ms[1];
                    best_cc = kCand[c];
                }
            }
            p->tuned_cc[k] = best_cc;
            a.cc = best_cc;
        }
        if (chosen) chosen[k] = p->tuned_cc[k];
        // leave this pass's output in place for the next axis
        if (!rc) rc = f64 ? (k > 0 ? adj_axis_f64(a, s) : adj_axis0_f64(a, s))
                          : (k > 0 ? adj_axis_f32(a, s) : adj_axis0_f32(a, s));
        X = a.Y;
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (!rc) rc = cuda_check(cudaStreamSynchronize(s), "tune: sync");
    return rc;
}

extern "C" int sg_grid_plan_untune(sg_grid_plan *p) {
    if (!p) return set_error(SG_ERR_INVALID_ARGUMENT, "plan is NULL");
    for (int k = 0; k < SG_MAX_NIN; ++k) p->tuned_cc[k] = 0;
    p->f2_adj_target = 0;
    plan_fused_tilings(p);
    return SG_OK;
}

extern "C" int sg_grid_plan_set_strategy(sg_grid_plan *p, int32_t strategy) {
    if (!p) return set_error(SG_ERR_INVALID_ARGUMENT, "plan is NULL");
    if (strategy != SG_STRATEGY_AUTO && strategy != SG_STRATEGY_SEPARABLE && strategy != SG_STRATEGY_FUSED)
        return set_error(SG_ERR_INVALID_ARGUMENT, "unknown strategy %d", strategy);
    if (strategy == SG_STRATEGY_FUSED && !p->f2_fwd_ok)
        return set_error(SG_ERR_UNSUPPORTED,
                         "the fused path takes non-NURBS grids with Nin = 2, degrees <= 3 and fewer "
                         "than 2^31 values");
    p->strategy = strategy;
    return SG_OK;
}

extern "C" int sg_grid_plan_paths(const sg_grid_plan *p, int32_t *forward, int32_t *adjoint) {
    if (!p) return set_error(SG_ERR_INVALID_ARGUMENT, "plan is NULL");
    if (forward) *forward = use_fused(p, p->f2_fwd_ok) ? SG_STRATEGY_FUSED : SG_STRATEGY_SEPARABLE;
    if (adjoint) *adjoint = use_fused(p, p->f2_adj_ok) ? SG_STRATEGY_FUSED : SG_STRATEGY_SEPARABLE;
    return SG_OK;
}
