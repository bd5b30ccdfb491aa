// sg_fit.cu -- the loss and update stages of a gradient-descent fit of spline grids.
//
// The reference's optimisation examples drive the hot path from a user loop
// (docs/src/examples_optics.md:184-191 and the Optimization.jl calls after it): evaluate!
// of the orders (0,0), (1,0), (0,1), a loss on the eval arrays, its gradient with respect
// to the control points through Enzyme (which runs evaluate_adjoint!,
// ext/SplineGridsEnzymeExt.jl), and an optimiser update.  The stages between the
// library's forward and adjoint are the ones here, as two device kernels over a fixed
// list of arrays so that the whole step can be captured into one CUDA graph:
//
//   loss:   for every term t (an eval array against a target of the same size, weight w_t)
//             cotangent_t = w_t (eval_t - target_t)
//             loss = sum_t w_t / 2 * sum_i (eval_t[i] - target_t[i])^2
//   update: for every parameter array u (control points) with gradient arrays g_u1..g_uk
//             u -= step * (g_u1 + ... + g_uk)
//
// The loss is a fixed-order two-level sum (per-block partials in FP64, then one block in
// index order), so a step is bitwise reproducible and a graph replay gives the bits of
// the eager step.  Each loss value is also appended to a device ring, so a replayed loop
// keeps its loss history without a host round trip.
#include "sg_common.cuh"

#include <algorithm>
#include <vector>

namespace sg {
namespace {

constexpr int kFitThreads = 256;
constexpr int kFitMaxGrads = 8;
constexpr int kFitRing = 1024;

template <class T>
struct FitTerm {
    const T *eval;
    const T *target;
    T *cot;
    int64_t n;
    T w;       // weight in the value type (the cotangent's scale)
    double hw; // w / 2 in FP64 (the loss's scale)
    int vec;   // all three arrays 16-byte aligned: 16-byte accesses
};

template <class T>
struct FitParam {
    T *p;
    int64_t n;
    const T *g[kFitMaxGrads];
    int ng;
    int vec;
};

struct FitState {
    double loss;
    unsigned long long count;       // loss values recorded so far
    double ring[kFitRing];          // loss of record k at ring[k % kFitRing]
};

// Sum of the block's values in a fixed order: lanes by butterfly, then warps by thread 0.
__device__ double block_sum(double v, double *sh) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) sh[w] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += sh[i];
    return s;
}

template <class T>
__device__ __forceinline__ double residual(const T e, const T t, const T w, T *c) {
    const T r = e - t;
    *c = w * r;
    return (double)r * (double)r;
}

// Blocks are dealt to the arrays in proportion to their sizes: array u owns blocks
// [first[u], first[u+1]) (first: n + 1 prefix values).  The array of block b.
__device__ __forceinline__ int owner(const int32_t *first, int n, int b) {
    int lo = 0, hi = n - 1;  // last u with first[u] <= b
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (first[mid] <= b) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// Block x of term t (its x-th of gx blocks) takes the values x*256 + i + k*gx*256.
template <class T>
__global__ void __launch_bounds__(kFitThreads)
k_fit_loss(const FitTerm<T> *terms, const int32_t *first, int n_terms, double *partial) {
    __shared__ double sh[kFitThreads / 32];
    const int u = owner(first, n_terms, (int)blockIdx.x);
    const FitTerm<T> t = terms[u];
    const int x = (int)blockIdx.x - first[u], gx = first[u + 1] - first[u];
    double acc = 0.0;
    const int64_t stride = (int64_t)gx * kFitThreads;
    constexpr int V = 16 / sizeof(T);
    if (t.vec) {
        const int64_t nv = t.n / V;
        for (int64_t i = (int64_t)x * kFitThreads + threadIdx.x; i < nv; i += stride) {
            Pack<T, V> e = ldp<T, V>(t.eval + i * V), g = ldp<T, V>(t.target + i * V), c;
#pragma unroll
            for (int j = 0; j < V; ++j) acc += residual(e.v[j], g.v[j], t.w, &c.v[j]);
            stp<T, V>(t.cot + i * V, c);
        }
        for (int64_t i = nv * V + (int64_t)x * kFitThreads + threadIdx.x; i < t.n; i += stride)
            acc += residual(t.eval[i], t.target[i], t.w, &t.cot[i]);
    } else {
        for (int64_t i = (int64_t)x * kFitThreads + threadIdx.x; i < t.n; i += stride)
            acc += residual(t.eval[i], t.target[i], t.w, &t.cot[i]);
    }
    const double s = block_sum(acc, sh);
    if (threadIdx.x == 0) partial[blockIdx.x] = t.hw * s;
}

// One block: the partials in index order (thread j takes j, j + 256, ...; then the
// fixed-order block sum), recorded as the loss and appended to the ring.
__global__ void __launch_bounds__(kFitThreads) k_fit_finish(const double *partial, int64_t n, FitState *st) {
    __shared__ double sh[kFitThreads / 32];
    double acc = 0.0;
    for (int64_t i = threadIdx.x; i < n; i += kFitThreads) acc += partial[i];
    const double s = block_sum(acc, sh);
    if (threadIdx.x == 0) {
        st->loss = s;
        st->ring[st->count % kFitRing] = s;
        st->count += 1;
    }
}

template <class T>
__device__ __forceinline__ T grad_sum(const FitParam<T> &q, int64_t i) {
    T s = q.g[0][i];
    for (int k = 1; k < q.ng; ++k) s += q.g[k][i];
    return s;
}

template <class T>
__global__ void __launch_bounds__(kFitThreads)
k_fit_update(const FitParam<T> *params, const int32_t *first, int n_params, T step) {
    const int u = owner(first, n_params, (int)blockIdx.x);
    const FitParam<T> q = params[u];
    const int x = (int)blockIdx.x - first[u], gx = first[u + 1] - first[u];
    const int64_t stride = (int64_t)gx * kFitThreads;
    constexpr int V = 16 / sizeof(T);
    int64_t head = 0;
    if (q.vec) {
        const int64_t nv = q.n / V;
        for (int64_t i = (int64_t)x * kFitThreads + threadIdx.x; i < nv; i += stride) {
            Pack<T, V> p = ldp<T, V>(q.p + i * V), s = ldp<T, V>(q.g[0] + i * V);
            for (int k = 1; k < q.ng; ++k) {
                const Pack<T, V> g = ldp<T, V>(q.g[k] + i * V);
#pragma unroll
                for (int j = 0; j < V; ++j) s.v[j] += g.v[j];
            }
#pragma unroll
            for (int j = 0; j < V; ++j) p.v[j] = p.v[j] - step * s.v[j];
            stp<T, V>(q.p + i * V, p);
        }
        head = nv * V;
    }
    for (int64_t i = head + (int64_t)x * kFitThreads + threadIdx.x; i < q.n; i += stride)
        q.p[i] = q.p[i] - step * grad_sum(q, i);
}

bool aligned16(const void *p) { return ((uintptr_t)p & 15) == 0; }

// Blocks of each array, in proportion to its size: about `total` blocks together (a few
// waves of resident blocks), at least one per array, none with less than one vector per
// thread; returned as the prefix `first` (n + 1 values).
std::vector<int32_t> deal_blocks(const std::vector<int64_t> &sizes, int64_t total) {
    int64_t all = 0;
    for (int64_t n : sizes) all += n;
    std::vector<int32_t> first(sizes.size() + 1, 0);
    for (size_t u = 0; u < sizes.size(); ++u) {
        const int64_t cap = std::max<int64_t>(1, (sizes[u] + kFitThreads * 4 - 1) / (kFitThreads * 4));
        const int64_t share = all > 0 ? (int64_t)((double)total * (double)sizes[u] / (double)all + 0.5) : 1;
        first[u + 1] = first[u] + (int32_t)std::max<int64_t>(1, std::min<int64_t>(cap, share));
    }
    return first;
}

// blocks of a launch: 8 resident blocks of 256 threads on every SM, four waves
int64_t launch_blocks() {
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return (int64_t)sms * 8 * 4;
}

}  // namespace
}  // namespace sg

using namespace sg;

struct sg_fit_plan {
    int32_t dtype = SG_F32;
    int32_t n_terms = 0, n_params = 0;
    int32_t blocks_loss = 0, blocks_update = 0;
    void *terms = nullptr;   // device FitTerm<T>[n_terms]
    void *params = nullptr;  // device FitParam<T>[n_params]
    int32_t *first = nullptr;  // device: the loss's block prefix [n_terms + 1], then the update's [n_params + 1]
    double *partial = nullptr; // one per loss block
    FitState *state = nullptr;
};

template <class T>
static int fit_upload(sg_fit_plan *p, int32_t n_terms, void *const *evals, const void *const *targets,
                      void *const *cotangents, const int64_t *n_values, const double *weights,
                      int32_t n_params, void *const *params, const int64_t *param_sizes,
                      const int32_t *grad_counts, void *const *grads) {
    std::vector<FitTerm<T>> ht(n_terms);
    std::vector<int64_t> tsz(n_terms), psz(n_params);
    for (int32_t t = 0; t < n_terms; ++t) {
        if (n_values[t] < 0) return set_error(SG_ERR_INVALID_ARGUMENT, "fit: term %d has a negative size", t);
        if (n_values[t] > 0 && (!evals[t] || !targets[t] || !cotangents[t]))
            return set_error(SG_ERR_INVALID_ARGUMENT, "fit: term %d has a NULL array", t);
        const double w = weights ? weights[t] : 1.0;
        ht[t] = FitTerm<T>{(const T *)evals[t], (const T *)targets[t], (T *)cotangents[t],
                           n_values[t], (T)w, 0.5 * w,
                           aligned16(evals[t]) && aligned16(targets[t]) && aligned16(cotangents[t])};
        tsz[t] = n_values[t];
    }
    std::vector<FitParam<T>> hp(n_params);
    int64_t gi = 0;
    for (int32_t u = 0; u < n_params; ++u) {
        const int ng = grad_counts[u];
        if (ng < 1 || ng > kFitMaxGrads)
            return set_error(SG_ERR_INVALID_ARGUMENT, "fit: parameter %d has %d gradients (1..%d)", u,
                             ng, kFitMaxGrads);
        if (param_sizes[u] < 0) return set_error(SG_ERR_INVALID_ARGUMENT, "fit: parameter %d has a negative size", u);
        FitParam<T> q{};
        q.p = (T *)params[u];
        q.n = param_sizes[u];
        q.ng = ng;
        bool vec = aligned16(q.p);
        for (int k = 0; k < ng; ++k) {
            q.g[k] = (const T *)grads[gi + k];
            vec = vec && aligned16(q.g[k]);
            if (q.n > 0 && !q.g[k]) return set_error(SG_ERR_INVALID_ARGUMENT, "fit: parameter %d has a NULL gradient", u);
        }
        if (q.n > 0 && !q.p) return set_error(SG_ERR_INVALID_ARGUMENT, "fit: parameter %d is NULL", u);
        q.vec = vec;
        gi += ng;
        hp[u] = q;
        psz[u] = q.n;
    }
    const int64_t nb = launch_blocks();
    std::vector<int32_t> first = deal_blocks(tsz, nb);
    const std::vector<int32_t> fu = deal_blocks(psz, nb);
    p->blocks_loss = first.back();
    p->blocks_update = fu.back();
    first.insert(first.end(), fu.begin(), fu.end());
    int rc = dev_alloc(&p->terms, sizeof(FitTerm<T>) * std::max(1, n_terms), "fit: terms");
    if (!rc) rc = dev_alloc(&p->params, sizeof(FitParam<T>) * std::max(1, n_params), "fit: parameters");
    if (!rc) rc = dev_alloc((void **)&p->first, sizeof(int32_t) * first.size(), "fit: block tables");
    if (!rc)
        rc = dev_alloc((void **)&p->partial, sizeof(double) * (size_t)std::max(1, p->blocks_loss),
                       "fit: partial sums");
    if (!rc) rc = dev_alloc((void **)&p->state, sizeof(FitState), "fit: state");
    if (!rc && n_terms)
        rc = cuda_check(cudaMemcpy(p->terms, ht.data(), sizeof(FitTerm<T>) * n_terms, cudaMemcpyHostToDevice),
                        "fit: upload terms");
    if (!rc && n_params)
        rc = cuda_check(cudaMemcpy(p->params, hp.data(), sizeof(FitParam<T>) * n_params, cudaMemcpyHostToDevice),
                        "fit: upload parameters");
    if (!rc)
        rc = cuda_check(cudaMemcpy(p->first, first.data(), sizeof(int32_t) * first.size(), cudaMemcpyHostToDevice),
                        "fit: upload block tables");
    if (!rc) rc = cuda_check(cudaMemset(p->state, 0, sizeof(FitState)), "fit: clear state");
    return rc;
}

extern "C" int sg_fit_plan_destroy(sg_fit_plan *p) {
    if (!p) return SG_OK;
    dev_free(p->terms);
    dev_free(p->params);
    dev_free(p->first);
    dev_free(p->partial);
    dev_free(p->state);
    delete p;
    return SG_OK;
}

extern "C" int sg_fit_plan_create(int32_t dtype, int32_t n_terms, void *const *evals,
                                  const void *const *targets, void *const *cotangents,
                                  const int64_t *n_values, const double *weights, int32_t n_params,
                                  void *const *params, const int64_t *param_sizes,
                                  const int32_t *grad_counts, void *const *grads, sg_fit_plan **out) {
    if (!out) return set_error(SG_ERR_INVALID_ARGUMENT, "fit: output pointer is NULL");
    *out = nullptr;
    if (dtype != SG_F32 && dtype != SG_F64)
        return set_error(SG_ERR_INVALID_ARGUMENT, "fit: dtype must be SG_F32 or SG_F64");
    if (n_terms < 0 || n_params < 0 || (n_terms > 0 && (!evals || !targets || !cotangents || !n_values)) ||
        (n_params > 0 && (!params || !param_sizes || !grad_counts || !grads)))
        return set_error(SG_ERR_INVALID_ARGUMENT, "fit: bad term or parameter lists");
    if (n_terms > 65535 || n_params > 65535)
        return set_error(SG_ERR_UNSUPPORTED, "fit: more than 65535 terms or parameters");
    sg_fit_plan *p = new sg_fit_plan;
    p->dtype = dtype;
    p->n_terms = n_terms;
    p->n_params = n_params;
    const int rc = dtype == SG_F64
        ? fit_upload<double>(p, n_terms, evals, targets, cotangents, n_values, weights, n_params, params,
                             param_sizes, grad_counts, grads)
        : fit_upload<float>(p, n_terms, evals, targets, cotangents, n_values, weights, n_params, params,
                            param_sizes, grad_counts, grads);
    if (rc) {
        sg_fit_plan_destroy(p);
        return rc;
    }
    *out = p;
    return SG_OK;
}

extern "C" int sg_fit_loss(sg_fit_plan *p, sg_stream_t stream) {
    if (!p) return set_error(SG_ERR_INVALID_ARGUMENT, "fit: plan is NULL");
    cudaStream_t s = (cudaStream_t)stream;
    const int64_t np = p->n_terms ? p->blocks_loss : 0;
    if (p->n_terms) {
        if (p->dtype == SG_F64)
            k_fit_loss<double><<<p->blocks_loss, kFitThreads, 0, s>>>((const FitTerm<double> *)p->terms, p->first,
                                                                      p->n_terms, p->partial);
        else
            k_fit_loss<float><<<p->blocks_loss, kFitThreads, 0, s>>>((const FitTerm<float> *)p->terms, p->first,
                                                                     p->n_terms, p->partial);
    }
    k_fit_finish<<<1, kFitThreads, 0, s>>>(p->partial, np, p->state);
    return cuda_check(cudaGetLastError(), "fit: loss launch");
}

extern "C" int sg_fit_update(sg_fit_plan *p, double step, sg_stream_t stream) {
    if (!p) return set_error(SG_ERR_INVALID_ARGUMENT, "fit: plan is NULL");
    if (!p->n_params) return SG_OK;
    cudaStream_t s = (cudaStream_t)stream;
    const int32_t *fu = p->first + p->n_terms + 1;
    if (p->dtype == SG_F64)
        k_fit_update<double><<<p->blocks_update, kFitThreads, 0, s>>>((const FitParam<double> *)p->params, fu,
                                                                     p->n_params, step);
    else
        k_fit_update<float><<<p->blocks_update, kFitThreads, 0, s>>>((const FitParam<float> *)p->params, fu,
                                                                    p->n_params, (float)step);
    return cuda_check(cudaGetLastError(), "fit: update launch");
}

extern "C" int sg_fit_losses(sg_fit_plan *p, sg_stream_t stream, double *latest, int64_t *count,
                             double *history, int64_t capacity) {
    if (!p) return set_error(SG_ERR_INVALID_ARGUMENT, "fit: plan is NULL");
    cudaStream_t s = (cudaStream_t)stream;
    FitState h;
    int rc = cuda_check(cudaMemcpyAsync(&h, p->state, sizeof(FitState), cudaMemcpyDeviceToHost, s),
                        "fit: read losses");
    if (!rc) rc = cuda_check(cudaStreamSynchronize(s), "fit: sync");
    if (rc) return rc;
    if (latest) *latest = h.loss;
    if (count) *count = (int64_t)h.count;
    if (history && capacity > 0) {
        // the most recent min(count, ring, capacity) values, oldest first
        const int64_t n = std::min(std::min((int64_t)h.count, (int64_t)kFitRing), capacity);
        for (int64_t k = 0; k < n; ++k) {
            const int64_t rec = (int64_t)h.count - n + k;
            history[k] = h.ring[rec % kFitRing];
        }
    }
    return SG_OK;
}
