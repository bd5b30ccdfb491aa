// sg_lsqr.cu -- matrix-free LSQR on the device, for least-squares fits of spline grids.
//
// The reference fits control points by handing `LinearMap(spline_grid)`
// (ext/SplineGridsLinearMapsExt.jl:5-52: forward = evaluate!(control_points) then
// evaluate!(grid), adjoint = evaluate_adjoint!(grid) then evaluate_adjoint!(control_points))
// to IterativeSolvers.jl's `lsqr` (Project.toml compat 0.9; test/test_LinearMapsExt.jl).
// IterativeSolvers is not part of the reference tree; its `lsqr` is the published LSQR
// of Paige & Saunders (ACM TOMS 8(1):43-71, 1982, "LSQR: An algorithm for sparse linear
// equations and sparse least squares"), restated here from that paper: Golub-Kahan
// bidiagonalisation, a Givens QR update of the bidiagonal system, and the paper's stopping
// rules 1-3 with the estimates of ||A||, cond(A), ||r||, ||A'r|| and ||x||.
//
// Layout of one iteration on the device (vectors stay in HBM, scalars in a device struct):
//   F = A V                      (caller: the grid's forward evaluation)
//   U = F/alpha - (alpha/beta) U ; partial sums of U^2       k_lsqr_axpby
//   beta = ||U||, ||A|| estimate                              k_lsqr_scalar (phase U)
//   G = A' U                     (caller: the grid's adjoint)
//   V = G/beta - (beta/alpha) V ; partial sums of V^2, W^2    k_lsqr_axpby
//   alpha = ||V||, Givens rotation, estimates, stopping rules k_lsqr_scalar (phase V)
//   X += t1 W ; W = V/alpha + t2 W                            k_lsqr_xw
// U and V are kept unnormalised (u = U/beta, v = V/alpha), so no pass over a vector only
// rescales it: the scale is folded into the next pass that reads it.  Every reduction is a
// fixed-order two-level sum (per-block partials, then one block), so a solve is bitwise
// reproducible.  The iteration can be captured once into a CUDA graph whose body runs in a
// device-side `while` conditional node: the scalar kernel sets the loop condition after
// every step (open while no stopping rule holds, closed when one does, and maxiter is one
// of the rules), so a whole solve is one graph launch with no host round trip.
#include <math.h>

#include "sg_common.cuh"

namespace sg {
namespace {

constexpr int kLsqrThreads = 256;
constexpr int kLsqrMaxBlocks = 8 * 152;  // grid of the vector passes: at most 8 blocks per SM

struct LsqrState {
    // Golub-Kahan scalars of the current iteration
    double alpha, beta;
    // QR recurrence (paper section 4.1) and the norm / condition estimates (section 5)
    double rhobar, phibar, anorm, acond, ddnorm, res2, xnorm, xxnorm, z, cs2, sn2;
    double bnorm, rnorm, arnorm;
    // coefficients of the vector passes, written by the scalar kernel
    double cu_a, cu_b, cv_a, cv_b, t1, t2, inv_alpha;
    // parameters
    double damp, atol, btol, ctol, eps;
    long long itn, maxiter;
    int istop, done;
};

int n_blocks(int64_t n) {
    int64_t b = (n + (int64_t)kLsqrThreads * 4 - 1) / ((int64_t)kLsqrThreads * 4);
    return (int)(b < 1 ? 1 : (b > kLsqrMaxBlocks ? kLsqrMaxBlocks : b));
}

// Block-wide sum of one double, fixed order (warp shuffles, then warp 0 over the warps).
__device__ __forceinline__ double block_sum(double v, double *sh) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) sh[w] = v;
    __syncthreads();
    double r = 0.0;
    if (w == 0) {
        r = l < (int)(blockDim.x >> 5) ? sh[l] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
    }
    return r;  // valid in thread 0
}

// U = b, and (n-space) X = 0, W = 0; partial sums of b^2.
template <typename T>
__global__ void __launch_bounds__(kLsqrThreads) k_lsqr_start(const T *__restrict__ b, T *__restrict__ U, int64_t m,
                                                T *__restrict__ X, T *__restrict__ W, int64_t n,
                                                double *__restrict__ part) {
    __shared__ double sh[kLsqrThreads / 32];
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    double s = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += stride) {
        const T v = b[i];
        U[i] = v;
        s += (double)v * (double)v;
    }
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        X[i] = T(0);
        W[i] = T(0);
    }
    s = block_sum(s, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// Y = a * Xin + b * Y with (a, b) = coef[0..1] read from the state; partial sums of the new
// Y^2 into part[block], and (when W is given) of W^2 into part2[block].
template <typename T>
__global__ void __launch_bounds__(kLsqrThreads) k_lsqr_axpby(const T *__restrict__ Xin, T *__restrict__ Y, int64_t n,
                                                const double *__restrict__ coef,
                                                const int *__restrict__ done,
                                                double *__restrict__ part,
                                                const T *__restrict__ W, double *__restrict__ part2) {
    __shared__ double sh[kLsqrThreads / 32];
    if (*done) return;  // the solve has stopped: leave every vector as it is
    const T a = (T)coef[0], bb = (T)coef[1];
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t i0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    double s = 0.0, s2 = 0.0;
    int64_t i = i0;
    // four independent elements in flight per thread
    for (; i + 3 * stride < n; i += 4 * stride) {
        T x[4], y[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) { x[k] = Xin[i + k * stride]; y[k] = Y[i + k * stride]; }
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const T r = bb == T(0) ? a * x[k] : fma(a, x[k], bb * y[k]);
            Y[i + k * stride] = r;
            s += (double)r * (double)r;
        }
    }
    for (; i < n; i += stride) {
        const T r = bb == T(0) ? a * Xin[i] : fma(a, Xin[i], bb * Y[i]);
        Y[i] = r;
        s += (double)r * (double)r;
    }
    if (W) {
        for (int64_t j = i0; j < n; j += stride) {
            const double w = (double)W[j];
            s2 += w * w;
        }
    }
    s = block_sum(s, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
    if (W) {
        s2 = block_sum(s2, sh);
        if (threadIdx.x == 0) part2[blockIdx.x] = s2;
    }
}

// X += t1 W ; W = inv_alpha V + t2 W.
template <typename T>
__global__ void __launch_bounds__(kLsqrThreads) k_lsqr_xw(const T *__restrict__ V, T *__restrict__ W, T *__restrict__ X,
                                             int64_t n, const LsqrState *__restrict__ st,
                                             const int *__restrict__ skip) {
    if (*skip) return;
    const T t1 = (T)st->t1, t2 = (T)st->t2, ia = (T)st->inv_alpha;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const T w = W[i];
        X[i] = fma(t1, w, X[i]);
        W[i] = fma(ia, V[i], t2 * w);
    }
}

// Sum of part[0..nb) in a fixed order by one block.
__device__ double sum_partials(const double *part, int nb, double *sh) {
    double s = 0.0;
    for (int i = threadIdx.x; i < nb; i += blockDim.x) s += part[i];
    return block_sum(s, sh);
}

enum { kPhaseStart = 0, kPhaseU = 1, kPhaseV = 2 };

template <typename T>
__device__ bool one_plus_is_one(double t) {
    return (T)1 + (T)t <= (T)1;
}

// One block.  Phase start: beta = ||b||.  Phase U: beta = ||U||.  Phase V: alpha = ||V||,
// the QR step, estimates and stopping rules (first call: the initialisation).
template <typename T>
__global__ void __launch_bounds__(kLsqrThreads) k_lsqr_scalar(LsqrState *st, const double *__restrict__ part,
                                                 const double *__restrict__ part2, int nb,
                                                 int nb2, int phase, int *skip_xw,
                                                 cudaGraphConditionalHandle cond, int has_cond) {
    __shared__ double sh[kLsqrThreads / 32];
    if (phase != kPhaseStart && st->done) {
        if (threadIdx.x == 0) {
            *skip_xw = 1;
            if (has_cond) cudaGraphSetConditional(cond, 0);
        }
        return;
    }
    const double s = sum_partials(part, nb, sh);
    double s2 = 0.0;
    if (phase == kPhaseV) s2 = sum_partials(part2, nb2, sh);
    if (threadIdx.x != 0) return;
    LsqrState S = *st;
    *skip_xw = 1;
    if (phase == kPhaseStart) {
        // a new solve: the recurrence starts afresh, the parameters stay
        S.alpha = S.rhobar = S.phibar = S.anorm = S.acond = S.ddnorm = S.res2 = 0.0;
        S.xnorm = S.xxnorm = S.z = S.sn2 = S.rnorm = S.arnorm = 0.0;
        S.cs2 = -1.0;  // c_0 of the rotation behind the ||x|| estimate
        S.t1 = S.t2 = S.inv_alpha = S.cu_a = S.cu_b = 0.0;
        S.istop = 0;
        S.done = 0;
        S.beta = sqrt(s);
        S.bnorm = S.beta;
        S.cv_a = S.beta > 0.0 ? 1.0 / S.beta : 0.0;  // V = A'u = G / beta
        S.cv_b = 0.0;
        S.itn = 0;
    } else if (phase == kPhaseU) {
        const double beta = sqrt(s);
        // paper section 5.1: ||B_k||_F accumulates alpha_k^2 + beta_{k+1}^2 (+ damp^2)
        if (beta > 0.0) {
            S.anorm = sqrt(S.anorm * S.anorm + S.alpha * S.alpha + beta * beta + S.damp * S.damp);
            S.cv_a = 1.0 / beta;                                 // A'u = G / beta
            S.cv_b = S.alpha > 0.0 ? -beta / S.alpha : 0.0;      // - beta v = -(beta/alpha) V
        } else {
            S.cv_a = 0.0;  // u is zero: v keeps its value (the paper's "if beta > 0")
            S.cv_b = 1.0;
        }
        S.beta = beta;
    } else if (S.itn == 0) {
        // initialisation (paper section 4.1, step 1): alpha_1 v_1 = A' u_1, w_1 = v_1
        const double alpha = sqrt(s);
        S.alpha = alpha;
        S.rhobar = alpha;
        S.phibar = S.beta;
        S.rnorm = S.beta;
        S.arnorm = alpha * S.beta;
        S.inv_alpha = alpha > 0.0 ? 1.0 / alpha : 0.0;
        S.t1 = 0.0;
        S.t2 = 0.0;
        S.cu_a = S.inv_alpha;  // A v = F / alpha
        S.cu_b = S.beta > 0.0 ? -alpha / S.beta : 0.0;
        *skip_xw = 0;
        if (S.arnorm == 0.0) {  // x = 0 solves the problem exactly
            S.istop = 0;
            S.done = 1;
        }
        S.itn = 1;
    } else {
        // with beta == 0 the previous v was kept, so alpha is unchanged
        const double alpha = S.beta > 0.0 ? sqrt(s) : S.alpha;
        const double beta = S.beta;
        // the damped system's extra rotation (paper section 4.3)
        const double dampsq = S.damp * S.damp;
        const double rhobar1 = sqrt(S.rhobar * S.rhobar + dampsq);
        const double cs1 = S.rhobar / rhobar1, sn1 = S.damp / rhobar1;
        const double psi = sn1 * S.phibar;
        const double phibar0 = cs1 * S.phibar;
        // plane rotation eliminating beta (section 4.1, step 4)
        const double rho = sqrt(rhobar1 * rhobar1 + beta * beta);
        const double cs = rhobar1 / rho, sn = beta / rho;
        const double theta = sn * alpha;
        S.rhobar = -cs * alpha;
        const double phi = cs * phibar0;
        S.phibar = sn * phibar0;
        const double tau = sn * phi;
        // x and w update coefficients (step 5)
        S.t1 = phi / rho;
        S.t2 = -theta / rho;
        S.inv_alpha = alpha > 0.0 ? 1.0 / alpha : 0.0;
        // estimates (section 5): ||D_k||_F from ||w_k||^2 / rho_k^2, ||x|| via the
        // rotation of the lower bidiagonal factor
        S.ddnorm += s2 / (rho * rho);
        const double delta = S.sn2 * rho;
        const double gambar = -S.cs2 * rho;
        const double rhs = phi - delta * S.z;
        const double zbar = rhs / gambar;
        S.xnorm = sqrt(S.xxnorm + zbar * zbar);
        const double gamma = sqrt(gambar * gambar + theta * theta);
        S.cs2 = gambar / gamma;
        S.sn2 = theta / gamma;
        S.z = rhs / gamma;
        S.xxnorm += S.z * S.z;
        S.acond = S.anorm * sqrt(S.ddnorm);
        S.res2 += psi * psi;
        S.rnorm = sqrt(S.phibar * S.phibar + S.res2);
        S.arnorm = alpha * fabs(tau);
        S.alpha = alpha;
        S.cu_a = S.inv_alpha;
        S.cu_b = beta > 0.0 ? -alpha / beta : 0.0;
        *skip_xw = 0;
        // stopping rules (section 6); the later assignment wins, as in the paper's order
        const double test1 = S.rnorm / S.bnorm;
        const double test2 = S.arnorm / (S.anorm * S.rnorm + S.eps);
        const double test3 = 1.0 / (S.acond + S.eps);
        const double t1s = test1 / (1.0 + S.anorm * S.xnorm / S.bnorm);
        const double rtol = S.btol + S.atol * S.anorm * S.xnorm / S.bnorm;
        int istop = 0;
        if (S.itn >= S.maxiter) istop = 7;
        if (one_plus_is_one<T>(test3)) istop = 6;
        if (one_plus_is_one<T>(test2)) istop = 5;
        if (one_plus_is_one<T>(t1s)) istop = 4;
        if (test3 <= S.ctol) istop = 3;
        if (test2 <= S.atol) istop = 2;
        if (test1 <= rtol) istop = 1;
        if (!(isfinite(alpha) && isfinite(beta) && isfinite(S.rnorm))) istop = -1;
        S.istop = istop;
        if (istop != 0) S.done = 1;
        else S.itn += 1;
    }
    *st = S;
    // The loop handle starts each launch at 0 (no iteration): the initialisation opens
    // the loop, the step that meets a stopping rule closes it.  Only phase V sets it.
    if (has_cond && phase == kPhaseV) cudaGraphSetConditional(cond, S.done ? 0u : 1u);
}

}  // namespace
}  // namespace sg

using namespace sg;

struct sg_lsqr {
    int32_t dtype = SG_F32;
    int64_t m = 0, n = 0;
    void *U = nullptr, *V = nullptr, *W = nullptr, *X = nullptr, *F = nullptr, *G = nullptr;
    LsqrState *st = nullptr;  // device
    double *part = nullptr;   // 2 * kLsqrMaxBlocks partial sums
    int *skip = nullptr;      // device flag: skip the x/w pass of this iteration
    cudaGraphConditionalHandle cond = 0;
    int has_cond = 0;
    cudaStream_t body = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int capture = 0;  // 0 none, 1 prologue, 2 body
};

namespace {

int lsqr_launch_axpby(sg_lsqr *h, const void *Xin, void *Y, int64_t len, int which,
                      const void *Wn, cudaStream_t s) {
    const double *coef = which == 0 ? &h->st->cu_a : &h->st->cv_a;
    const int *done = &h->st->done;
    const int nb = n_blocks(len);
    if (h->dtype == SG_F64)
        k_lsqr_axpby<double><<<nb, kLsqrThreads, 0, s>>>(
            (const double *)Xin, (double *)Y, len, coef, done, h->part, (const double *)Wn,
            h->part + kLsqrMaxBlocks);
    else
        k_lsqr_axpby<float><<<nb, kLsqrThreads, 0, s>>>(
            (const float *)Xin, (float *)Y, len, coef, done, h->part, (const float *)Wn,
            h->part + kLsqrMaxBlocks);
    return cuda_check(cudaGetLastError(), "k_lsqr_axpby launch");
}

int lsqr_launch_scalar(sg_lsqr *h, int nb, int nb2, int phase, cudaStream_t s) {
    if (h->dtype == SG_F64)
        k_lsqr_scalar<double><<<1, kLsqrThreads, 0, s>>>(h->st, h->part, h->part + kLsqrMaxBlocks,
                                                        nb, nb2, phase, h->skip, h->cond,
                                                        h->has_cond);
    else
        k_lsqr_scalar<float><<<1, kLsqrThreads, 0, s>>>(h->st, h->part, h->part + kLsqrMaxBlocks,
                                                       nb, nb2, phase, h->skip, h->cond,
                                                       h->has_cond);
    return cuda_check(cudaGetLastError(), "k_lsqr_scalar launch");
}

bool vec_ok(const void *p) { return p && ((uintptr_t)p % 8) == 0; }

}  // namespace

extern "C" int sg_lsqr_create(int32_t dtype, int64_t m, int64_t n, void *U, void *V, void *W,
                              void *X, void *F, void *G, double damp, double atol, double btol,
                              double conlim, int64_t maxiter, sg_lsqr **out) {
    if (!out) return set_error(SG_ERR_INVALID_ARGUMENT, "sg_lsqr_create: NULL out");
    *out = nullptr;
    if (dtype != SG_F32 && dtype != SG_F64)
        return set_error(SG_ERR_INVALID_ARGUMENT, "sg_lsqr_create: dtype must be F32 or F64");
    if (m < 1 || n < 1 || maxiter < 1)
        return set_error(SG_ERR_INVALID_ARGUMENT, "sg_lsqr_create: sizes and maxiter must be >= 1");
    if (!vec_ok(U) || !vec_ok(V) || !vec_ok(W) || !vec_ok(X) || !vec_ok(F) || !vec_ok(G))
        return set_error(SG_ERR_INVALID_ARGUMENT, "sg_lsqr_create: NULL or misaligned vector");
    if (!(damp >= 0.0) || !(atol >= 0.0) || !(btol >= 0.0) || !(conlim >= 0.0))
        return set_error(SG_ERR_INVALID_ARGUMENT, "sg_lsqr_create: tolerances must be >= 0");
    sg_lsqr *h = new sg_lsqr;
    h->dtype = dtype;
    h->m = m;
    h->n = n;
    h->U = U; h->V = V; h->W = W; h->X = X; h->F = F; h->G = G;
    int rc = dev_alloc((void **)&h->st, sizeof(LsqrState), "lsqr: state");
    if (!rc) rc = dev_alloc((void **)&h->part, 2 * kLsqrMaxBlocks * sizeof(double), "lsqr: partials");
    if (!rc) rc = dev_alloc((void **)&h->skip, sizeof(int), "lsqr: flag");
    if (!rc) {
        LsqrState S = {};
        S.damp = damp;
        S.atol = atol;
        S.btol = btol;
        S.ctol = conlim > 0.0 ? 1.0 / conlim : 0.0;
        S.eps = dtype == SG_F64 ? 2.220446049250313e-16 : 1.1920928955078125e-07;
        S.maxiter = maxiter;
        S.done = 1;  // nothing to do before sg_lsqr_start
        rc = cuda_check(cudaMemcpy(h->st, &S, sizeof(S), cudaMemcpyHostToDevice), "lsqr: init");
    }
    if (rc) {
        sg_lsqr_destroy(h);
        return rc;
    }
    *out = h;
    return SG_OK;
}

extern "C" int sg_lsqr_destroy(sg_lsqr *h) {
    if (!h) return SG_OK;
    if (h->exec) cudaGraphExecDestroy(h->exec);
    if (h->graph) cudaGraphDestroy(h->graph);
    if (h->body) cudaStreamDestroy(h->body);
    dev_free(h->st);
    dev_free(h->part);
    dev_free(h->skip);
    delete h;
    return SG_OK;
}

extern "C" int sg_lsqr_start(sg_lsqr *h, const void *b, sg_stream_t stream) {
    if (!h || !vec_ok(b)) return set_error(SG_ERR_INVALID_ARGUMENT, "sg_lsqr_start: NULL argument");
    cudaStream_t s = (cudaStream_t)stream;
    const int nb = n_blocks(h->m > h->n ? h->m : h->n);
    if (h->dtype == SG_F64)
        k_lsqr_start<double><<<nb, kLsqrThreads, 0, s>>>((const double *)b, (double *)h->U, h->m,
                                                        (double *)h->X, (double *)h->W, h->n,
                                                        h->part);
    else
        k_lsqr_start<float><<<nb, kLsqrThreads, 0, s>>>((const float *)b, (float *)h->U, h->m,
                                                       (float *)h->X, (float *)h->W, h->n,
                                                       h->part);
    int rc = cuda_check(cudaGetLastError(), "k_lsqr_start launch");
    if (rc) return rc;
    return lsqr_launch_scalar(h, nb, 0, kPhaseStart, s);
}

extern "C" int sg_lsqr_after_forward(sg_lsqr *h, sg_stream_t stream) {
    if (!h) return set_error(SG_ERR_INVALID_ARGUMENT, "sg_lsqr_after_forward: NULL handle");
    cudaStream_t s = (cudaStream_t)stream;
    int rc = lsqr_launch_axpby(h, h->F, h->U, h->m, 0, nullptr, s);
    if (!rc) rc = lsqr_launch_scalar(h, n_blocks(h->m), 0, kPhaseU, s);
    return rc;
}

extern "C" int sg_lsqr_after_adjoint(sg_lsqr *h, sg_stream_t stream) {
    if (!h) return set_error(SG_ERR_INVALID_ARGUMENT, "sg_lsqr_after_adjoint: NULL handle");
    cudaStream_t s = (cudaStream_t)stream;
    int rc = lsqr_launch_axpby(h, h->G, h->V, h->n, 1, h->W, s);
    if (!rc) rc = lsqr_launch_scalar(h, n_blocks(h->n), n_blocks(h->n), kPhaseV, s);
    if (rc) return rc;
    const int nb = n_blocks(h->n);
    if (h->dtype == SG_F64)
        k_lsqr_xw<double><<<nb, kLsqrThreads, 0, s>>>((const double *)h->V, (double *)h->W,
                                                     (double *)h->X, h->n, h->st, h->skip);
    else
        k_lsqr_xw<float><<<nb, kLsqrThreads, 0, s>>>((const float *)h->V, (float *)h->W,
                                                    (float *)h->X, h->n, h->st, h->skip);
    return cuda_check(cudaGetLastError(), "k_lsqr_xw launch");
}

extern "C" int sg_lsqr_capture_begin(sg_lsqr *h, sg_stream_t stream) {
    if (!h) return set_error(SG_ERR_INVALID_ARGUMENT, "sg_lsqr_capture_begin: NULL handle");
    if (h->capture) return set_error(SG_ERR_INVALID_ARGUMENT, "sg_lsqr_capture_begin: already capturing");
    cudaStream_t s = (cudaStream_t)stream;
    int rc = SG_OK;
    if (!h->body)
        rc = cuda_check(cudaStreamCreateWithFlags(&h->body, cudaStreamNonBlocking), "lsqr: body stream");
    if (rc) return rc;
    if (h->exec) { cudaGraphExecDestroy(h->exec); h->exec = nullptr; }
    if (h->graph) { cudaGraphDestroy(h->graph); h->graph = nullptr; }
    rc = cuda_check(cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed), "lsqr: begin capture");
    if (rc) return rc;
    h->capture = 1;
    cudaStreamCaptureStatus cs;
    cudaGraph_t g = nullptr;
    rc = cuda_check(cudaStreamGetCaptureInfo(s, &cs, nullptr, &g, nullptr, nullptr, nullptr),
                    "lsqr: capture info");
    // the loop runs while the handle is non-zero; every launch of the graph starts it at 0
    // and the prologue's initialisation step opens it, so the loop never runs unless a
    // kernel of this solve set it
    if (!rc) rc = cuda_check(cudaGraphConditionalHandleCreate(&h->cond, g, 0, cudaGraphCondAssignDefault),
                             "lsqr: conditional handle");
    if (!rc) h->has_cond = 1;
    return rc;
}

extern "C" int sg_lsqr_capture_body(sg_lsqr *h, sg_stream_t stream, sg_stream_t *body) {
    if (!h || !body) return set_error(SG_ERR_INVALID_ARGUMENT, "sg_lsqr_capture_body: NULL argument");
    if (h->capture != 1) return set_error(SG_ERR_INVALID_ARGUMENT, "sg_lsqr_capture_body: not in the prologue");
    cudaStream_t s = (cudaStream_t)stream;
    cudaStreamCaptureStatus cs;
    cudaGraph_t g = nullptr;
    const cudaGraphNode_t *deps = nullptr;
    size_t ndeps = 0;
    int rc = cuda_check(cudaStreamGetCaptureInfo(s, &cs, nullptr, &g, &deps, nullptr, &ndeps),
                        "lsqr: capture info");
    if (rc) return rc;
    cudaGraphNodeParams p = {};
    p.type = cudaGraphNodeTypeConditional;
    p.conditional.handle = h->cond;
    p.conditional.type = cudaGraphCondTypeWhile;
    p.conditional.size = 1;
    cudaGraphNode_t node;
    rc = cuda_check(cudaGraphAddNode(&node, g, deps, nullptr, ndeps, &p), "lsqr: while node");
    if (!rc) rc = cuda_check(cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1,
                                                                 cudaStreamSetCaptureDependencies),
                             "lsqr: capture dependencies");
    if (!rc) rc = cuda_check(cudaStreamBeginCaptureToGraph(h->body, p.conditional.phGraph_out[0],
                                                           nullptr, nullptr, 0,
                                                           cudaStreamCaptureModeRelaxed),
                             "lsqr: begin body capture");
    if (rc) return rc;
    h->capture = 2;
    *body = (sg_stream_t)h->body;
    return SG_OK;
}

extern "C" int sg_lsqr_capture_end(sg_lsqr *h, sg_stream_t stream) {
    if (!h) return set_error(SG_ERR_INVALID_ARGUMENT, "sg_lsqr_capture_end: NULL handle");
    cudaStream_t s = (cudaStream_t)stream;
    int rc = SG_OK;
    if (h->capture == 2) {
        cudaGraph_t bg = nullptr;
        rc = cuda_check(cudaStreamEndCapture(h->body, &bg), "lsqr: end body capture");
    }
    cudaGraph_t g = nullptr;
    if (h->capture >= 1) {
        const int rc2 = cuda_check(cudaStreamEndCapture(s, &g), "lsqr: end capture");
        if (!rc) rc = rc2;
    }
    const int complete = h->capture == 2;
    h->capture = 0;
    h->has_cond = 0;
    if (!rc && !complete)
        rc = set_error(SG_ERR_INVALID_ARGUMENT, "sg_lsqr_capture_end: the loop body was not captured");
    if (!rc) rc = cuda_check(cudaGraphInstantiate(&h->exec, g, 0), "lsqr: instantiate");
    if (rc) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    h->graph = g;
    return SG_OK;
}

extern "C" int sg_lsqr_launch(sg_lsqr *h, sg_stream_t stream) {
    if (!h || !h->exec) return set_error(SG_ERR_INVALID_ARGUMENT, "sg_lsqr_launch: no captured solve");
    return cuda_check(cudaGraphLaunch(h->exec, (cudaStream_t)stream), "lsqr: graph launch");
}

extern "C" int sg_lsqr_info(sg_lsqr *h, sg_stream_t stream, int64_t *counts, double *norms) {
    if (!h || !counts || !norms) return set_error(SG_ERR_INVALID_ARGUMENT, "sg_lsqr_info: NULL argument");
    LsqrState S;
    cudaStream_t s = (cudaStream_t)stream;
    int rc = cuda_check(cudaMemcpyAsync(&S, h->st, sizeof(S), cudaMemcpyDeviceToHost, s), "lsqr: read state");
    if (!rc) rc = cuda_check(cudaStreamSynchronize(s), "lsqr: sync");
    if (rc) return rc;
    counts[0] = S.itn;
    counts[1] = S.istop;
    counts[2] = S.done;
    norms[0] = S.anorm;
    norms[1] = S.acond;
    norms[2] = S.rnorm;
    norms[3] = S.arnorm;
    norms[4] = S.xnorm;
    norms[5] = S.bnorm;
    return SG_OK;
}
