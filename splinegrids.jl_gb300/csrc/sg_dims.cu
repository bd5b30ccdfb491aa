// sg_dims.cu -- per-SplineDimension kernels: knot expansion, knot-span search and the
// Cox-de Boor basis tables (values and derivatives).
//
// Reference: src/knot_vector.jl:21-49, src/util_kernels.jl:1-67,
// src/spline_dimension.jl:160-272 (SouthEndMusic/SplineGrids.jl v0.1.1).
#include "sg_common.cuh"

namespace sg {

// expand_knot_vector_kernel (src/util_kernels.jl:1-20): one thread per knot value
// writes it `multiplicity` times after the running sum of the earlier multiplicities,
// as the reference does.  Writes are bounded by n_knots (the caller's allocation).
template <typename T>
__global__ void k_expand_knots(const T *__restrict__ vals, const int32_t *__restrict__ mult,
                               int64_t n_values, int64_t n_knots, T *__restrict__ knots_all) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n_values) return;
    int64_t s = 0;
    for (int64_t j = 0; j < i; ++j) s += mult[j];
    const T v = vals[i];
    for (int64_t k = s; k < s + mult[i] && k < n_knots; ++k)
        if (k >= 0) knots_all[k] = v;
}

// set_sample_indices_kernel (src/util_kernels.jl:22-49).  The reference counts, by a
// linear scan with early exit, the leading knots for which `!(t < knot)`.  Because
// knots_all is sorted, `t < knots_all[i]` is false..false,true..true in i (also for
// NaN t, where it is always false), so the count is the first i with t < knots[i]:
// a binary search on the same predicate gives the identical integer.
template <typename T>
__global__ void k_sample_indices(const T *__restrict__ samples, int64_t ns,
                                 const T *__restrict__ knots, int64_t n_knots, int degree,
                                 int32_t *__restrict__ out) {
    int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (l >= ns) return;
    const T t = samples[l];
    int64_t lo = 0, hi = n_knots;
    while (lo < hi) {
        int64_t mid = (lo + hi) >> 1;
        if (t < knots[mid]) hi = mid; else lo = mid + 1;
    }
    int64_t idx = clamp64(lo, degree + 1, n_knots - degree - 1);
    out[l] = (int32_t)idx;
}

// spline_dimension_kernel (src/spline_dimension.jl:160-215): Cox-de Boor values and
// derivatives, one thread per sample, computed in Float64 whatever the storage type
// and stored as T into the reference layout eval[l + ns*(j + (d+1)*m)].
//
// In the reference recursion the order-m values at degree k are made from the
// order-(m-1) values at degree k-1 (:200-205), and the order-0 values from the order-0
// values one degree lower (:190-198).  So the order-m table at the final degree d is
// the order-0 table at degree d-m followed by m derivative steps.  Computing each
// order that way performs exactly the reference's operations on each value, in the
// same order, while keeping only two columns of d+1 values live.
// D = d+1 for the unrolled instances; D = 0 runs any degree up to SG_MAX_DEGREE.
template <int D, typename T>
__global__ void k_basis(const T *__restrict__ knots, int64_t n_knots, const T *__restrict__ samples,
                        const int32_t *__restrict__ sidx, int64_t ns, int degree_rt, int maxd,
                        T *__restrict__ eval) {
    constexpr int DA = D > 0 ? D : kDMax;
    const int deg = D > 0 ? D - 1 : degree_rt;
    int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (l >= ns) return;
    const double t = (double)samples[l];
    // 1-based knot-span index; clamped so every knot read below stays in range
    const int64_t i = clamp64((int64_t)sidx[l], deg + 1, n_knots - deg - 1);
    const T *kn = knots + (i - 1);  // kn[r] = knots_all[i + r] (1-based), r in [-deg, deg]
    for (int m = 0; m <= maxd; ++m) {
        double N[DA], tmp[DA];
#pragma unroll
        for (int a = 0; a < DA; ++a) N[a] = 0.0;
        N[0] = 1.0;
        const int p0 = deg - m;
#pragma unroll
        for (int k = 1; k < DA; ++k) {
            if (k > deg) break;
#pragma unroll
            for (int a = 0; a < DA; ++a) tmp[a] = 0.0;
            const bool value_step = (k <= p0);
#pragma unroll
            for (int kk = 1; kk < DA; ++kk) {
                if (kk > k) break;
                const double t_min = (double)kn[kk - k];
                const double t_max = (double)kn[kk];
                const double dt = t_max - t_min;
                if (value_step) {  // src/spline_dimension.jl:190-198
                    const double frac = N[kk - 1] / dt;
                    tmp[kk - 1] += frac * (t_max - t);
                    tmp[kk] = frac * (t - t_min);
                } else {           // src/spline_dimension.jl:200-205
                    const double dc = N[kk - 1] * (double)k / dt;
                    tmp[kk - 1] -= dc;
                    tmp[kk] = dc;
                }
            }
#pragma unroll
            for (int a = 0; a < DA; ++a) N[a] = tmp[a];
        }
#pragma unroll
        for (int a = 0; a < DA; ++a)
            if (a <= deg) eval[l + ns * (a + (int64_t)(deg + 1) * m)] = (T)N[a];
    }
}

// decompress_basis_function_eval_kernel (src/util_kernels.jl:51-67) into a zeroed
// dense [ns, n_basis] matrix: one thread per (sample, basis function) writes the
// table value inside the support and 0 outside, so no separate memset is needed.
template <typename T>
__global__ void k_decompress(const T *__restrict__ eval, const int32_t *__restrict__ sidx,
                             int64_t ns, int degree, int order, int64_t n_basis,
                             T *__restrict__ out) {
    int64_t lin = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (lin >= ns * n_basis) return;
    const int64_t l = lin % ns, k = lin / ns;  // k: 0-based basis function
    const int64_t first = (int64_t)sidx[l] - degree - 1;  // 0-based support start
    const int64_t j = k - first;
    T v = (T)0;
    if (j >= 0 && j <= degree) v = eval[l + ns * (j + (int64_t)(degree + 1) * order)];
    out[lin] = v;
}

template <typename T>
static int launch_basis(int degree, const void *knots, int64_t n_knots, const void *samples,
                        const int32_t *sidx, int64_t ns, int maxd, void *eval, cudaStream_t s) {
    const int bs = 128;
    const unsigned g = (unsigned)((ns + bs - 1) / bs);
    const T *kn = (const T *)knots;
    const T *sp = (const T *)samples;
    T *ev = (T *)eval;
    if (degree > SG_MAX_DEGREE)
        return set_error(SG_ERR_UNSUPPORTED, "degree %d exceeds SG_MAX_DEGREE=%d", degree,
                         SG_MAX_DEGREE);
    switch (degree) {
        case 0: k_basis<1, T><<<g, bs, 0, s>>>(kn, n_knots, sp, sidx, ns, degree, maxd, ev); break;
        case 1: k_basis<2, T><<<g, bs, 0, s>>>(kn, n_knots, sp, sidx, ns, degree, maxd, ev); break;
        case 2: k_basis<3, T><<<g, bs, 0, s>>>(kn, n_knots, sp, sidx, ns, degree, maxd, ev); break;
        case 3: k_basis<4, T><<<g, bs, 0, s>>>(kn, n_knots, sp, sidx, ns, degree, maxd, ev); break;
        default: k_basis<0, T><<<g, bs, 0, s>>>(kn, n_knots, sp, sidx, ns, degree, maxd, ev); break;
    }
    return cuda_check(cudaGetLastError(), "k_basis launch");
}

}  // namespace sg

using namespace sg;

extern "C" int sg_expand_knots(int32_t dtype, const void *knot_values,
                               const int32_t *multiplicities, int64_t n_values,
                               int64_t n_knots, void *knots_all, sg_stream_t stream) {
    if (n_values <= 0 || n_knots <= 0 || !knot_values || !multiplicities || !knots_all)
        return set_error(SG_ERR_INVALID_ARGUMENT, "sg_expand_knots: empty or NULL input");
    cudaStream_t s = (cudaStream_t)stream;
    const int bs = 128;
    const unsigned g = (unsigned)((n_values + bs - 1) / bs);
    if (dtype == SG_F32)
        k_expand_knots<float><<<g, bs, 0, s>>>((const float *)knot_values, multiplicities,
                                              n_values, n_knots, (float *)knots_all);
    else if (dtype == SG_F64)
        k_expand_knots<double><<<g, bs, 0, s>>>((const double *)knot_values, multiplicities,
                                               n_values, n_knots, (double *)knots_all);
    else
        return set_error(SG_ERR_INVALID_ARGUMENT, "sg_expand_knots: dtype must be F32 or F64");
    return cuda_check(cudaGetLastError(), "k_expand_knots launch");
}

extern "C" int sg_sample_indices(int32_t dtype, const void *sample_points, int64_t n_samples,
                                 const void *knots_all, int64_t n_knots, int32_t degree,
                                 int32_t *sample_indices, sg_stream_t stream) {
    if (n_samples < 0 || n_knots < 2 * degree + 2 || degree < 0)
        return set_error(SG_ERR_INVALID_ARGUMENT,
                         "sg_sample_indices: need n_knots >= 2*degree+2 (got %lld, degree %d)",
                         (long long)n_knots, degree);
    if (n_samples == 0) return SG_OK;
    if (!sample_points || !knots_all || !sample_indices)
        return set_error(SG_ERR_INVALID_ARGUMENT, "sg_sample_indices: NULL pointer");
    cudaStream_t s = (cudaStream_t)stream;
    const int bs = 256;
    const unsigned g = (unsigned)((n_samples + bs - 1) / bs);
    if (dtype == SG_F32)
        k_sample_indices<float><<<g, bs, 0, s>>>((const float *)sample_points, n_samples,
                                                (const float *)knots_all, n_knots, degree,
                                                sample_indices);
    else if (dtype == SG_F64)
        k_sample_indices<double><<<g, bs, 0, s>>>((const double *)sample_points, n_samples,
                                                 (const double *)knots_all, n_knots, degree,
                                                 sample_indices);
    else
        return set_error(SG_ERR_INVALID_ARGUMENT, "sg_sample_indices: dtype must be F32 or F64");
    return cuda_check(cudaGetLastError(), "k_sample_indices launch");
}

extern "C" int sg_basis_eval(int32_t dtype, const void *knots_all, int64_t n_knots,
                             const void *sample_points, const int32_t *sample_indices,
                             int64_t n_samples, int32_t degree, int32_t max_derivative_order,
                             void *eval, sg_stream_t stream) {
    if (degree < 0 || degree > SG_MAX_DEGREE)
        return set_error(SG_ERR_UNSUPPORTED, "sg_basis_eval: degree %d outside 0..%d", degree,
                         SG_MAX_DEGREE);
    if (max_derivative_order < 0 || max_derivative_order > degree)
        return set_error(SG_ERR_INVALID_ARGUMENT,
                         "sg_basis_eval: max_derivative_order must be in 0..degree "
                         "(src/spline_dimension.jl:309)");
    if (n_knots < 2 * degree + 2)
        return set_error(SG_ERR_INVALID_ARGUMENT, "sg_basis_eval: too few knots");
    if (n_samples == 0) return SG_OK;
    if (!knots_all || !sample_points || !sample_indices || !eval || n_samples < 0)
        return set_error(SG_ERR_INVALID_ARGUMENT, "sg_basis_eval: NULL pointer");
    cudaStream_t s = (cudaStream_t)stream;
    if (dtype == SG_F32)
        return launch_basis<float>(degree, knots_all, n_knots, sample_points, sample_indices,
                                   n_samples, max_derivative_order, eval, s);
    if (dtype == SG_F64)
        return launch_basis<double>(degree, knots_all, n_knots, sample_points, sample_indices,
                                    n_samples, max_derivative_order, eval, s);
    return set_error(SG_ERR_INVALID_ARGUMENT, "sg_basis_eval: dtype must be F32 or F64");
}

extern "C" int sg_decompress(int32_t dtype, const void *eval, const int32_t *sample_indices,
                             int64_t n_samples, int32_t degree, int32_t max_derivative_order,
                             int32_t derivative_order, int64_t n_basis, void *out,
                             sg_stream_t stream) {
    if (degree < 0 || max_derivative_order < 0 || max_derivative_order > degree ||
        derivative_order < 0 || derivative_order > max_derivative_order || n_basis <= degree)
        return set_error(SG_ERR_INVALID_ARGUMENT, "sg_decompress: bad degree/order/n_basis");
    const int64_t tot = n_samples * n_basis;
    if (tot == 0) return SG_OK;
    if (!eval || !sample_indices || !out)
        return set_error(SG_ERR_INVALID_ARGUMENT, "sg_decompress: NULL pointer");
    cudaStream_t s = (cudaStream_t)stream;
    const int bs = 256;
    const unsigned g = (unsigned)((tot + bs - 1) / bs);
    if (dtype == SG_F32)
        k_decompress<float><<<g, bs, 0, s>>>((const float *)eval, sample_indices, n_samples,
                                            degree, derivative_order, n_basis, (float *)out);
    else if (dtype == SG_F64)
        k_decompress<double><<<g, bs, 0, s>>>((const double *)eval, sample_indices, n_samples,
                                             degree, derivative_order, n_basis, (double *)out);
    else
        return set_error(SG_ERR_INVALID_ARGUMENT, "sg_decompress: dtype must be F32 or F64");
    return cuda_check(cudaGetLastError(), "k_decompress launch");
}
