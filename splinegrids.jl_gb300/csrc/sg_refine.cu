// sg_refine.cu -- refinement-matrix application (mult!, mult_adjoint!) and the
// local-refinement overwrite (and its adjoint) that build the finest-level control
// points of LocallyRefinedControlPoints (src/control_points.jl:319-349,
// src/adjoint.jl:85-205, src/refinement_matrix.jl:365-445).
#include "sg_common.cuh"

namespace sg {

constexpr int kMaxDims = SG_MAX_NIN + 1;  // control-point dims + the Nout dim

// The banded matrices of one mult!/mult_adjoint! call, by value in kernel parameters.
struct MultArgs {
    int ndims;
    int64_t size_Y[kMaxDims];
    int64_t size_B[kMaxDims];
    int32_t rm_of_dim[kMaxDims];  // index into the arrays below, -1 when not refined
    const int32_t *rp[kMaxDims];  // row_pointer (1-based)
    const int32_t *cs[kMaxDims];  // column_start (1-based)
    const void *nz[kMaxDims];
    int64_t m[kMaxDims], n[kMaxDims], nnz[kMaxDims];
};

// Row i (0-based) of a banded matrix: 0-based first column, column count, 0-based
// nzval offset (get_column_range, src/refinement_matrix.jl:101-125).
__device__ __forceinline__ void row_extent(const MultArgs &a, int r, int64_t i, int64_t &c0,
                                           int64_t &nc, int64_t &z0) {
    const int64_t next = (i == a.m[r] - 1) ? a.nnz[r] + 1 : (int64_t)a.rp[r][i + 1];
    nc = next - a.rp[r][i];
    c0 = (int64_t)a.cs[r][i] - 1;
    z0 = (int64_t)a.rp[r][i] - 1;
}

// refinement_matrix_array_mul_kernel (src/refinement_matrix.jl:365-403): one thread per
// entry of Y sums B over the product of the row bands, in the reference's order
// (first dim fastest) with the factors multiplied in dim order.
template <typename T>
__global__ void k_mult(MultArgs a, const T *__restrict__ B, T *__restrict__ Y, int64_t NY) {
    for (int64_t lin = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; lin < NY;
         lin += (int64_t)gridDim.x * blockDim.x) {
        int64_t I[kMaxDims], c0[kMaxDims], nc[kMaxDims], z0[kMaxDims], Jb[kMaxDims];
        int64_t rem = lin, tot = 1;
        for (int dd = 0; dd < a.ndims; ++dd) {
            I[dd] = rem % a.size_Y[dd];
            rem /= a.size_Y[dd];
            const int r = a.rm_of_dim[dd];
            if (r < 0) { c0[dd] = I[dd]; nc[dd] = 1; z0[dd] = 0; }
            else row_extent(a, r, I[dd], c0[dd], nc[dd], z0[dd]);
            if (nc[dd] < 0) nc[dd] = 0;
            tot *= nc[dd];
            Jb[dd] = 0;
        }
        T out = T(0);
        for (int64_t t = 0; t < tot; ++t) {
            int64_t off = 0, stride = 1;
            bool ok = true;
            for (int dd = 0; dd < a.ndims; ++dd) {
                const int64_t J = Jb[dd] + c0[dd];
                ok = ok && J >= 0 && J < a.size_B[dd];
                off += J * stride;
                stride *= a.size_B[dd];
            }
            if (ok) {
                T contrib = B[off];
                for (int dd = 0; dd < a.ndims; ++dd) {
                    const int r = a.rm_of_dim[dd];
                    if (r >= 0) contrib *= ((const T *)a.nz[r])[z0[dd] + Jb[dd]];
                }
                out += contrib;
            }
            for (int dd = 0; dd < a.ndims; ++dd) {  // odometer, first dim fastest
                if (++Jb[dd] < nc[dd]) break;
                Jb[dd] = 0;
            }
        }
        Y[lin] = out;
    }
}

// Rows [lo, hi) of a banded matrix whose band covers column j.  column_start and the
// row ends are non-decreasing in a valid RefinementMatrix (the row checks of
// src/refinement_matrix.jl:163-178), so both bounds are binary searches.
__device__ __forceinline__ void rows_covering(const MultArgs &a, int r, int64_t j, int64_t &lo,
                                              int64_t &hi) {
    int64_t l = 0, h = a.m[r];
    while (l < h) {  // first row with column_start > j
        const int64_t mid = (l + h) >> 1;
        if ((int64_t)a.cs[r][mid] - 1 > j) h = mid; else l = mid + 1;
    }
    hi = l;
    l = 0;
    h = a.m[r];
    while (l < h) {  // first row whose last column >= j
        const int64_t mid = (l + h) >> 1;
        int64_t c0, nc, z0;
        row_extent(a, r, mid, c0, nc, z0);
        if (c0 + nc - 1 < j) l = mid + 1; else h = mid;
    }
    lo = l;
}

// mult_adjoint! (src/adjoint.jl:85-152) in gather form: one thread per entry J of B
// sums Y[I] prod A[I_d, J_d] over the rows I whose bands cover J, in a fixed order
// (first dim fastest).  Deterministic and without atomics.
template <typename T>
__global__ void k_mult_adjoint(MultArgs a, const T *__restrict__ Y, T *__restrict__ B,
                               int64_t NB) {
    for (int64_t lin = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; lin < NB;
         lin += (int64_t)gridDim.x * blockDim.x) {
        int64_t J[kMaxDims], lo[kMaxDims], cnt[kMaxDims], Ib[kMaxDims];
        int64_t rem = lin, tot = 1;
        for (int dd = 0; dd < a.ndims; ++dd) {
            J[dd] = rem % a.size_B[dd];
            rem /= a.size_B[dd];
            const int r = a.rm_of_dim[dd];
            if (r < 0) { lo[dd] = J[dd]; cnt[dd] = 1; }
            else {
                int64_t l, h;
                rows_covering(a, r, J[dd], l, h);
                lo[dd] = l;
                cnt[dd] = h > l ? h - l : 0;
            }
            tot *= cnt[dd];
            Ib[dd] = 0;
        }
        T acc = T(0);
        for (int64_t t = 0; t < tot; ++t) {
            int64_t off = 0, stride = 1;
            for (int dd = 0; dd < a.ndims; ++dd) {
                off += (lo[dd] + Ib[dd]) * stride;
                stride *= a.size_Y[dd];
            }
            T contrib = Y[off];
            for (int dd = 0; dd < a.ndims; ++dd) {
                const int r = a.rm_of_dim[dd];
                if (r >= 0) {
                    int64_t c0, nc, z0;
                    row_extent(a, r, lo[dd] + Ib[dd], c0, nc, z0);
                    contrib *= ((const T *)a.nz[r])[z0 + (J[dd] - c0)];
                }
            }
            acc += contrib;
            for (int dd = 0; dd < a.ndims; ++dd) {
                if (++Ib[dd] < cnt[dd]) break;
                Ib[dd] = 0;
            }
        }
        B[lin] = acc;
    }
}

struct RefIdx {
    int nin;
    int64_t cp_size[SG_MAX_NIN];
};

// Set by the overwrite kernels when a refinement index lies outside the control-point
// grid (that entry is skipped, so no access leaves the array).  The Python and Julia
// wrappers validate indices at set-up; this flag is a last line of defence.
__device__ int g_bad_refinement_index = 0;

__device__ __forceinline__ bool ref_linear(const RefIdx &r, const int32_t *ridx, int64_t n_ref,
                                           int64_t i, int64_t &lin) {
    lin = 0;
    int64_t stride = 1;
    for (int dd = 0; dd < r.nin; ++dd) {
        const int64_t c = (int64_t)ridx[i + n_ref * dd] - 1;
        if (c < 0 || c >= r.cp_size[dd]) return false;
        lin += c * stride;
        stride *= r.cp_size[dd];
    }
    return true;
}

// local_refinement_kernel (src/control_points.jl:296-311)
template <typename T>
__global__ void k_local_refinement(RefIdx r, int nout, int64_t n_ref, const int32_t *ridx,
                                   const T *vals, T *cp, int64_t ncp) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n_ref) return;
    int64_t lin;
    if (!ref_linear(r, ridx, n_ref, i, lin)) { g_bad_refinement_index = 1; return; }
    for (int o = 0; o < nout; ++o) cp[lin + ncp * o] = vals[i + n_ref * o];
}

// local_refinement_adjoint_kernel (src/adjoint.jl:154-170)
template <typename T>
__global__ void k_local_refinement_adjoint(RefIdx r, int nout, int64_t n_ref,
                                           const int32_t *ridx, T *vals, T *cp, int64_t ncp) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n_ref) return;
    int64_t lin;
    if (!ref_linear(r, ridx, n_ref, i, lin)) { g_bad_refinement_index = 1; return; }
    for (int o = 0; o < nout; ++o) {
        vals[i + n_ref * o] = cp[lin + ncp * o];
        cp[lin + ncp * o] = T(0);
    }
}

}  // namespace sg

using namespace sg;

static int build_mult_args(int32_t dtype, int32_t ndims, const int64_t *size_Y,
                           const int64_t *size_B, int32_t n_refmat, const sg_refmat *As,
                           const int32_t *dims_refinement, MultArgs &a, const char *who) {
    if (dtype != SG_F32 && dtype != SG_F64)
        return set_error(SG_ERR_INVALID_ARGUMENT, "%s: dtype must be F32 or F64", who);
    if (ndims < 1 || ndims > kMaxDims || !size_Y || !size_B)
        return set_error(SG_ERR_INVALID_ARGUMENT, "%s: ndims %d outside 1..%d", who, ndims, kMaxDims);
    if (n_refmat < 0 || n_refmat > ndims || (n_refmat > 0 && (!As || !dims_refinement)))
        return set_error(SG_ERR_INVALID_ARGUMENT, "%s: bad refinement matrix list", who);
    memset(&a, 0, sizeof(a));
    a.ndims = ndims;
    for (int d = 0; d < ndims; ++d) {
        a.size_Y[d] = size_Y[d];
        a.size_B[d] = size_B[d];
        a.rm_of_dim[d] = -1;
        if (size_Y[d] < 0 || size_B[d] < 0)
            return set_error(SG_ERR_INVALID_ARGUMENT, "%s: negative size", who);
    }
    // validate_mult_input, src/validation.jl:90-107
    for (int r = 0; r < n_refmat; ++r) {
        const int d = dims_refinement[r];
        if (d < 0 || d >= ndims)
            return set_error(SG_ERR_INVALID_ARGUMENT, "%s: refinement dimension %d out of range", who, d);
        if (a.rm_of_dim[d] >= 0)
            return set_error(SG_ERR_INVALID_ARGUMENT, "Refinement dimensions must be unique.");
        if (As[r].m != size_Y[d] || As[r].n != size_B[d])
            return set_error(SG_ERR_INVALID_ARGUMENT,
                             "Size of refinement matrix does not match `B` and `Y` along "
                             "refinement dimension %d.", d + 1);
        if (As[r].m > 0 && (!As[r].row_pointer || !As[r].column_start || !As[r].nzval))
            return set_error(SG_ERR_INVALID_ARGUMENT, "%s: NULL refinement matrix array", who);
        a.rm_of_dim[d] = r;
        a.rp[r] = As[r].row_pointer;
        a.cs[r] = As[r].column_start;
        a.nz[r] = As[r].nzval;
        a.m[r] = As[r].m;
        a.n[r] = As[r].n;
        a.nnz[r] = As[r].nnz;
    }
    for (int d = 0; d < ndims; ++d)
        if (a.rm_of_dim[d] < 0 && size_Y[d] != size_B[d])
            return set_error(SG_ERR_INVALID_ARGUMENT,
                             "`B` and `Y` don't have the same size along dimension %d.", d + 1);
    return SG_OK;
}

static unsigned grid_for(int64_t n, int bs) {
    int64_t g = (n + bs - 1) / bs;
    if (g > 152 * 64) g = 152 * 64;  // grid-stride beyond this
    return (unsigned)(g < 1 ? 1 : g);
}

extern "C" int sg_mult(int32_t dtype, int32_t ndims, const int64_t *size_Y,
                       const int64_t *size_B, int32_t n_refmat, const sg_refmat *As,
                       const int32_t *dims_refinement, const void *B, void *Y,
                       sg_stream_t stream) {
    MultArgs a;
    int rc = build_mult_args(dtype, ndims, size_Y, size_B, n_refmat, As, dims_refinement, a,
                             "sg_mult");
    if (rc) return rc;
    int64_t NY = 1;
    for (int d = 0; d < ndims; ++d) NY *= size_Y[d];
    if (NY == 0) return SG_OK;
    if (!B || !Y) return set_error(SG_ERR_INVALID_ARGUMENT, "sg_mult: NULL array");
    cudaStream_t s = (cudaStream_t)stream;
    if (dtype == SG_F32) k_mult<float><<<grid_for(NY, 256), 256, 0, s>>>(a, (const float *)B, (float *)Y, NY);
    else k_mult<double><<<grid_for(NY, 256), 256, 0, s>>>(a, (const double *)B, (double *)Y, NY);
    return cuda_check(cudaGetLastError(), "k_mult launch");
}

extern "C" int sg_mult_adjoint(int32_t dtype, int32_t ndims, const int64_t *size_Y,
                               const int64_t *size_B, int32_t n_refmat, const sg_refmat *As,
                               const int32_t *dims_refinement, const void *Y, void *B,
                               sg_stream_t stream) {
    MultArgs a;
    int rc = build_mult_args(dtype, ndims, size_Y, size_B, n_refmat, As, dims_refinement, a,
                             "sg_mult_adjoint");
    if (rc) return rc;
    int64_t NB = 1;
    for (int d = 0; d < ndims; ++d) NB *= size_B[d];
    if (NB == 0) return SG_OK;
    if (!B || !Y) return set_error(SG_ERR_INVALID_ARGUMENT, "sg_mult_adjoint: NULL array");
    cudaStream_t s = (cudaStream_t)stream;
    if (dtype == SG_F32)
        k_mult_adjoint<float><<<grid_for(NB, 256), 256, 0, s>>>(a, (const float *)Y, (float *)B, NB);
    else
        k_mult_adjoint<double><<<grid_for(NB, 256), 256, 0, s>>>(a, (const double *)Y, (double *)B, NB);
    return cuda_check(cudaGetLastError(), "k_mult_adjoint launch");
}

static int overwrite_common(int32_t dtype, int32_t nin, int32_t nout, const int64_t *cp_size,
                            int64_t n_refined, const int32_t *ridx, const void *vals, void *cp,
                            RefIdx &r, int64_t &ncp, const char *who) {
    if (dtype != SG_F32 && dtype != SG_F64)
        return set_error(SG_ERR_INVALID_ARGUMENT, "%s: dtype must be F32 or F64", who);
    if (nin < 1 || nin > SG_MAX_NIN || nout < 1 || !cp_size || n_refined < 0)
        return set_error(SG_ERR_INVALID_ARGUMENT, "%s: bad dimensions", who);
    r.nin = nin;
    ncp = 1;
    for (int d = 0; d < nin; ++d) {
        r.cp_size[d] = cp_size[d];
        ncp *= cp_size[d];
    }
    if (n_refined > 0 && (!ridx || !vals || !cp))
        return set_error(SG_ERR_INVALID_ARGUMENT, "%s: NULL array", who);
    return SG_OK;
}

extern "C" int sg_local_refinement(int32_t dtype, int32_t nin, int32_t nout,
                                   const int64_t *cp_size, int64_t n_refined,
                                   const int32_t *refinement_indices,
                                   const void *refinement_values, void *control_points,
                                   sg_stream_t stream) {
    RefIdx r;
    int64_t ncp;
    int rc = overwrite_common(dtype, nin, nout, cp_size, n_refined, refinement_indices,
                              refinement_values, control_points, r, ncp, "sg_local_refinement");
    if (rc || n_refined == 0) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    const unsigned g = (unsigned)((n_refined + 255) / 256);
    if (dtype == SG_F32)
        k_local_refinement<float><<<g, 256, 0, s>>>(r, nout, n_refined, refinement_indices,
                                                    (const float *)refinement_values,
                                                    (float *)control_points, ncp);
    else
        k_local_refinement<double><<<g, 256, 0, s>>>(r, nout, n_refined, refinement_indices,
                                                     (const double *)refinement_values,
                                                     (double *)control_points, ncp);
    return cuda_check(cudaGetLastError(), "k_local_refinement launch");
}

extern "C" int sg_local_refinement_adjoint(int32_t dtype, int32_t nin, int32_t nout,
                                           const int64_t *cp_size, int64_t n_refined,
                                           const int32_t *refinement_indices,
                                           void *refinement_values, void *control_points,
                                           sg_stream_t stream) {
    RefIdx r;
    int64_t ncp;
    int rc = overwrite_common(dtype, nin, nout, cp_size, n_refined, refinement_indices,
                              refinement_values, control_points, r, ncp,
                              "sg_local_refinement_adjoint");
    if (rc || n_refined == 0) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    const unsigned g = (unsigned)((n_refined + 255) / 256);
    if (dtype == SG_F32)
        k_local_refinement_adjoint<float><<<g, 256, 0, s>>>(r, nout, n_refined, refinement_indices,
                                                            (float *)refinement_values,
                                                            (float *)control_points, ncp);
    else
        k_local_refinement_adjoint<double><<<g, 256, 0, s>>>(r, nout, n_refined, refinement_indices,
                                                             (double *)refinement_values,
                                                             (double *)control_points, ncp);
    return cuda_check(cudaGetLastError(), "k_local_refinement_adjoint launch");
}
