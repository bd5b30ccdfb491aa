/*
 * sg_oracle.c -- CPU restatement of the SplineGrids.jl grid-evaluation hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity oracle and the timed CPU
 * baseline.  Only tests/, __graft_entry__.smoke() and bench.py (its cpu_baseline
 * leg and its reference arm) may load it.  The product library never links it.
 *
 * Every function restates one KernelAbstractions kernel of the reference
 * (SouthEndMusic/SplineGrids.jl v0.1.1) with the same loop order and the same
 * accumulation type Tv.  Array layouts are the reference's: Julia column-major,
 * first index fastest, 1-based Int32 sample indices.  The reference runs on the
 * KA CPU() backend, which splits the ndrange over threads; the OpenMP loops here
 * do the same over the slowest sample dimension.
 *
 * Parity pins: the golden vectors and known-answer tests of the reference's own
 * test files (test/test_spline_grid.jl:29-53, test/test_knot_vector.jl:26-42,
 * test/test_nurbs_grid.jl:25-52, test/test_local_refinement.jl:48-67,
 * test/test_spline_dimension.jl:10-66), checked in tests/test_oracle_golden.py.
 *
 * Every function exists for Tv = double (suffix _f64) and Tv = float (_f32).
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define OR_MAX_NIN 8

int or_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void or_set_num_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

/* ------------------------------------------------------------------------ */
/* Integer work: identical for both value types.                            */
/* ------------------------------------------------------------------------ */

/* Multi-index helper: linear index -> Cartesian (first dim fastest). */
static void lin2cart(int64_t lin, int nd, const int64_t *sz, int64_t *out) {
    for (int d = 0; d < nd; ++d) {
        out[d] = lin % sz[d];
        lin /= sz[d];
    }
}

static int64_t cart2lin(int nd, const int64_t *sz, const int64_t *I) {
    int64_t lin = 0, stride = 1;
    for (int d = 0; d < nd; ++d) {
        lin += I[d] * stride;
        stride *= sz[d];
    }
    return lin;
}

/* Row extent of a banded RefinementMatrix, 1-based format of
 * src/refinement_matrix.jl:101-125 (get_column_end / get_column_range). */
static void rm_row(const int32_t *row_pointer, const int32_t *column_start, int64_t m,
                   int64_t nnz, int64_t i /*0-based*/, int64_t *cs0, int64_t *ncols,
                   int64_t *rp0) {
    int64_t next = (i == m - 1) ? nnz + 1 : row_pointer[i + 1];
    *ncols = next - row_pointer[i];
    *cs0 = (int64_t)column_start[i] - 1;
    *rp0 = (int64_t)row_pointer[i] - 1;
}

/* local_refinement_kernel's index read: refinement_indices[i, dim] (column-major,
 * n_refined x Nin, 1-based). */
static int64_t ref_lin_index(const int32_t *ridx, int64_t n_ref, int64_t i, int nin,
                             const int64_t *cp_size) {
    int64_t lin = 0, stride = 1;
    for (int d = 0; d < nin; ++d) {
        lin += ((int64_t)ridx[i + n_ref * d] - 1) * stride;
        stride *= cp_size[d];
    }
    return lin;
}

/* ------------------------------------------------------------------------ */
/* Value-type templated code.                                               */
/* ------------------------------------------------------------------------ */

#define OR_DEFINE(Tv, SFX)                                                                 \
                                                                                           \
/* expand_knot_vector_kernel, src/util_kernels.jl:1-20 */                                  \
void or_expand_knots_##SFX(const Tv *knot_values, const int32_t *mult, int64_t n_values,   \
                           Tv *knots_all) {                                                \
    for (int64_t i = 0; i < n_values; ++i) {                                               \
        int64_t s = 0;                                                                     \
        for (int64_t j = 0; j < i; ++j) s += mult[j];                                      \
        for (int64_t k = s; k < s + mult[i]; ++k) knots_all[k] = knot_values[i];           \
    }                                                                                      \
}                                                                                          \
                                                                                           \
/* set_sample_indices_kernel, src/util_kernels.jl:22-49: linear scan with early break,  */ \
/* then clamp to [degree+1, n_knots-degree-1]; output 1-based.                          */ \
void or_sample_indices_##SFX(const Tv *samples, int64_t ns, const Tv *knots_all,          \
                             int64_t n_knots, int degree, int32_t *out) {                  \
    _Pragma("omp parallel for schedule(static)")                                           \
    for (int64_t l = 0; l < ns; ++l) {                                                     \
        Tv t = samples[l];                                                                 \
        int64_t idx = 0;                                                                   \
        for (int64_t k = 0; k < n_knots; ++k) {                                            \
            if (t < knots_all[k]) break;                                                   \
            idx += 1;                                                                      \
        }                                                                                  \
        int64_t lo = degree + 1, hi = n_knots - degree - 1;                                \
        if (idx < lo) idx = lo;                                                            \
        if (idx > hi) idx = hi;                                                            \
        out[l] = (int32_t)idx;                                                             \
    }                                                                                      \
}                                                                                          \
                                                                                           \
/* spline_dimension_kernel, src/spline_dimension.jl:160-215.  eval and the private      */ \
/* eval_prev are [ns, degree+1, max_deriv+1] column-major; this keeps the reference's   */ \
/* per-sample loop order, including the clears and the copies into eval_prev.           */ \
void or_basis_##SFX(const Tv *knots_all, const Tv *samples, const int32_t *sidx,           \
                    int64_t ns, int degree, int maxd, Tv *eval) {                          \
    const int D = degree + 1, MD = maxd + 1;                                               \
    _Pragma("omp parallel")                                                                \
    {                                                                                      \
        Tv *prev = (Tv *)malloc(sizeof(Tv) * (size_t)(D * MD));                            \
        Tv *cur = (Tv *)malloc(sizeof(Tv) * (size_t)(D * MD));                             \
        _Pragma("omp for schedule(static)")                                                \
        for (int64_t l = 0; l < ns; ++l) {                                                 \
            Tv t = samples[l];                                                             \
            int64_t i = sidx[l]; /* 1-based */                                             \
            for (int q = 0; q < D * MD; ++q) { prev[q] = (Tv)0; cur[q] = (Tv)0; }          \
            cur[0] = (Tv)1;                                                                \
            prev[0] = (Tv)1;                                                               \
            for (int k = 1; k <= degree; ++k) {                                            \
                for (int q = 0; q < D * MD; ++q) cur[q] = (Tv)0;                           \
                for (int k_ = 1; k_ <= k; ++k_) {                                          \
                    Tv t_min = knots_all[i + k_ - k - 1];                                  \
                    Tv t_max = knots_all[i + k_ - 1];                                      \
                    Tv dt = t_max - t_min;                                                 \
                    Tv B_prev = prev[(k_ - 1)];                                            \
                    Tv frac = B_prev / dt;                                                 \
                    cur[k_ - 1] += frac * (t_max - t);                                     \
                    cur[k_] = frac * (t - t_min);                                          \
                    for (int m = 1; m <= maxd + k - degree; ++m) {                         \
                        Tv Bp = prev[(k_ - 1) + D * (m - 1)];                              \
                        Tv dc = Bp * (Tv)k / dt;                                           \
                        cur[(k_ - 1) + D * m] -= dc;                                       \
                        cur[k_ + D * m] = dc;                                              \
                    }                                                                      \
                }                                                                          \
                if (k != degree)                                                           \
                    for (int q = 0; q < D * MD; ++q) prev[q] = cur[q];                     \
            }                                                                              \
            for (int m = 0; m < MD; ++m)                                                   \
                for (int j = 0; j < D; ++j)                                                \
                    eval[l + ns * (j + (int64_t)D * m)] = cur[j + D * m];                  \
        }                                                                                  \
        free(prev);                                                                        \
        free(cur);                                                                         \
    }                                                                                      \
}                                                                                          \
                                                                                           \
/* spline_eval_kernel, src/spline_grid.jl:119-183.  One work item per sample J; the     */ \
/* (d+1)^Nin support loop runs first dim fastest; the basis product is formed in dim    */ \
/* order; NURBS multiplies by the weight, accumulates the denominator and divides.      */ \
/* basis[k] points at the whole [ns_k, d_k+1, maxd_k+1] table of dim k.                 */ \
void or_eval_##SFX(int nin, int nout, const int64_t *ns, const int64_t *ncp,               \
                   const int32_t *deg, const int32_t *maxd, const int32_t *const *sidx,    \
                   const Tv *const *basis, const int32_t *order, const Tv *cp,             \
                   const Tv *w, Tv *eval) {                                                \
    int64_t V = 1, NCP = 1, K = 1;                                                         \
    int64_t ksz[OR_MAX_NIN];                                                               \
    for (int k = 0; k < nin; ++k) { V *= ns[k]; NCP *= ncp[k]; ksz[k] = deg[k] + 1;        \
                                    K *= ksz[k]; }                                         \
    (void)maxd;                                                                            \
    const int64_t slow = ns[nin - 1], inner = V / slow;                                    \
    _Pragma("omp parallel for schedule(static)")                                           \
    for (int64_t js = 0; js < slow; ++js) {                                                \
        for (int64_t ji = 0; ji < inner; ++ji) {                                           \
            int64_t lin = ji + inner * js;                                                 \
            int64_t J[OR_MAX_NIN], base[OR_MAX_NIN], I[OR_MAX_NIN], c[OR_MAX_NIN];         \
            lin2cart(lin, nin, ns, J);                                                     \
            for (int o = 0; o < nout; ++o) eval[lin + V * o] = (Tv)0;                      \
            Tv denom = (Tv)0;                                                              \
            for (int k = 0; k < nin; ++k) base[k] = (int64_t)sidx[k][J[k]] - deg[k] - 1;   \
            for (int64_t kk = 0; kk < K; ++kk) {                                           \
                lin2cart(kk, nin, ksz, I);                                                 \
                for (int k = 0; k < nin; ++k) c[k] = base[k] + I[k];                       \
                Tv prod = (Tv)1;                                                           \
                for (int k = 0; k < nin; ++k)                                              \
                    prod *= basis[k][J[k] + ns[k] * (I[k] + ksz[k] * (int64_t)order[k])];  \
                int64_t clin = cart2lin(nin, ncp, c);                                      \
                Tv bm = prod;                                                              \
                if (w) { bm = prod * w[clin]; denom += bm; }                               \
                for (int o = 0; o < nout; ++o)                                             \
                    eval[lin + V * o] += bm * cp[clin + NCP * o];                          \
            }                                                                              \
            if (w)                                                                         \
                for (int o = 0; o < nout; ++o) eval[lin + V * o] /= denom;                 \
        }                                                                                  \
    }                                                                                      \
}                                                                                          \
                                                                                           \
/* spline_eval_adjoint_kernel + evaluate_adjoint!, src/adjoint.jl:1-83: zero the        */ \
/* control points, then scatter prod * eval_bar into every support control point.  The  */ \
/* reference scatters with atomics; here each thread scatters into a private buffer and */ \
/* the buffers are summed in thread order, so the result is deterministic for a given   */ \
/* thread count.  Non-NURBS only, as in the reference.                                  */ \
void or_eval_adjoint_##SFX(int nin, int nout, const int64_t *ns, const int64_t *ncp,       \
                           const int32_t *deg, const int32_t *const *sidx,                 \
                           const Tv *const *basis, const int32_t *order,                   \
                           const Tv *ebar, Tv *cpbar) {                                    \
    int64_t V = 1, NCP = 1, K = 1;                                                         \
    int64_t ksz[OR_MAX_NIN];                                                               \
    for (int k = 0; k < nin; ++k) { V *= ns[k]; NCP *= ncp[k]; ksz[k] = deg[k] + 1;        \
                                    K *= ksz[k]; }                                         \
    const int64_t tot = NCP * nout;                                                        \
    const int nth = or_num_threads();                                                      \
    Tv *priv = (Tv *)calloc((size_t)tot * (size_t)nth, sizeof(Tv));                        \
    const int64_t slow = ns[nin - 1], inner = V / slow;                                    \
    _Pragma("omp parallel")                                                                \
    {                                                                                      \
        int tid = 0;                                                                       \
        IF_OMP(tid = omp_get_thread_num();)                                                \
        Tv *mine = priv + (size_t)tid * (size_t)tot;                                       \
        _Pragma("omp for schedule(static)")                                                \
        for (int64_t js = 0; js < slow; ++js) {                                            \
            for (int64_t ji = 0; ji < inner; ++ji) {                                       \
                int64_t lin = ji + inner * js;                                             \
                int64_t J[OR_MAX_NIN], base[OR_MAX_NIN], I[OR_MAX_NIN], c[OR_MAX_NIN];     \
                lin2cart(lin, nin, ns, J);                                                 \
                for (int k = 0; k < nin; ++k)                                              \
                    base[k] = (int64_t)sidx[k][J[k]] - deg[k] - 1;                         \
                for (int64_t kk = 0; kk < K; ++kk) {                                       \
                    lin2cart(kk, nin, ksz, I);                                             \
                    for (int k = 0; k < nin; ++k) c[k] = base[k] + I[k];                   \
                    Tv prod = (Tv)1;                                                       \
                    for (int k = 0; k < nin; ++k)                                          \
                        prod *= basis[k][J[k] + ns[k] * (I[k] + ksz[k] *                   \
                                                         (int64_t)order[k])];              \
                    int64_t clin = cart2lin(nin, ncp, c);                                  \
                    for (int o = 0; o < nout; ++o)                                         \
                        mine[clin + NCP * o] += prod * ebar[lin + V * o];                  \
                }                                                                          \
            }                                                                              \
        }                                                                                  \
    }                                                                                      \
    for (int64_t q = 0; q < tot; ++q) {                                                    \
        Tv s = (Tv)0;                                                                      \
        for (int t = 0; t < nth; ++t) s += priv[(size_t)t * (size_t)tot + (size_t)q];      \
        cpbar[q] = s;                                                                      \
    }                                                                                      \
    free(priv);                                                                            \
}                                                                                          \
                                                                                           \
/* refinement_matrix_array_mul_kernel + mult!, src/refinement_matrix.jl:365-445 and     */ \
/* get_row_extends, src/utils.jl:204-235.  Y[I] = sum_J B[J] prod_dims A_d[I_d, J_d];   */ \
/* refmat_of_dim[d] = -1 for a dimension that is not refined.  Matrices are in the      */ \
/* reference's 1-based banded format.                                                   */ \
void or_mult_##SFX(int ndims, const int64_t *size_Y, const int64_t *size_B,                \
                   const int32_t *refmat_of_dim, const int32_t *const *row_pointer,        \
                   const int32_t *const *column_start, const Tv *const *nzval,             \
                   const int64_t *m_rows, const int64_t *nnz, const Tv *B, Tv *Y) {        \
    int64_t NY = 1;                                                                        \
    for (int d = 0; d < ndims; ++d) NY *= size_Y[d];                                       \
    _Pragma("omp parallel for schedule(static)")                                           \
    for (int64_t lin = 0; lin < NY; ++lin) {                                               \
        int64_t I[OR_MAX_NIN + 1], cs[OR_MAX_NIN + 1], nc[OR_MAX_NIN + 1],                 \
            rp[OR_MAX_NIN + 1], Jb[OR_MAX_NIN + 1], J[OR_MAX_NIN + 1];                     \
        lin2cart(lin, ndims, size_Y, I);                                                   \
        int64_t tot = 1;                                                                   \
        for (int d = 0; d < ndims; ++d) {                                                  \
            int r = refmat_of_dim[d];                                                      \
            if (r < 0) { cs[d] = I[d]; nc[d] = 1; rp[d] = 0; }                             \
            else rm_row(row_pointer[r], column_start[r], m_rows[r], nnz[r], I[d], &cs[d],  \
                        &nc[d], &rp[d]);                                                   \
            tot *= nc[d];                                                                  \
        }                                                                                  \
        Tv out = (Tv)0;                                                                    \
        for (int64_t t = 0; t < tot; ++t) {                                                \
            lin2cart(t, ndims, nc, Jb);                                                    \
            for (int d = 0; d < ndims; ++d) J[d] = Jb[d] + cs[d];                          \
            Tv contrib = B[cart2lin(ndims, size_B, J)];                                    \
            for (int d = 0; d < ndims; ++d) {                                              \
                int r = refmat_of_dim[d];                                                  \
                if (r >= 0) contrib *= nzval[r][rp[d] + Jb[d]];                            \
            }                                                                              \
            out += contrib;                                                                \
        }                                                                                  \
        Y[lin] = out;                                                                      \
    }                                                                                      \
}                                                                                          \
                                                                                           \
/* refinement_matrix_array_mul_adjoint_kernel + mult_adjoint!, src/adjoint.jl:85-152:   */ \
/* B .= 0, then scatter Y[I] * prod A into B[J].  Serial, so deterministic.             */ \
void or_mult_adjoint_##SFX(int ndims, const int64_t *size_Y, const int64_t *size_B,        \
                           const int32_t *refmat_of_dim, const int32_t *const *row_pointer, \
                           const int32_t *const *column_start, const Tv *const *nzval,     \
                           const int64_t *m_rows, const int64_t *nnz, const Tv *Y, Tv *B) { \
    int64_t NY = 1, NB = 1;                                                                \
    for (int d = 0; d < ndims; ++d) { NY *= size_Y[d]; NB *= size_B[d]; }                  \
    for (int64_t q = 0; q < NB; ++q) B[q] = (Tv)0;                                         \
    for (int64_t lin = 0; lin < NY; ++lin) {                                               \
        int64_t I[OR_MAX_NIN + 1], cs[OR_MAX_NIN + 1], nc[OR_MAX_NIN + 1],                 \
            rp[OR_MAX_NIN + 1], Jb[OR_MAX_NIN + 1], J[OR_MAX_NIN + 1];                     \
        lin2cart(lin, ndims, size_Y, I);                                                   \
        int64_t tot = 1;                                                                   \
        for (int d = 0; d < ndims; ++d) {                                                  \
            int r = refmat_of_dim[d];                                                      \
            if (r < 0) { cs[d] = I[d]; nc[d] = 1; rp[d] = 0; }                             \
            else rm_row(row_pointer[r], column_start[r], m_rows[r], nnz[r], I[d], &cs[d],  \
                        &nc[d], &rp[d]);                                                   \
            tot *= nc[d];                                                                  \
        }                                                                                  \
        for (int64_t t = 0; t < tot; ++t) {                                                \
            lin2cart(t, ndims, nc, Jb);                                                    \
            for (int d = 0; d < ndims; ++d) J[d] = Jb[d] + cs[d];                          \
            Tv contrib = Y[lin];                                                           \
            for (int d = 0; d < ndims; ++d) {                                              \
                int r = refmat_of_dim[d];                                                  \
                if (r >= 0) contrib *= nzval[r][rp[d] + Jb[d]];                            \
            }                                                                              \
            B[cart2lin(ndims, size_B, J)] += contrib;                                      \
        }                                                                                  \
    }                                                                                      \
}                                                                                          \
                                                                                           \
/* local_refinement_kernel, src/control_points.jl:296-311: cp[idx_i, o] = vals[i, o].   */ \
void or_local_refinement_##SFX(int nin, int nout, const int64_t *cp_size, int64_t n_ref,   \
                               const int32_t *ridx, const Tv *vals, Tv *cp) {              \
    int64_t NCP = 1;                                                                       \
    for (int d = 0; d < nin; ++d) NCP *= cp_size[d];                                       \
    for (int64_t i = 0; i < n_ref; ++i) {                                                  \
        int64_t lin = ref_lin_index(ridx, n_ref, i, nin, cp_size);                         \
        for (int o = 0; o < nout; ++o) cp[lin + NCP * o] = vals[i + n_ref * o];            \
    }                                                                                      \
}                                                                                          \
                                                                                           \
/* local_refinement_adjoint_kernel, src/adjoint.jl:154-170: gather, then zero.          */ \
void or_local_refinement_adjoint_##SFX(int nin, int nout, const int64_t *cp_size,          \
                                       int64_t n_ref, const int32_t *ridx, Tv *vals,       \
                                       Tv *cp) {                                           \
    int64_t NCP = 1;                                                                       \
    for (int d = 0; d < nin; ++d) NCP *= cp_size[d];                                       \
    for (int64_t i = 0; i < n_ref; ++i) {                                                  \
        int64_t lin = ref_lin_index(ridx, n_ref, i, nin, cp_size);                         \
        for (int o = 0; o < nout; ++o) {                                                   \
            vals[i + n_ref * o] = cp[lin + NCP * o];                                       \
            cp[lin + NCP * o] = (Tv)0;                                                     \
        }                                                                                  \
    }                                                                                      \
}

#ifdef _OPENMP
#define IF_OMP(x) x
#else
#define IF_OMP(x)
#endif

OR_DEFINE(double, f64)
OR_DEFINE(float, f32)

/* decompress_basis_function_eval_kernel, src/util_kernels.jl:51-67 with
 * decompress, src/spline_dimension.jl:251-272: dense [ns, n_basis] basis matrix for one
 * derivative order.  out must be zeroed by the caller (the reference allocates zeros). */
void or_decompress_f64(const double *eval, const int32_t *sidx, int64_t ns, int degree,
                       int order, int64_t n_basis, double *out) {
    (void)n_basis;
    for (int64_t i = 0; i < ns; ++i) {
        int64_t l = sidx[i];
        int j = 0;
        for (int64_t k = l - degree; k <= l; ++k) {
            out[i + ns * (k - 1)] = eval[i + ns * (j + (int64_t)(degree + 1) * order)];
            ++j;
        }
    }
}

/* RefinementMatrix structural validity, validate_refinement_matrix_kernel,
 * src/refinement_matrix.jl:127-181.  valid[i] = 1 when row i passes. */
void or_validate_refinement_matrix(const int32_t *row_pointer, const int32_t *column_start,
                                   int64_t m, int64_t nnz, int64_t n_columns, uint8_t *valid) {
    for (int64_t i = 0; i < m; ++i) {
        int64_t cs, nc, rp;
        rm_row(row_pointer, column_start, m, nnz, i, &cs, &nc, &rp);
        int64_t c0 = cs + 1, c1 = cs + nc; /* 1-based start/end */
        int ok = (c1 >= c0);
        if (ok) ok = (c0 >= 1) && (c1 <= n_columns);
        if (i == 0) ok = (c0 == 1) && (row_pointer[0] == 1);
        if (ok && i > 0) {
            int64_t pcs, pnc, prp;
            rm_row(row_pointer, column_start, m, nnz, i - 1, &pcs, &pnc, &prp);
            int64_t p0 = pcs + 1, p1 = pcs + pnc;
            ok = (p0 <= c0) && (c0 <= p1 + 1);
            if (ok) ok = (c1 >= p1);
        }
        valid[i] = (uint8_t)ok;
    }
}
