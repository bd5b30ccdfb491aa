// sg_refmat.cu -- the refinement matrix of a multi-knot refinement, built on the device.
//
// The reference's refine(::SplineDimension; knots_new) (src/refinement.jl:256-284)
// inserts the knots one at a time on the host loop: each insertion builds the (n+1) x n
// single-knot matrix (build_refinement_matrix_kernel, src/refinement.jl:3-36) and the
// result is composed by the banded product R = R_knot * R
// (refinement_matrix_mul_nonzeros_kernel / refinement_matrix_multiplication_kernel,
// src/refinement_matrix.jl:184-327), one launch pair and a host round trip per knot.
//
// Here the whole sequence runs in ONE single-CTA launch: the matrix lives in a fixed-
// stride band form (row i: first column, count, and up to d+2 values at i*(d+2)), two
// copies ping-pong in global memory (L2-resident), and per knot every thread updates
// its rows from the previous copy, then the block synchronizes.  Row i of R_knot * R is
// row i of R (left of the knot), row i-1 (right of it), or (1-alpha) row(i-1) + alpha
// row(i) over the union of their bands (the affected rows), which is exactly the
// reference's structural product for these two-nonzero rows; values accumulate in the
// reference's order, 0 + a0*b0 + a1*b1, each product and sum rounded separately
// (no contraction), so the matrix is bit-identical to the composed products.  A final
// exclusive scan packs the band form into the reference's RefinementMatrix layout
// (1-based row_pointer, column_start, nzval).
#include "sg_common.cuh"

namespace sg {
namespace {

constexpr int kRmThreads = 1024;

template <typename T>
__device__ __forceinline__ T mul_rn(T a, T b);
template <>
__device__ __forceinline__ float mul_rn<float>(float a, float b) { return __fmul_rn(a, b); }
template <>
__device__ __forceinline__ double mul_rn<double>(double a, double b) { return __dmul_rn(a, b); }
template <typename T>
__device__ __forceinline__ T add_rn(T a, T b);
template <>
__device__ __forceinline__ float add_rn<float>(float a, float b) { return __fadd_rn(a, b); }
template <>
__device__ __forceinline__ double add_rn<double>(double a, double b) { return __dadd_rn(a, b); }

template <typename T>
struct Band {      // fixed-stride band form
    T *val;        // [rows][W]
    int32_t *cs;   // first column (0-based)
    int32_t *cnt;  // stored values
};

template <typename T>
__global__ void __launch_bounds__(kRmThreads)
k_refine_matrix(int degree, const T *__restrict__ knots_old, int64_t n_knots_old, int64_t n_insert,
                const T *__restrict__ knots_new, const int32_t *__restrict__ ksi_all, int W,
                T *knots_a, T *knots_b, Band<T> ba, Band<T> bb, int32_t *__restrict__ row_pointer,
                int32_t *__restrict__ column_start, T *__restrict__ nzval, int64_t *__restrict__ nnz_out,
                int *__restrict__ bad) {
    __shared__ int s_bad;
    __shared__ int64_t s_run;
    __shared__ int64_t s_part[kRmThreads / 32];
    const int tid = threadIdx.x;
    const int64_t n0 = n_knots_old - degree - 1;  // basis functions before refinement
    if (tid == 0) s_bad = 0;
    // R = identity, knots = old knots
    for (int64_t i = tid; i < n0; i += kRmThreads) {
        ba.val[i * W] = T(1);
        ba.cs[i] = (int32_t)i;
        ba.cnt[i] = 1;
    }
    for (int64_t j = tid; j < n_knots_old; j += kRmThreads) knots_a[j] = knots_old[j];
    __syncthreads();
    Band<T> cur = ba, nxt = bb;
    T *kc = knots_a, *kn = knots_b;
    int64_t n = n0, nk = n_knots_old;
    for (int64_t q = 0; q < n_insert; ++q) {
        const int ksi = ksi_all[q];  // 1-based: knots[ksi] <= t < knots[ksi + 1]
        const T t = knots_new[q];
        // every thread reads the same span and knots: the check and the exit are uniform
        if (ksi < degree + 1 || ksi > nk - degree - 1 || !(kc[ksi - 1] <= t && t < kc[ksi])) {
            if (tid == 0) *bad = 2;
            return;
        }
        // rows of R_knot * R (1-based i = 1 .. n+1, as the reference's kernel)
        for (int64_t r = tid; r <= n; r += kRmThreads) {
            const int64_t i = r + 1;
            if (i <= ksi - degree) {  // unaffected, left of the knot: row i of R
                const int c = cur.cnt[r];
                nxt.cs[r] = cur.cs[r];
                nxt.cnt[r] = c;
                for (int k = 0; k < c; ++k) nxt.val[r * W + k] = add_rn(T(0), mul_rn(T(1), cur.val[r * W + k]));
            } else if (i <= ksi) {  // affected: (1 - alpha) row(i-1) + alpha row(i)
                const T alpha = (t - kc[i - 1]) / (kc[i + degree - 1] - kc[i - 1]);
                const T a0 = T(1) - alpha, a1 = alpha;
                const int64_t k0 = r - 1, k1 = r;  // 0-based rows of R
                const int b00 = cur.cs[k0], b01 = cur.cs[k0] + cur.cnt[k0] - 1;
                const int b10 = cur.cs[k1], b11 = cur.cs[k1] + cur.cnt[k1] - 1;
                const int c0 = b00 < b10 ? b00 : b10, c1 = b01 > b11 ? b01 : b11;
                const int c = c1 - c0 + 1;
                if (c > W) {
                    atomicExch(&s_bad, 1);
                    continue;
                }
                nxt.cs[r] = c0;
                nxt.cnt[r] = c;
                for (int j = c0; j <= c1; ++j) {
                    T acc = T(0);
                    if (b00 <= j && j <= b01) acc = add_rn(acc, mul_rn(a0, cur.val[k0 * W + (j - b00)]));
                    if (b10 <= j && j <= b11) acc = add_rn(acc, mul_rn(a1, cur.val[k1 * W + (j - b10)]));
                    nxt.val[r * W + (j - c0)] = acc;
                }
            } else {  // unaffected, right of the knot: row i-1 of R
                const int64_t k = r - 1;
                const int c = cur.cnt[k];
                nxt.cs[r] = cur.cs[k];
                nxt.cnt[r] = c;
                for (int kk = 0; kk < c; ++kk) nxt.val[r * W + kk] = add_rn(T(0), mul_rn(T(1), cur.val[k * W + kk]));
            }
        }
        // knots: insert t after the first ksi knots
        for (int64_t j = tid; j <= nk; j += kRmThreads)
            kn[j] = j < ksi ? kc[j] : (j == ksi ? t : kc[j - 1]);
        __syncthreads();
        if (s_bad) break;
        Band<T> tb = cur; cur = nxt; nxt = tb;
        T *tk = kc; kc = kn; kn = tk;
        ++n;
        ++nk;
    }
    if (s_bad) {
        if (tid == 0) *bad = 1;
        return;
    }
    // pack: row_pointer = 1 + exclusive scan of counts
    if (tid == 0) s_run = 0;
    __syncthreads();
    const int lane = tid & 31, w = tid >> 5;
    for (int64_t r0 = 0; r0 < n; r0 += kRmThreads) {
        const int64_t r = r0 + tid;
        const int64_t c = r < n ? cur.cnt[r] : 0;
        int64_t x = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int64_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) s_part[w] = x;
        __syncthreads();
        if (w == 0) {
            int64_t s = s_part[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int64_t y = __shfl_up_sync(0xffffffffu, s, o);
                if (lane >= o) s += y;
            }
            s_part[lane] = s;
        }
        __syncthreads();
        const int64_t before = s_run + (w > 0 ? s_part[w - 1] : 0) + x - c;
        if (r < n) {
            row_pointer[r] = (int32_t)(before + 1);
            column_start[r] = cur.cs[r] + 1;
            for (int k = 0; k < c; ++k) nzval[before + k] = cur.val[r * W + k];
        }
        __syncthreads();
        if (tid == 0) s_run += s_part[kRmThreads / 32 - 1];
        __syncthreads();
    }
    if (tid == 0) *nnz_out = s_run;
}

}  // namespace
}  // namespace sg

using namespace sg;

extern "C" int64_t sg_refine_matrix_workspace_bytes(int32_t dtype, int32_t degree, int64_t n_knots_old,
                                                    int64_t n_insert) {
    if (degree < 0 || n_knots_old < 0 || n_insert < 0) return 0;
    const int64_t es = dtype == SG_F64 ? 8 : 4;
    const int64_t rows = n_knots_old - degree - 1 + n_insert;
    const int64_t W = degree + 2;
    const int64_t knots = n_knots_old + n_insert + 1;
    auto a16 = [](int64_t b) { return (b + 15) / 16 * 16; };
    return 2 * a16(knots * es) + 2 * (a16(rows * W * es) + 2 * a16(rows * 4)) + 16;
}

extern "C" int sg_refine_matrix(int32_t dtype, int32_t degree, const void *knots_all_old,
                                int64_t n_knots_old, int64_t n_insert, const void *knots_new,
                                const int32_t *knot_span_index, int32_t *row_pointer,
                                int32_t *column_start, void *nzval, int64_t *nnz, void *workspace,
                                sg_stream_t stream) {
    if (dtype != SG_F32 && dtype != SG_F64)
        return set_error(SG_ERR_INVALID_ARGUMENT, "sg_refine_matrix: dtype must be F32 or F64");
    if (degree < 0 || degree > SG_MAX_DEGREE || n_knots_old < degree + 2 || n_insert < 0 || !nnz ||
        !workspace || !knots_all_old || !row_pointer || !column_start || !nzval ||
        (n_insert > 0 && (!knots_new || !knot_span_index)))
        return set_error(SG_ERR_INVALID_ARGUMENT, "sg_refine_matrix: bad arguments");
    const int64_t es = dtype == SG_F64 ? 8 : 4;
    const int64_t rows = n_knots_old - degree - 1 + n_insert;
    const int W = degree + 2;
    const int64_t knots = n_knots_old + n_insert + 1;
    auto a16 = [](int64_t b) { return (b + 15) / 16 * 16; };
    char *p = (char *)workspace;
    void *ka = p; p += a16(knots * es);
    void *kb = p; p += a16(knots * es);
    void *va = p; p += a16(rows * W * es);
    int32_t *csa = (int32_t *)p; p += a16(rows * 4);
    int32_t *cna = (int32_t *)p; p += a16(rows * 4);
    void *vb = p; p += a16(rows * W * es);
    int32_t *csb = (int32_t *)p; p += a16(rows * 4);
    int32_t *cnb = (int32_t *)p; p += a16(rows * 4);
    int *bad = (int *)p;
    int64_t *nnz_dev = nullptr;
    cudaStream_t s = (cudaStream_t)stream;
    // the packed count travels through the flag word's neighbour (16 bytes reserved)
    int rc = cuda_check(cudaMemsetAsync(bad, 0, 16, s), "sg_refine_matrix: clear flag");
    if (rc) return rc;
    nnz_dev = (int64_t *)(bad + 2);
    if (dtype == SG_F64)
        k_refine_matrix<double><<<1, kRmThreads, 0, s>>>(
            degree, (const double *)knots_all_old, n_knots_old, n_insert, (const double *)knots_new,
            knot_span_index, W, (double *)ka, (double *)kb, Band<double>{(double *)va, csa, cna},
            Band<double>{(double *)vb, csb, cnb}, row_pointer, column_start, (double *)nzval, nnz_dev, bad);
    else
        k_refine_matrix<float><<<1, kRmThreads, 0, s>>>(
            degree, (const float *)knots_all_old, n_knots_old, n_insert, (const float *)knots_new,
            knot_span_index, W, (float *)ka, (float *)kb, Band<float>{(float *)va, csa, cna},
            Band<float>{(float *)vb, csb, cnb}, row_pointer, column_start, (float *)nzval, nnz_dev, bad);
    rc = cuda_check(cudaGetLastError(), "k_refine_matrix launch");
    int hbad[4] = {0, 0, 0, 0};
    if (!rc) rc = cuda_check(cudaMemcpyAsync(hbad, bad, 16, cudaMemcpyDeviceToHost, s), "sg_refine_matrix: read");
    if (!rc) rc = cuda_check(cudaStreamSynchronize(s), "sg_refine_matrix: sync");
    if (rc) return rc;
    if (hbad[0] == 2)
        return set_error(SG_ERR_DEVICE_CHECK,
                         "sg_refine_matrix: a knot span index does not bracket its knot "
                         "(knots[span] <= knot < knots[span + 1] with degree < span <= n_basis)");
    if (hbad[0])
        return set_error(SG_ERR_DEVICE_CHECK,
                         "sg_refine_matrix: a row's band exceeded degree + 2 values (knots out of order?)");
    int64_t v;
    memcpy(&v, &hbad[2], sizeof(v));
    *nnz = v;
    return SG_OK;
}
