// sg_select.cu -- device selection for local refinement: the reductions and
// order-preserving compactions behind error_informed_local_refinement!
// (src/control_points.jl:555-578) and deactivate_overwritten_control_points!
// (src/control_points.jl:584-680).
//
// The reference maps the error onto the control points with the adjoint, sums it over
// the outputs, compares each control point with threshold_factor * mean and collects the
// selected positions with `findall` (column-major order), then merges them with a
// level's existing indices by `unique` on the CPU.  The deactivation propagates Boolean
// `Flag` values through the adjoint refinement and keeps the rows whose flag survives
// (`findall` again).  Here every step stays on the device:
//   * sg_sum_outputs: per control point, the sum over outputs in output order (the
//     reference's `sum(...; dims = Nin + 1)`), and the total in FP64 by a fixed-order
//     two-level reduction (per-block partials, then one block);
//   * sg_select_above / sg_select_rows: flag -> per-tile counts -> one-block exclusive
//     scan -> scatter, so the selected entries keep their order exactly as `findall`
//     returns them, and the result is the same on every run.
#include "sg_common.cuh"

namespace sg {
namespace {

constexpr int kSelThreads = 256;
constexpr int kSelPer = 4;                        // consecutive elements per thread
constexpr int kSelTile = kSelThreads * kSelPer;   // elements per block
constexpr int kRedBlocks = 1024;                  // partial sums of sg_sum_outputs

int64_t sel_tiles(int64_t n) { return (n + kSelTile - 1) / kSelTile; }

// Workspace layout (bytes): [counts int64 tiles][offsets int64 tiles][total int64 2]
// [partials double kRedBlocks][mask uint8 n]
struct SelWork {
    int64_t *counts, *offs, *total;
    double *partials;
    unsigned char *mask;
};
SelWork carve(void *ws, int64_t n) {
    const int64_t t = sel_tiles(n) + 1;
    SelWork w;
    w.counts = reinterpret_cast<int64_t *>(ws);
    w.offs = w.counts + t;
    w.total = w.offs + t;
    w.partials = reinterpret_cast<double *>(w.total + 2);
    w.mask = reinterpret_cast<unsigned char *>(w.partials + kRedBlocks);
    return w;
}

__device__ __forceinline__ double block_sum_d(double v, double *sh) {
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
    return r;
}

// Exclusive scan of one int per thread over the block; returns the thread's offset and
// writes the block total to *tot (all threads).
__device__ __forceinline__ int block_exscan(int v, int *sh, int *tot) {
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (l >= o) x += y;
    }
    __syncthreads();
    if (l == 31) sh[w] = x;
    __syncthreads();
    if (w == 0) {
        int s = l < (int)(blockDim.x >> 5) ? sh[l] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, s, o);
            if (l >= o) s += y;
        }
        if (l < (int)(blockDim.x >> 5)) sh[l] = s;  // inclusive warp prefix
    }
    __syncthreads();
    const int before = (w > 0 ? sh[w - 1] : 0) + x - v;
    *tot = sh[(blockDim.x >> 5) - 1];
    return before;
}

// ------------------------------------------------------------------ sum over outputs
template <typename T>
__global__ void __launch_bounds__(kSelThreads) k_sum_outputs(const T *__restrict__ in, int64_t ncp, int nout,
                                                T *__restrict__ out, double *__restrict__ partials) {
    __shared__ double sh[kSelThreads / 32];
    double s = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < ncp;
         i += (int64_t)gridDim.x * blockDim.x) {
        T v = in[i];
        for (int o = 1; o < nout; ++o) v += in[i + ncp * o];
        out[i] = v;
        s += (double)v;
    }
    s = block_sum_d(s, sh);
    if (threadIdx.x == 0) partials[blockIdx.x] = s;
}

__global__ void __launch_bounds__(kSelThreads) k_sum_partials(const double *__restrict__ partials, int nb,
                                                 double *__restrict__ total) {
    __shared__ double sh[kSelThreads / 32];
    double s = 0.0;
    for (int i = threadIdx.x; i < nb; i += blockDim.x) s += partials[i];
    s = block_sum_d(s, sh);
    if (threadIdx.x == 0) *total = s;
}

// ------------------------------------------------------------------ compaction
struct AboveFlag {  // values[i] > factor * total / n, and i not excluded
    const void *values;
    int dtype;
    const double *total;
    double factor;
    int64_t n;
    const unsigned char *mask;
    __device__ bool operator()(int64_t i) const {
        const double thr = factor * (*total) / (double)n;
        const double v = dtype == SG_F64 ? ((const double *)values)[i] : (double)((const float *)values)[i];
        return v > thr && !(mask && mask[i]);
    }
};
struct KeepFlag {  // keep[i] > 0
    const double *keep;
    __device__ bool operator()(int64_t i) const { return keep[i] > 0.0; }
};

template <typename F>
__global__ void __launch_bounds__(kSelThreads) k_sel_count(F flag, int64_t n, int64_t *__restrict__ counts) {
    __shared__ int sh[kSelThreads / 32];
    const int64_t base = (int64_t)blockIdx.x * kSelTile + (int64_t)threadIdx.x * kSelPer;
    int c = 0;
#pragma unroll
    for (int k = 0; k < kSelPer; ++k)
        if (base + k < n && flag(base + k)) ++c;
    int tot;
    (void)block_exscan(c, sh, &tot);
    if (threadIdx.x == 0) counts[blockIdx.x] = tot;
}

// one block: offs = exclusive scan of counts, total[0] = sum
__global__ void __launch_bounds__(kSelThreads) k_sel_scan(const int64_t *__restrict__ counts, int64_t tiles,
                                             int64_t *__restrict__ offs, int64_t *__restrict__ total) {
    __shared__ int sh[kSelThreads / 32];
    int64_t run = 0;
    for (int64_t t0 = 0; t0 < tiles; t0 += kSelThreads) {
        const int64_t t = t0 + threadIdx.x;
        const int c = t < tiles ? (int)counts[t] : 0;
        int tot;
        const int before = block_exscan(c, sh, &tot);
        if (t < tiles) offs[t] = run + before;
        run += tot;
        __syncthreads();
    }
    if (threadIdx.x == 0) total[0] = run;
}

struct AboveWriter {  // linear control point i -> 1-based multi-index (+ gathered values)
    int nin;
    int64_t size[SG_MAX_NIN];
    int64_t ncp;
    int nout;
    int dtype;
    const void *src;
    int32_t *out_idx;
    void *out_vals;
    int64_t cap;
    __device__ void operator()(int64_t i, int64_t pos) const {
        int64_t r = i;
        for (int d = 0; d < nin; ++d) {
            out_idx[pos + cap * d] = (int32_t)(r % size[d] + 1);
            r /= size[d];
        }
        if (src) {
            for (int o = 0; o < nout; ++o) {
                if (dtype == SG_F64)
                    ((double *)out_vals)[pos + cap * o] = ((const double *)src)[i + ncp * o];
                else
                    ((float *)out_vals)[pos + cap * o] = ((const float *)src)[i + ncp * o];
            }
        }
    }
};
struct RowWriter {  // row i of [n, nin] indices and [n, nout] values -> row pos
    int nin, nout, dtype;
    int64_t n;
    const int32_t *idx_in;
    const void *vals_in;
    int32_t *idx_out;
    void *vals_out;
    __device__ void operator()(int64_t i, int64_t pos) const {
        for (int d = 0; d < nin; ++d) idx_out[pos + n * d] = idx_in[i + n * d];
        for (int o = 0; o < nout; ++o) {
            if (dtype == SG_F64)
                ((double *)vals_out)[pos + n * o] = ((const double *)vals_in)[i + n * o];
            else
                ((float *)vals_out)[pos + n * o] = ((const float *)vals_in)[i + n * o];
        }
    }
};

template <typename F, typename W>
__global__ void __launch_bounds__(kSelThreads) k_sel_scatter(F flag, W write, int64_t n, const int64_t *__restrict__ offs) {
    __shared__ int sh[kSelThreads / 32];
    const int64_t base = (int64_t)blockIdx.x * kSelTile + (int64_t)threadIdx.x * kSelPer;
    bool f[kSelPer];
    int c = 0;
#pragma unroll
    for (int k = 0; k < kSelPer; ++k) {
        f[k] = base + k < n && flag(base + k);
        c += f[k] ? 1 : 0;
    }
    int tot;
    int64_t pos = offs[blockIdx.x] + block_exscan(c, sh, &tot);
#pragma unroll
    for (int k = 0; k < kSelPer; ++k)
        if (f[k]) write(base + k, pos++);
}

// mask[linear index of row r] = 1 for rows of 1-based indices [n_rows, nin]; rows outside
// the grid are ignored
__global__ void k_sel_mark(const int32_t *__restrict__ idx, int64_t n_rows, int nin,
                           AboveWriter geo, unsigned char *__restrict__ mask) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n_rows) return;
    int64_t lin = 0, stride = 1;
    for (int d = 0; d < nin; ++d) {
        const int64_t v = (int64_t)idx[r + n_rows * d] - 1;
        if (v < 0 || v >= geo.size[d]) return;
        lin += v * stride;
        stride *= geo.size[d];
    }
    mask[lin] = 1;
}

template <typename F, typename W>
int compact(F flag, W write, int64_t n, SelWork w, int64_t *n_out, cudaStream_t s) {
    const int64_t tiles = sel_tiles(n);
    if (tiles > 0) {
        k_sel_count<<<(unsigned)tiles, kSelThreads, 0, s>>>(flag, n, w.counts);
        k_sel_scan<<<1, kSelThreads, 0, s>>>(w.counts, tiles, w.offs, w.total);
        k_sel_scatter<<<(unsigned)tiles, kSelThreads, 0, s>>>(flag, write, n, w.offs);
    } else {
        cudaMemsetAsync(w.total, 0, sizeof(int64_t), s);
    }
    int rc = cuda_check(cudaGetLastError(), "select: launch");
    if (!rc) rc = cuda_check(cudaMemcpyAsync(n_out, w.total, sizeof(int64_t), cudaMemcpyDeviceToHost, s),
                             "select: read count");
    if (!rc) rc = cuda_check(cudaStreamSynchronize(s), "select: sync");
    return rc;
}

}  // namespace
}  // namespace sg

using namespace sg;

extern "C" int64_t sg_select_workspace_bytes(int64_t n) {
    if (n < 0) return 0;
    return (int64_t)sizeof(int64_t) * (2 * (sel_tiles(n) + 1) + 2) + (int64_t)sizeof(double) * kRedBlocks +
           ((n + 15) / 16) * 16;
}

extern "C" int sg_sum_outputs(int32_t dtype, int64_t ncp, int32_t nout, const void *in, void *out,
                              double *total, void *workspace, sg_stream_t stream) {
    if (dtype != SG_F32 && dtype != SG_F64)
        return set_error(SG_ERR_INVALID_ARGUMENT, "sg_sum_outputs: dtype must be F32 or F64");
    if (ncp < 0 || nout < 1 || !total || !workspace || (ncp > 0 && (!in || !out)))
        return set_error(SG_ERR_INVALID_ARGUMENT, "sg_sum_outputs: bad arguments");
    cudaStream_t s = (cudaStream_t)stream;
    SelWork w = carve(workspace, ncp);
    int64_t nb = (ncp + kSelThreads - 1) / kSelThreads;
    nb = nb < 1 ? 1 : (nb > kRedBlocks ? kRedBlocks : nb);
    if (dtype == SG_F64)
        k_sum_outputs<double><<<(unsigned)nb, kSelThreads, 0, s>>>((const double *)in, ncp, nout,
                                                                  (double *)out, w.partials);
    else
        k_sum_outputs<float><<<(unsigned)nb, kSelThreads, 0, s>>>((const float *)in, ncp, nout,
                                                                 (float *)out, w.partials);
    k_sum_partials<<<1, kSelThreads, 0, s>>>(w.partials, (int)nb, total);
    return cuda_check(cudaGetLastError(), "sg_sum_outputs launch");
}

extern "C" int sg_select_above(int32_t dtype, int32_t nin, const int64_t *cp_size, int32_t nout,
                               const void *values, const double *total, double threshold_factor,
                               const int32_t *exclude_idx, int64_t n_exclude,
                               const void *gather_src, int32_t *out_idx, void *out_vals,
                               int64_t *n_selected, void *workspace, sg_stream_t stream) {
    if (dtype != SG_F32 && dtype != SG_F64)
        return set_error(SG_ERR_INVALID_ARGUMENT, "sg_select_above: dtype must be F32 or F64");
    if (nin < 1 || nin > SG_MAX_NIN || !cp_size || nout < 1 || !n_selected || !workspace ||
        !total || n_exclude < 0 || (n_exclude > 0 && !exclude_idx) || (gather_src && !out_vals))
        return set_error(SG_ERR_INVALID_ARGUMENT, "sg_select_above: bad arguments");
    AboveWriter wr{};
    wr.nin = nin;
    int64_t ncp = 1;
    for (int d = 0; d < nin; ++d) {
        if (cp_size[d] < 0) return set_error(SG_ERR_INVALID_ARGUMENT, "sg_select_above: negative size");
        wr.size[d] = cp_size[d];
        ncp *= cp_size[d];
    }
    *n_selected = 0;
    if (ncp == 0) return SG_OK;
    if (!values || !out_idx) return set_error(SG_ERR_INVALID_ARGUMENT, "sg_select_above: NULL array");
    cudaStream_t s = (cudaStream_t)stream;
    SelWork w = carve(workspace, ncp);
    const unsigned char *mask = nullptr;
    if (n_exclude > 0) {
        int rc = cuda_check(cudaMemsetAsync(w.mask, 0, (size_t)ncp, s), "select: clear mask");
        if (rc) return rc;
        k_sel_mark<<<(unsigned)((n_exclude + 255) / 256), 256, 0, s>>>(exclude_idx, n_exclude, nin, wr,
                                                                       w.mask);
        mask = w.mask;
    }
    wr.ncp = ncp;
    wr.nout = nout;
    wr.dtype = dtype;
    wr.src = gather_src;
    wr.out_idx = out_idx;
    wr.out_vals = out_vals;
    wr.cap = ncp;
    AboveFlag fl{values, dtype, total, threshold_factor, ncp, mask};
    return compact(fl, wr, ncp, w, n_selected, s);
}

extern "C" int sg_select_rows(int32_t dtype, int64_t n, const double *keep, int32_t nin,
                              const int32_t *idx_in, int32_t nout, const void *vals_in,
                              int32_t *idx_out, void *vals_out, int64_t *n_kept, void *workspace,
                              sg_stream_t stream) {
    if (dtype != SG_F32 && dtype != SG_F64)
        return set_error(SG_ERR_INVALID_ARGUMENT, "sg_select_rows: dtype must be F32 or F64");
    if (n < 0 || nin < 1 || nin > SG_MAX_NIN || nout < 0 || !n_kept || !workspace)
        return set_error(SG_ERR_INVALID_ARGUMENT, "sg_select_rows: bad arguments");
    *n_kept = 0;
    if (n == 0) return SG_OK;
    if (!keep || !idx_in || !idx_out || (nout > 0 && (!vals_in || !vals_out)))
        return set_error(SG_ERR_INVALID_ARGUMENT, "sg_select_rows: NULL array");
    RowWriter wr{nin, nout, dtype, n, idx_in, vals_in, idx_out, vals_out};
    return compact(KeepFlag{keep}, wr, n, carve(workspace, n), n_kept, (cudaStream_t)stream);
}
