// sg_noalloc.cu -- evaluate! without any device allocation.
//
// Who needs this: host code that is not allowed to call cudaMalloc.  Examples are a
// Julia task running inside a stream-ordered memory pool it must not grow, a plugin
// host that hands this library a fixed device budget, and real-time loops that must
// never take the allocator's lock or risk an out-of-memory failure mid-run.  Such
// callers cannot create a plan (sg_grid_plan_create allocates the plan's scratch) but
// can still call this entry point with their own input and output arrays.
//
// How: the intermediate tensors of the separable passes live in one file-scope device
// array, `g_noalloc_scratch` (kNoAllocScratchBytes = 64 MiB, split into two 32 MiB
// halves used alternately by consecutive passes).  Every GPU that loads this library
// holds that array until the process exits.  Host code cannot use the array's name as
// a device address (in host code it names a host-side shadow), so each call looks the
// address up with cudaGetSymbolAddress while the device is current; a call made during
// a stream capture uses the address of the last call on that device, so one call should
// happen before any capture begins.  Every pass overwrites all of its output before the next pass reads
// it, so nothing in the array has to start at zero and the previous call's leftovers
// are never read.  All calls share the one array: two calls whose kernels overlap on
// the GPU (for example on two streams) race on it and must be serialized by the caller.
#include <mutex>

#include "sg_passes.cuh"

namespace sg {

constexpr size_t kNoAllocScratchBytes = size_t(64) << 20;  // 64 MiB per device
constexpr size_t kNoAllocHalfBytes = kNoAllocScratchBytes / 2;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
static void *g_noalloc_ptr[kMaxDevices] = {};
static std::mutex g_noalloc_mu;

// Device address of g_noalloc_scratch on the current device.  Looked up on every call
// that is not being captured (cheap; the address moves if the context was torn down and
// re-created, e.g. after cudaDeviceReset); during a stream capture, where the lookup
// may not be allowed, the address of the last lookup on this device is used.
static int noalloc_scratch(cudaStream_t s, void **out) {
    int dev = 0;
    int rc = cuda_check(cudaGetDevice(&dev), "noalloc: cudaGetDevice");
    if (rc) return rc;
    if (dev < 0 || dev >= kMaxDevices)
        return set_error(SG_ERR_UNSUPPORTED, "noalloc: device ordinal %d >= %d", dev, kMaxDevices);
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    rc = cuda_check(cudaStreamIsCapturing(s, &cs), "noalloc: cudaStreamIsCapturing");
    if (rc) return rc;
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (cs == cudaStreamCaptureStatusNone || !g_noalloc_ptr[dev]) {
        void *p = nullptr;
        rc = cuda_check(cudaGetSymbolAddress(&p, g_noalloc_scratch),
                        "noalloc: cudaGetSymbolAddress(g_noalloc_scratch)");
        if (rc) return rc;
        g_noalloc_ptr[dev] = p;
    }
    *out = g_noalloc_ptr[dev];
    return SG_OK;
}

}  // namespace sg

using namespace sg;

extern "C" int sg_evaluate_noalloc(const sg_grid_desc *d, const int32_t *derivative_order,
                                   const void *control_points, const void *weights, void *eval,
                                   sg_stream_t stream) {
    if (!d) return set_error(SG_ERR_INVALID_ARGUMENT, "sg_evaluate_noalloc: descriptor is NULL");
    if (d->nin < 1 || d->nin > SG_MAX_NIN || d->nout < 1)
        return set_error(SG_ERR_INVALID_ARGUMENT, "sg_evaluate_noalloc: bad nin/nout");
    if (d->dtype != SG_F32 && d->dtype != SG_F64 && d->dtype != SG_BF16_F32)
        return set_error(SG_ERR_INVALID_ARGUMENT, "sg_evaluate_noalloc: unknown dtype");
    if (!derivative_order)
        return set_error(SG_ERR_INVALID_ARGUMENT, "sg_evaluate_noalloc: derivative_order is NULL");
    const bool nurbs = d->has_weights != 0;
    if (nurbs != (weights != nullptr))
        return set_error(SG_ERR_INVALID_ARGUMENT,
                         "sg_evaluate_noalloc: weights must be given exactly for NURBS grids");
    int64_t V = 1;
    for (int k = 0; k < d->nin; ++k) {
        if (d->degree[k] < 0 || d->degree[k] > SG_MAX_DEGREE || d->n_basis[k] < d->degree[k] + 1 ||
            d->max_derivative_order[k] < 0 || d->max_derivative_order[k] > d->degree[k] ||
            d->n_samples[k] < 0 || d->n_samples[k] > INT32_MAX)
            return set_error(SG_ERR_INVALID_ARGUMENT, "sg_evaluate_noalloc: bad dimension %d", k + 1);
        V *= d->n_samples[k];
    }
    int rc = check_orders(*d, derivative_order);  // sg_evaluate's codes and messages
    if (rc) return rc;
    if (V == 0) return SG_OK;
    if (!control_points || !eval)
        return set_error(SG_ERR_INVALID_ARGUMENT, "sg_evaluate_noalloc: NULL array");
    for (int k = 0; k < d->nin; ++k)
        if (!d->sample_indices[k] || !d->basis_eval[k])
            return set_error(SG_ERR_INVALID_ARGUMENT, "sg_evaluate_noalloc: NULL dimension array");

    // The largest intermediate, [ns_0..ns_{k-1}, n_k..n_{nin-1}, channels], must fit one
    // half of the static array.
    const size_t es = d->dtype == SG_F64 ? 8 : 4;
    const int64_t ch = d->nout + (nurbs ? 1 : 0);
    for (int k = 1; k < d->nin; ++k) {
        double e = (double)ch * (double)es;
        for (int i = 0; i < d->nin; ++i) e *= (double)(i < k ? d->n_samples[i] : d->n_basis[i]);
        if (e > (double)kNoAllocHalfBytes)
            return set_error(SG_ERR_UNSUPPORTED,
                             "sg_evaluate_noalloc: this grid needs %.0f bytes of scratch after axis "
                             "%d; the allocation-free path has %zu (use a plan instead)",
                             e, k, kNoAllocHalfBytes);
    }
    cudaStream_t s = (cudaStream_t)stream;
    void *base = nullptr;
    rc = noalloc_scratch(s, &base);
    if (rc) return rc;
    void *half[2] = {base, (unsigned char *)base + kNoAllocHalfBytes};

    const bool f64 = d->dtype == SG_F64;
    const size_t bes = f64 ? 8 : 4;
    const void *X = control_points;
    for (int k = 0; k < d->nin; ++k) {
        AxisPass a;
        a.idx = d->sample_indices[k];
        a.ns = d->n_samples[k];
        a.d = d->degree[k];
        a.n = d->n_basis[k];
        a.B = (const char *)d->basis_eval[k] +
              bes * (size_t)(a.ns * (a.d + 1) * (int64_t)derivative_order[k]);
        const bool last = (k == d->nin - 1);
        a.X = X;
        a.Y = last ? eval : half[k % 2];
        a.nch = d->nout;
        a.final_pass = last;
        if (k == 0) {
            int64_t Qr = 1;
            for (int i = 1; i < d->nin; ++i) Qr *= d->n_basis[i];
            a.M = 1;
            a.Q = Qr;
            a.w = weights;
            a.mode = !nurbs ? kPlain : (last ? kRational : kHomog);
            a.x_dtype = d->dtype;
            rc = f64 ? fwd_axis0_f64(a, s) : fwd_axis0_f32(a, s);
        } else {
            int64_t M = 1, Q = ch;
            for (int i = 0; i < k; ++i) M *= d->n_samples[i];
            for (int i = k + 1; i < d->nin; ++i) Q *= d->n_basis[i];
            a.M = M;
            a.Q = Q;
            a.mode = (nurbs && last) ? kRational : kPlain;
            rc = f64 ? fwd_axis_f64(a, s) : fwd_axis_f32(a, s);
        }
        if (rc) return rc;
        X = a.Y;
    }
    return SG_OK;
}
