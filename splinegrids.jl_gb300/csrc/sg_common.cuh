// sg_common.cuh -- shared device helpers of libsplinegrids_b200 (sm_103a only).
#pragma once

#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <stdint.h>

#include "splinegrids_b200.h"

#if defined(__CUDA_ARCH__) && (__CUDA_ARCH__ != 1030)
#error "libsplinegrids_b200 is built for sm_103a (GB300) only"
#endif

namespace sg {

// Register windows of the generic (runtime-degree) kernels hold this many values.
constexpr int kDMax = SG_MAX_DEGREE + 1;

// Status / error plumbing (host side, sg_api.cu).
int set_error(int code, const char *fmt, ...);
int cuda_check(cudaError_t e, const char *what);
// Device allocations of plans and handles (counted; a test hook can make them fail).
// dev_alloc sets *out to NULL and returns SG_ERR_OUT_OF_MEMORY on failure; dev_free
// accepts NULL.
int dev_alloc(void **out, size_t bytes, const char *what);
void dev_free(void *p);
// Derivative orders of an evaluate call against the descriptor (sg_api.cu): the
// reference's codes and messages for NURBS derivatives and unavailable orders.
int check_orders(const sg_grid_desc &d, const int32_t *ord);

// ------------------------------------------------------------------ loads / stores
__device__ __forceinline__ float to_f(float v) { return v; }
__device__ __forceinline__ double to_f(double v) { return v; }
__device__ __forceinline__ float to_f(__nv_bfloat16 v) { return __bfloat162float(v); }

template <typename TO, typename TI>
__device__ __forceinline__ TO ld_as(const TI *p) {
    return (TO)to_f(*p);
}

// A group of VEC consecutive values of T, moved as one 4/8/16-byte access when the
// caller guarantees alignment.
template <typename T, int VEC>
struct alignas((VEC * sizeof(T)) < 16 ? (VEC * sizeof(T)) : 16) Pack {
    T v[VEC];
};

template <typename T, int VEC>
__device__ __forceinline__ Pack<T, VEC> ldp(const T *p) {
    Pack<T, VEC> r;
    if constexpr (VEC == 4 && sizeof(T) == 4) {
        float4 t = *reinterpret_cast<const float4 *>(p);
        r.v[0] = t.x; r.v[1] = t.y; r.v[2] = t.z; r.v[3] = t.w;
    } else if constexpr (VEC == 2 && sizeof(T) == 8) {
        double2 t = *reinterpret_cast<const double2 *>(p);
        r.v[0] = t.x; r.v[1] = t.y;
    } else {
#pragma unroll
        for (int i = 0; i < VEC; ++i) r.v[i] = p[i];
    }
    return r;
}

// Streaming store (evict-first): used for eval, which is written once and not
// re-read by this launch, so it does not push the separable intermediates out of L2.
template <typename T, int VEC>
__device__ __forceinline__ void stp_stream(T *p, const Pack<T, VEC> &a) {
    if constexpr (VEC == 4 && sizeof(T) == 4) {
        __stcs(reinterpret_cast<float4 *>(p), make_float4(a.v[0], a.v[1], a.v[2], a.v[3]));
    } else if constexpr (VEC == 2 && sizeof(T) == 8) {
        __stcs(reinterpret_cast<double2 *>(p), make_double2(a.v[0], a.v[1]));
    } else {
#pragma unroll
        for (int i = 0; i < VEC; ++i) __stcs(p + i, a.v[i]);
    }
}

template <typename T, int VEC>
__device__ __forceinline__ void stp(T *p, const Pack<T, VEC> &a) {
    if constexpr (VEC == 4 && sizeof(T) == 4) {
        *reinterpret_cast<float4 *>(p) = make_float4(a.v[0], a.v[1], a.v[2], a.v[3]);
    } else if constexpr (VEC == 2 && sizeof(T) == 8) {
        *reinterpret_cast<double2 *>(p) = make_double2(a.v[0], a.v[1]);
    } else {
#pragma unroll
        for (int i = 0; i < VEC; ++i) p[i] = a.v[i];
    }
}

__device__ __forceinline__ int64_t clamp64(int64_t v, int64_t lo, int64_t hi) {
    return v < lo ? lo : (v > hi ? hi : v);
}

// 0-based first control point of the support of a sample with 1-based knot-span
// index `idx` (control_point_index_base of src/spline_grid.jl:145-146, made 0-based).
// Clamped into [0, n-1-d] so that malformed indices never address outside the
// control-point array.
__device__ __forceinline__ int64_t support_start(int32_t idx, int d, int64_t n) {
    return clamp64((int64_t)idx - d - 1, 0, n - 1 - d);
}

}  // namespace sg
