// sg_passes_f32.cu -- Float32 instantiations of the separable passes (control points
// may be stored as bfloat16 on the axis-0 forward pass).
#include "sg_passes.cuh"

namespace sg {

int fwd_axis0_f32(const AxisPass &p, cudaStream_t s) {
    if (p.x_dtype == SG_BF16_F32) launch_fwd_axis0_m<float, __nv_bfloat16>(p, s);
    else launch_fwd_axis0_m<float, float>(p, s);
    return cuda_check(cudaGetLastError(), "fwd_axis0_f32 launch");
}

int fwd_axis_f32(const AxisPass &p, cudaStream_t s) {
    launch_fwd_axis<float>(p, s);
    return cuda_check(cudaGetLastError(), "fwd_axis_f32 launch");
}

int adj_axis_f32(const AxisPass &p, cudaStream_t s) {
    launch_adj_axis<float>(p, s);
    return cuda_check(cudaGetLastError(), "adj_axis_f32 launch");
}

int adj_axis0_f32(const AxisPass &p, cudaStream_t s) {
    launch_adj_axis0<float>(p, s);
    return cuda_check(cudaGetLastError(), "adj_axis0_f32 launch");
}

}  // namespace sg
