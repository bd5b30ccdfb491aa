// sg_passes_f64.cu -- Float64 instantiations of the separable passes.
#include "sg_passes.cuh"

namespace sg {

int fwd_axis0_f64(const AxisPass &p, cudaStream_t s) {
    launch_fwd_axis0_m<double, double>(p, s);
    return cuda_check(cudaGetLastError(), "fwd_axis0_f64 launch");
}

int fwd_axis_f64(const AxisPass &p, cudaStream_t s) {
    launch_fwd_axis<double>(p, s);
    return cuda_check(cudaGetLastError(), "fwd_axis_f64 launch");
}

int adj_axis_f64(const AxisPass &p, cudaStream_t s) {
    launch_adj_axis<double>(p, s);
    return cuda_check(cudaGetLastError(), "adj_axis_f64 launch");
}

int adj_axis0_f64(const AxisPass &p, cudaStream_t s) {
    launch_adj_axis0<double>(p, s);
    return cuda_check(cudaGetLastError(), "adj_axis0_f64 launch");
}

}  // namespace sg
