// Sweep kernels of the PolF32x2 element type (see sweep_star7_impl.cuh).
#include "sweep_star7_impl.cuh"

namespace scafes {

cudaError_t launch_star7_f32x2(const Star7Launch& a, cudaStream_t stream) {
    return launch_prec<PolF32x2>(a, stream);
}

cudaError_t launch_star7_tb_f32x2(const Star7Launch& a, cudaStream_t stream) {
    return launch_tb_prec<PolF32x2>(a, stream);
}

cudaError_t prepare_star7_tb_f32x2() { return prepare_tb_prec<PolF32x2>(); }

}  // namespace scafes
