// Fused single-pass leapfrog schedule (see the kernel comment).
#include "sj_physics.cuh"

namespace sj {

template <typename real>
cudaError_t launch_fused_step(const InstDev<real>*, const InstDev<real>*, int, DevState*,
                              cudaStream_t, int) {
    return cudaErrorNotSupported;
}

template cudaError_t launch_fused_step<double>(const InstDev<double>*, const InstDev<double>*, int,
                                               DevState*, cudaStream_t, int);
template cudaError_t launch_fused_step<float>(const InstDev<float>*, const InstDev<float>*, int,
                                              DevState*, cudaStream_t, int);
}  // namespace sj
