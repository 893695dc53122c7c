// jv_kern_f64r.cu -- double-precision R2C / C2R instances of the shared-memory kernel.
#include "jv_launch.cuh"

namespace jv {
bool launch_smem_real_f64(const Job &j, cudaStream_t s) {
    return j.kind == K_R2C ? launch_smem_t<double, K_R2C>(j, s) : launch_smem_t<double, K_C2R>(j, s);
}
}  // namespace jv
