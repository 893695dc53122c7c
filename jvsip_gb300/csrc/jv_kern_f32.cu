// jv_kern_f32.cu -- single-precision instances of the general kernels (c2c
// shared-memory kernel, global-memory path, capacity query); the real
// transforms' shared-memory kernels are in jv_kern_f32r.cu.
#include "jv_launch.cuh"

namespace jv {
bool launch_smem_f32(const Job &j, cudaStream_t s) {
    if (j.kind == K_C2C) return launch_smem_t<float, K_C2C>(j, s);
    return launch_smem_real_f32(j, s);
}
bool launch_global_f32(const Job &j, cudaStream_t s) { return launch_global_t<float>(j, s); }
long smem_max_len_f32(int kind) { return smem_len_limit<float>(kind); }
}  // namespace jv
