// jv_kern_f32.cu -- single-precision instances of the general kernels (c2c
// shared-memory kernel, global-memory path, capacity query, helper kernels of
// the real long transforms); the real
// transforms' shared-memory kernels are in jv_kern_f32r.cu.
#include "jv_launch.cuh"

namespace jv {
bool launch_smem_f32(const Job &j, cudaStream_t s) {
    if (j.kind == K_C2C && j.cin.cst == 1 && j.cout.cst == 1) return launch_smem_split_f32(j, s);
    if (j.kind == K_C2C) return launch_smem_t<float, K_C2C>(j, s);
    return launch_smem_real_f32(j, s);
}
bool launch_global_f32(const Job &j, cudaStream_t s) { return launch_global_t<float>(j, s); }
long smem_max_len_f32(int kind) { return smem_len_limit<float>(kind); }
bool launch_r2c_pairs_f32(void *z, long es, long vs, long N, long nvec, int has_scale, double scale,
                         const void *thalf, cudaStream_t s) {
    return launch_r2c_pairs_t<float>(z, es, vs, N, nvec, has_scale, scale, thalf, s);
}
bool launch_c2r_unsplit_f32(const Job &j, void *ydst, cudaStream_t s) { return launch_c2r_unsplit_t<float>(j, ydst, s); }
bool launch_c2r_unpack_f32(const Job &j, const void *y, cudaStream_t s) { return launch_c2r_unpack_t<float>(j, y, s); }
}  // namespace jv
