// jv_kern_f32s.cu -- single-precision c2c instance of the shared-memory
// kernel for split complex views (real and imaginary parts in separate
// arrays, cstride 1): the fused first and last passes read and write the two
// arrays directly.
#include "jv_launch.cuh"

namespace jv {
bool launch_smem_split_f32(const Job &j, cudaStream_t s) { return launch_smem_t<float, KX_C2C_SPLIT>(j, s); }
}  // namespace jv
