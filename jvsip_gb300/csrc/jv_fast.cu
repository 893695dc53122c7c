// jv_fast.cu -- specialised register-resident kernels for the hot shapes.
#include "jv_core.h"

namespace jv {
bool launch_fast_f32(const Job &j, cudaStream_t s) {
    (void)j;
    (void)s;
    return false;
}
}  // namespace jv
