// jv_kern_komega.cu -- the k-omega pipeline's instances of the shared-memory
// kernel (single precision): R2C rows whose first pass tapers the real pairs
// it loads (and writes them back), and c2c columns whose last pass stores the
// power and accumulates it into the gram.  Views and lengths the
// register-resident kernel takes go there first.
#include "jv_launch.cuh"

namespace jv {
bool launch_komega_r2c_f32(const Job &j, cudaStream_t s) {
    if (j.kind != K_R2C || !j.taper_n || !j.taper_t) {
        set_error(E_ARG, "tapered R2C without tapers");
        return false;
    }
    const int e0 = jvsip_gpu_last_error();
    if (launch_fast_komega_r2c_f32(j, s)) return true;
    if (jvsip_gpu_last_error() != e0) return false;
    return launch_smem_t<float, KX_R2C_TAPER>(j, s);
}
bool launch_komega_power_f32(const Job &j, cudaStream_t s) {
    if (j.kind != K_C2C || !j.gram) {
        set_error(E_ARG, "power columns without a gram");
        return false;
    }
    const int e0 = jvsip_gpu_last_error();
    if (launch_fast_komega_power_f32(j, s)) return true;
    if (jvsip_gpu_last_error() != e0) return false;
    return launch_smem_t<float, KX_C2C_POWER>(j, s);
}
}  // namespace jv
