// jv_batch.cu -- batching form: many independent c2c fftm calls in one
// persistent launch fed by a device work queue.
#include "jv_core.h"

using namespace jv;

struct jvsip_fftm_batchplan_s {
    int dummy;
};

extern "C" {
int jvsip_fftm_batch_f(size_t n, const vsip_fftm_f *const plans[], const vsip_cmview_f *const in[],
                       const vsip_cmview_f *const out[]) {
    (void)n; (void)plans; (void)in; (void)out;
    set_error(E_UNSUPPORTED, "batching form not available");
    return E_UNSUPPORTED;
}
jvsip_fftm_batchplan_f *jvsip_fftm_batch_create_f(size_t n, const vsip_fftm_f *const plans[],
                                                  const vsip_cmview_f *const in[], const vsip_cmview_f *const out[]) {
    (void)n; (void)plans; (void)in; (void)out;
    set_error(E_UNSUPPORTED, "batching form not available");
    return nullptr;
}
int jvsip_fftm_batch_run_f(jvsip_fftm_batchplan_f *b) { (void)b; return E_UNSUPPORTED; }
int jvsip_fftm_batch_destroy_f(jvsip_fftm_batchplan_f *b) { (void)b; return 0; }
}
