// jv_komega.cu -- jvsip_komega_f: the k-omega power estimate of the
// reference's kw example (examples/komegaExamples/kw_c/kw.c:8-26) as two
// launches of the shared-memory kernel.
//
// The reference runs it as seven library calls, each a pass over the data:
//   vsip_vmmul_f(ts_taper, data, VSIP_ROW, data)      data[i][j] = ts[j] * data[i][j]
//   vsip_vmmul_f(array_taper, data, VSIP_COL, data)   data[i][j] = arr[i] * data[i][j]
//   vsip_rcfftmop_f(rcfftm, data, freq)               rows, real -> complex
//   vsip_ccfftmip_f(ccfftm, freq)                     columns, in place
//   vsip_mcmagsq_f(freq, real(freq))                  p = re*re + im*im
//   vsip_smmul_f(scale, real(freq), real(freq))       p = scale * p
//   vsip_madd_f(real(freq), gram, gram)               gram = p + gram
// Here the tapers are applied (and written back to data) as the R2C's first
// pass loads the rows, and the column transform's last pass stores (p, Im X)
// into freq and adds p to the gram: two HBM round trips of the data and the
// spectrum instead of seven.  Every product and sum of the tapers and of the
// power is rounded in the reference's order; the transforms agree with the
// reference within the fftm acceptance tolerance.
#include <string.h>

#include "jv_core.h"

namespace jv {

static void plan_job(Job &j, const Plan *p, int kind) {
    j.kind = kind;
    j.prec = p->prec;
    j.N = p->MN;
    j.nvec = p->mN;
    j.inv = (p->dir == 1) ? 1 : 0;
    j.has_scale = (p->scale != 1.0) ? 1 : 0;
    j.scale = p->scale;
    j.tw = p->d_tw;
    j.thalf = p->d_thalf;
    j.twp = p->d_twp;
    j.twg = p->d_twg;
    j.pc = p->d_pc;
    j.form = 0;
    j.no_fast = p->no_fast;  // JVSIP_GPU_NO_FAST: the shared-memory kernel's instances only
    j.tma_columns = p->tma_columns;
    j.npass = (int)p->radix.size();
    for (int i = 0; i < j.npass && i < 40; i++) j.radix[i] = p->radix[i];
}

// device address of real element 0 of a real block (its own mirror, or the
// real / imaginary part of a mirrored complex parent); nullptr when not resident
static float *real_base(const vsip_block_f *b) {
    Mirror *m = mirror_find(b);
    if (m) return (float *)m->d;
    if (b->parent) {
        Mirror *pm = mirror_find(b->parent);
        if (pm) {
            const bool split = b->parent->cstride == 1;
            if (b == b->parent->R) return (float *)pm->d;
            return split ? (float *)pm->d_im : (float *)pm->d + 1;
        }
    }
    return nullptr;
}

static int fail(int code, const char *msg) {
    set_error(code, msg);
    return code;
}

static int komega(const vsip_fftm_f *rcp, const vsip_fftm_f *ccp, const vsip_vview_f *ts,
                  const vsip_vview_f *arr, const vsip_mview_f *data, const vsip_cmview_f *freq, float scale,
                  const vsip_mview_f *gram) {
    Plan *rc = plan_of(rcp), *cc = plan_of(ccp);
    if (!rc || !cc || !ts || !arr || !data || !freq || !gram) return fail(E_ARG, "null plan or view");
    if (rc->type != JV_RCFFTOP || rc->major != 0 || rc->prec != P_F32)
        return fail(E_ARG, "rcfftm must be a VSIP_ROW rcfftmop _f plan");
    if ((cc->type != JV_CCFFTIP && cc->type != JV_CCFFTOP) || cc->major != 1 || cc->prec != P_F32)
        return fail(E_ARG, "ccfftm must be a VSIP_COL ccfftm _f plan");
    const long Nsens = rc->mN, Nts = 2 * rc->MN, Nfreq = rc->MN + 1;
    if (cc->MN != Nsens || cc->mN != Nfreq) return fail(E_ARG, "ccfftm does not match rcfftm's spectrum");
    if (Nts < 4 || Nsens < 2) return fail(E_UNSUPPORTED, "k-omega needs at least 4 samples and 2 sensors");
    if ((long)data->row_length < Nts || (long)data->col_length < Nsens || (long)freq->row_length < Nfreq ||
        (long)freq->col_length < Nsens || (long)gram->row_length < Nfreq || (long)gram->col_length < Nsens ||
        (long)ts->length < Nts || (long)arr->length < Nsens)
        return fail(E_ARG, "view smaller than the plans");
    if (!rc->d_twg || !cc->d_twg || rc->lp || cc->lp || !rc->smooth || !cc->smooth)
        return fail(E_UNSUPPORTED, "k-omega needs lengths the shared-memory kernel takes");
    Device *d = device();
    if (!d) return E_NODEVICE;
    float *xd = real_base(data->block), *gd = real_base(gram->block);
    float *td = real_base(ts->block), *ad = real_base(arr->block);
    Mirror *fm = mirror_find(freq->block);
    if (!xd || !gd || !td || !ad || !fm)
        return fail(E_UNSUPPORTED, "k-omega needs admitted (device-resident) blocks");
    if (freq->block->cstride != 2) return fail(E_UNSUPPORTED, "k-omega needs an interleaved spectrum");
    std::lock_guard<std::mutex> l1(rc->mu);
    std::lock_guard<std::mutex> l2(cc->mu);
    cudaStream_t st = d->stream;
    // step 1: tapered rows -> R2C -> freq (rows of freq)
    Job a;
    plan_job(a, rc, K_R2C);
    a.rin.a = xd;
    a.rin.rst = data->block->rstride > 0 ? data->block->rstride : 1;
    a.rin.off = (long)data->offset;
    a.rin.es = data->row_stride;
    a.rin.vs = data->col_stride;
    a.cout.re = fm->d;
    a.cout.im = (float *)fm->d + 1;
    a.cout.cst = 2;
    a.cout.off = (long)freq->offset;
    a.cout.es = freq->row_stride;
    a.cout.vs = freq->col_stride;
    const long trs = ts->block->rstride > 0 ? ts->block->rstride : 1;
    const long ars = arr->block->rstride > 0 ? arr->block->rstride : 1;
    a.taper_n = td + trs * (long)ts->offset;
    a.taper_n_st = trs * ts->stride;
    a.taper_t = ad + ars * (long)arr->offset;
    a.taper_t_st = ars * arr->stride;
    a.taper_back = 1;
    if (!launch_komega_r2c_f32(a, st)) return jvsip_gpu_last_error() ? jvsip_gpu_last_error() : E_CUDA;
    // step 2: columns of freq in place, power into freq and the gram
    Job b;
    plan_job(b, cc, K_C2C);
    b.cin = a.cout;
    b.cin.es = freq->col_stride;
    b.cin.vs = freq->row_stride;
    b.cout = b.cin;
    b.inplace = 1;
    const long grs = gram->block->rstride > 0 ? gram->block->rstride : 1;
    b.gram = gd + grs * (long)gram->offset;
    b.gram_es = grs * gram->col_stride;
    b.gram_vs = grs * gram->row_stride;
    b.gram_scale = scale;
    if (!launch_komega_power_f32(b, st)) return jvsip_gpu_last_error() ? jvsip_gpu_last_error() : E_CUDA;
    for (const void *blk : {(const void *)data->block, (const void *)freq->block, (const void *)gram->block}) {
        Mirror *m = mirror_find(blk);
        if (m) m->device_newer = true;
    }
    if (data->block->parent) {
        Mirror *m = mirror_find(data->block->parent);
        if (m) m->device_newer = true;
    }
    if (gram->block->parent) {
        Mirror *m = mirror_find(gram->block->parent);
        if (m) m->device_newer = true;
    }
    return 0;
}

}  // namespace jv

extern "C" int jvsip_komega_f(const vsip_fftm_f *rcfftm, const vsip_fftm_f *ccfftm, const vsip_vview_f *ts_taper,
                              const vsip_vview_f *array_taper, const vsip_mview_f *data,
                              const vsip_cmview_f *freq, vsip_scalar_f scale, const vsip_mview_f *gram) {
    return jv::komega(rcfftm, ccfftm, ts_taper, array_taper, data, freq, scale, gram);
}
