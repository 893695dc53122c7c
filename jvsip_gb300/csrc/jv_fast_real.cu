// jv_fast_real.cu -- the register-resident kernel on real rows: vsip_rcfftmop_f
// (R2C) and vsip_crfftmop_f (C2R) with VSIP_ROW-contiguous real rows, as the
// half-length complex transform with the real packing fused into its first
// pass and the Hermitian split / merge fused into its last / first pass.
#include <stdint.h>

#include "jv_fast.cuh"

namespace jv {

template <int RM, int FXK = 0>
static bool launch_fast_real_t(const Job &j, cudaStream_t st) {
    switch (j.N) {
        case 64: return launch_fast_n<64, 4, 64, RList<16, 4>, false, false, false, false, RM, FXK>(j, st);
        case 128: return launch_fast_n<128, 8, 32, RList<16, 8>, false, false, false, false, RM, FXK>(j, st);
        case 256: return launch_fast_n<256, 16, 16, RList<16, 16>, false, false, false, false, RM, FXK>(j, st);
        case 512: return launch_fast_n<512, 32, 8, RList<16, 16, 2>, false, false, false, false, RM, FXK>(j, st);
        // 768 points: 4 rows per CTA, 7 CTAs per SM (measured on 4096 x 1536
        // R2C / C2R: 21.1 / 21.6 us against 23.8 / 23.3 us for 8 rows per CTA
        // at 3 CTAs per SM)
        case 768: return launch_fast_n<768, 32, 4, RList<12, 8, 8>, false, false, false, false, RM, FXK>(j, st);
        case 1000: return launch_fast_n<1000, 100, 4, RList<10, 10, 10>, false, false, false, false, RM, FXK>(j, st);
        case 1024: return launch_fast_n<1024, 64, 4, RList<16, 16, 4>, false, false, false, false, RM, FXK>(j, st);
        case 2048: return launch_fast_n<2048, 128, 2, RList<16, 16, 8>, false, false, false, false, RM, FXK>(j, st);
        case 4096: return launch_fast_n<4096, 256, 1, RList<16, 16, 16>, false, false, false, false, RM, FXK>(j, st);
        case 8192: return launch_fast_n<8192, 512, 1, RList<16, 16, 16, 2>, false, false, false, false, RM, FXK>(j, st);
        default: return false;
    }
}

// Real rows of unit stride in a real block (not a real view of a complex
// block), even offset and pitch and 8-byte aligned, so x_{2n}, x_{2n+1} form
// one complex element; complex rows interleaved, unit element stride, 8-byte
// aligned; rows of one call not overlapping.  False when the call does not
// qualify (the shared-memory kernel takes it).
static bool real_rows(const RView &r, long len, long nvec) {
    if (r.rst != 1 || r.es != 1 || (r.off & 1) || (nvec > 1 && ((r.vs & 1) || labs(r.vs) < len))) return false;
    return ((uintptr_t)r.a % 8) == 0;
}
static bool complex_rows(const CView &c, long len, long nvec) {
    if (c.cst != 2 || (const float *)c.im != (const float *)c.re + 1 || ((uintptr_t)c.re % 8)) return false;
    return c.es == 1 && (nvec <= 1 || labs(c.vs) >= len);
}
// R2C output: interleaved rows of any element stride whose elements are
// distinct -- unit-stride rows not overlapping, or rows interleaved element by
// element (|vs| * nvec <= |es|, e.g. a column-major spectrum)
static bool complex_out(const CView &c, long len, long nvec) {
    if (c.cst != 2 || (const float *)c.im != (const float *)c.re + 1 || ((uintptr_t)c.re % 8)) return false;
    if (c.es == 1) return nvec <= 1 || labs(c.vs) >= len;
    return c.es != 0 && c.vs != 0 && labs(c.vs) * nvec <= labs(c.es);
}

bool launch_fast_real_f32(const Job &j, cudaStream_t st) {
    if (j.no_fast || j.prec != P_F32 || !j.thalf || !j.twp) return false;
    if (j.lp || j.nbatch > 1 || j.tw_lo || j.gram || j.taper_n) return false;
    if (j.nvec <= 0 || j.nvec > 0x7fffffffL) return false;
    if (j.kind == K_R2C) {
        if (!real_rows(j.rin, 2 * j.N, j.nvec) || !complex_out(j.cout, j.N + 1, j.nvec)) return false;
        return launch_fast_real_t<1>(j, st);
    }
    if (j.kind == K_C2R) {
        if (!complex_rows(j.cin, j.N + 1, j.nvec) || !real_rows(j.rout, 2 * j.N, j.nvec)) return false;
        return launch_fast_real_t<2>(j, st);
    }
    return false;
}

// The k-omega pipeline's R2C rows: tapers applied to the loaded real pairs
// and written back (kw.c's two vsip_vmmul_f) in the first pass.
bool launch_fast_komega_r2c_f32(const Job &j, cudaStream_t st) {
    if (j.no_fast || j.prec != P_F32 || j.kind != K_R2C || !j.thalf || !j.twp || !j.taper_n || !j.taper_t ||
        !j.taper_back)
        return false;
    if (j.nvec <= 0 || j.nvec > 0x7fffffffL) return false;
    if (!real_rows(j.rin, 2 * j.N, j.nvec) || !complex_out(j.cout, j.N + 1, j.nvec)) return false;
    return launch_fast_real_t<1, FX_TAPER>(j, st);
}

}  // namespace jv
