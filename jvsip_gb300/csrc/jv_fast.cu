// jv_fast.cu -- launchers of the register-resident kernel (jv_fast.cuh) for
// single-precision c2c calls: rows of unit element stride and any pitch,
// column tiles (adjacent transforms of any element stride), interleaved or
// split complex; the steps and Stockham passes of long transforms; the
// k-omega power transforms; and the radix schedule each length uses
// (fast_radices), from which the plans build the kernel's per-pass twiddle
// tables.  Each case names the CTA shape (T threads per transform, RPC
// transforms per CTA) that measured fastest.
#include <stdio.h>
#include <stdlib.h>

#include <vector>

#include "jv_fast.cuh"

namespace jv {

// Radix list of the specialised kernel for length N (empty: none).
std::vector<int> fast_radices(long N) {
    switch (N) {
        case 64: return {16, 4};
        case 128: return {16, 8};
        case 256: return {16, 16};
        case 512: return {16, 16, 2};
        case 768: return {12, 8, 8};
        case 1000: return {10, 10, 10};
        case 1024: return {16, 16, 4};
        case 2048: return {16, 16, 8};
        case 4096: return {16, 16, 16};
        case 8192: return {16, 16, 16, 2};
        default: return {};
    }
}

// Rows: T threads per transform, RPC transforms per CTA.
template <bool SPLIT, int FXK = 0>
static bool launch_fast_rows(const Job &j, cudaStream_t st) {
    switch (j.N) {
        case 64: return launch_fast_n<64, 4, 64, RList<16, 4>, SPLIT, false, false, false, 0, FXK>(j, st);
        case 128: return launch_fast_n<128, 8, 32, RList<16, 8>, SPLIT, false, false, false, 0, FXK>(j, st);
        case 256: return launch_fast_n<256, 16, 16, RList<16, 16>, SPLIT, false, false, false, 0, FXK>(j, st);
        case 512: return launch_fast_n<512, 32, 8, RList<16, 16, 2>, SPLIT, false, false, false, 0, FXK>(j, st);
        case 768: return launch_fast_n<768, 32, 4, RList<12, 8, 8>, SPLIT, false, false, false, 0, FXK>(j, st);
        case 1000: return launch_fast_n<1000, 100, 4, RList<10, 10, 10>, SPLIT, false, false, false, 0, FXK>(j, st);
        case 1024: return launch_fast_n<1024, 64, 4, RList<16, 16, 4>, SPLIT, false, false, false, 0, FXK>(j, st);
        case 2048: return launch_fast_n<2048, 128, 2, RList<16, 16, 8>, SPLIT, false, false, false, 0, FXK>(j, st);
        case 4096: return launch_fast_n<4096, 256, 1, RList<16, 16, 16>, SPLIT, false, false, false, 0, FXK>(j, st);
        case 8192: return launch_fast_n<8192, 512, 1, RList<16, 16, 16, 2>, SPLIT, false, false, false, 0, FXK>(j, st);
        default: return false;
    }
}

// Column tiles: V adjacent transforms per CTA (V * 8 bytes of each row per
// warp access), shared memory about 70 KB per CTA for the long ones.
// Measured on 2^24 points (GB/s, against the shared-memory kernel's column
// tiles): 64 points 5624 (3664), 256: 5377 (4088), 512: 3478 (2220), 1024:
// 2927 (2472), 2048: 2059 (2000), 1000 x 4096: 2054 (1785).  1000 points take
// 4 columns per CTA, 2 CTAs per SM: 29.6 us on 1000 x 4096 against 31.4 us
// for 8 columns per CTA (one CTA per SM) and 40.9 us for 2.
template <bool SPLIT, int FXK = 0>
static bool launch_fast_cols(const Job &j, cudaStream_t st) {
    switch (j.N) {
        case 64: return launch_fast_n<64, 4, 64, RList<16, 4>, SPLIT, true, false, false, 0, FXK>(j, st);
        case 128: return launch_fast_n<128, 8, 32, RList<16, 8>, SPLIT, true, false, false, 0, FXK>(j, st);
        case 256: return launch_fast_n<256, 16, 16, RList<16, 16>, SPLIT, true, false, false, 0, FXK>(j, st);
        case 512: return launch_fast_n<512, 32, 16, RList<16, 16, 2>, SPLIT, true, false, false, 0, FXK>(j, st);
        case 1000: return launch_fast_n<1000, 100, 4, RList<10, 10, 10>, SPLIT, true, false, false, 0, FXK>(j, st);
        case 1024: return launch_fast_n<1024, 64, 8, RList<16, 16, 4>, SPLIT, true, false, false, 0, FXK>(j, st);
        case 2048: return launch_fast_n<2048, 128, 4, RList<16, 16, 8>, SPLIT, true, false, false, 0, FXK>(j, st);
        // 4096 points: 4 columns per 1024-thread CTA (139 KB of shared memory),
        // 2874 GB/s on 4096 x 4096 against 1807 for 2 columns per CTA and 1823
        // for the shared-memory kernel
        case 4096: return launch_fast_n<4096, 256, 4, RList<16, 16, 16>, SPLIT, true, false, false, 0, FXK>(j, st);
        default: return false;
    }
}

// A step of a long transform (single vector: one group) in column-tile mode:
// the first step with its output twiddle (TW) and row-contiguous output, the
// second plain.  Both steps conjugate on load and store when inverse (each is
// an inverse transform of its own; the first step's twiddle is applied in the
// conjugated domain, which conjugates it).
template <bool TW>
static bool launch_fast_step_t(const Job &j, cudaStream_t st) {
    switch (j.N) {
        case 64: return launch_fast_n<64, 4, 64, RList<16, 4>, false, true, TW>(j, st);
        case 128: return launch_fast_n<128, 8, 32, RList<16, 8>, false, true, TW>(j, st);
        case 256: return launch_fast_n<256, 16, 16, RList<16, 16>, false, true, TW>(j, st);
        case 512: return launch_fast_n<512, 32, 16, RList<16, 16, 2>, false, true, TW>(j, st);
        case 1000: return launch_fast_n<1000, 100, 8, RList<10, 10, 10>, false, true, TW>(j, st);
        case 1024: return launch_fast_n<1024, 64, 8, RList<16, 16, 4>, false, true, TW>(j, st);
        case 2048: return launch_fast_n<2048, 128, 4, RList<16, 16, 8>, false, true, TW>(j, st);
        case 4096: return launch_fast_n<4096, 256, 2, RList<16, 16, 16>, false, true, TW>(j, st);
        default: return false;
    }
}

bool fast_step_len(long N) {
    return N == 64 || N == 128 || N == 256 || N == 512 || N == 1000 || N == 1024 || N == 2048 || N == 4096;
}

// A step of a long transform as column tiles: single vectors (one group), and
// the steps of several vectors, a group per grid row (the vectors of a group
// along the tiles, or the groups' twiddle exponent from the grid row).
bool launch_fast_step_f32(const Job &j, cudaStream_t st) {
    if (j.kind != K_C2C || j.prec != P_F32 || j.nbatch < 1 || j.nbatch > 65535 || !fast_step_len(j.N) || !j.twp)
        return false;
    const int ci = j.conj_in < 0 ? j.inv : j.conj_in, co = j.conj_out < 0 ? j.inv : j.conj_out;
    if (ci != j.inv || co != j.inv) return false;
    const CView &a = j.cin, &b = j.cout;
    if (a.cst != 2 || b.cst != 2 || (const float *)a.im != (const float *)a.re + 1 ||
        (const float *)b.im != (const float *)b.re + 1 || ((uintptr_t)a.re % 8) || ((uintptr_t)b.re % 8))
        return false;
    return j.tw_lo ? launch_fast_step_t<true>(j, st) : launch_fast_step_t<false>(j, st);
}

// One pass of a large-radix Stockham transform (j.sp_* set; radix j.N).
bool launch_fast_sp_f32(const Job &j, cudaStream_t st) {
    switch (j.N) {
        case 64: return launch_fast_n<64, 4, 64, RList<16, 4>, false, true, false, true>(j, st);
        case 128: return launch_fast_n<128, 8, 32, RList<16, 8>, false, true, false, true>(j, st);
        case 256: return launch_fast_n<256, 16, 16, RList<16, 16>, false, true, false, true>(j, st);
        case 512: return launch_fast_n<512, 32, 16, RList<16, 16, 2>, false, true, false, true>(j, st);
        case 1024: return launch_fast_n<1024, 64, 8, RList<16, 16, 4>, false, true, false, true>(j, st);
        case 2048: return launch_fast_n<2048, 128, 4, RList<16, 16, 8>, false, true, false, true>(j, st);
        case 4096: return launch_fast_n<4096, 256, 2, RList<16, 16, 16>, false, true, false, true>(j, st);
        default: return false;
    }
}

// The k-omega pipeline's c2c transforms down the spectrum's columns: the last
// pass stores (p, Im X) with p = s|X|^2 and adds p to the gram (kw.c's
// vsip_mcmagsq_f, vsip_smmul_f, vsip_madd_f).  Interleaved views: contiguous
// transforms (a column-major spectrum, as kw.c creates it) on the row
// mapping, adjacent transforms (a row-major one) as column tiles.
bool launch_fast_komega_power_f32(const Job &j, cudaStream_t st) {
    if (j.no_fast || j.prec != P_F32 || j.kind != K_C2C || !j.gram || !j.twp || j.lp || j.nbatch > 1 || j.tw_lo)
        return false;
    const CView &ci = j.cin, &co = j.cout;
    if (ci.cst != 2 || co.cst != 2 || (const float *)ci.im != (const float *)ci.re + 1 ||
        (const float *)co.im != (const float *)co.re + 1 || ((uintptr_t)ci.re % 8) || ((uintptr_t)co.re % 8))
        return false;
    if (j.nvec <= 0 || j.nvec > 0x7fffffffL) return false;
    if (ci.es == 1 && co.es == 1) {
        if (j.nvec > 1 && (labs(ci.vs) < j.N || labs(co.vs) < j.N)) return false;
        return launch_fast_rows<false, FX_POWER>(j, st);
    }
    if (j.nvec < 16 || labs(ci.vs) != 1 || labs(co.vs) != 1) return false;
    if (labs(ci.es) < j.nvec || labs(co.es) < j.nvec) return false;
    return launch_fast_cols<false, FX_POWER>(j, st);
}

// Specialised kernels: rows of unit element stride, or column tiles
// (adjacent transforms, any element stride), interleaved or split complex
// (both views alike), forward or inverse (conjugation folded into load and
// store), optional scale.
bool launch_fast_f32(const Job &j, cudaStream_t st) {
    if (j.no_fast) return false;
    if (j.kind != K_C2C) return launch_fast_real_f32(j, st);
    if (j.prec != P_F32) return false;
    if (j.lp || j.nbatch > 1 || j.tw_lo || j.gram || j.taper_n) return false;
    const CView &ci = j.cin, &co = j.cout;
    // split complex: separate real and imaginary arrays on both sides
    const bool split = ci.cst == 1 && co.cst == 1;
    if (!split) {
        // interleaved, 8-byte aligned
        if (ci.cst != 2 || co.cst != 2) return false;
        if ((const float *)ci.im != (const float *)ci.re + 1 || (const float *)co.im != (const float *)co.re + 1)
            return false;
        if (((uintptr_t)ci.re % 8) || ((uintptr_t)co.re % 8)) return false;
    }
    if (j.nvec <= 0 || j.nvec > 0x7fffffffL * 1L) return false;
    const bool rows = ci.es == 1 && co.es == 1;
    const bool cols = !rows && labs(ci.vs) == 1 && labs(co.vs) == 1 && j.nvec >= 16;
    if (rows) {
        // rows of an in-place call must not overlap each other (each CTA reads its
        // rows completely before it writes them)
        if (j.nvec > 1 && (labs(ci.vs) < j.N || labs(co.vs) < j.N)) return false;
        return split ? launch_fast_rows<true>(j, st) : launch_fast_rows<false>(j, st);
    }
    if (cols) {
        // columns of an in-place call: each CTA reads all elements of its
        // transforms before it writes them; transforms must not share elements
        if (labs(ci.es) < j.nvec || labs(co.es) < j.nvec) return false;
        return split ? launch_fast_cols<true>(j, st) : launch_fast_cols<false>(j, st);
    }
    return false;
}

}  // namespace jv
