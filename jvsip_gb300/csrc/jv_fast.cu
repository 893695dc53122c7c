// jv_fast.cu -- register-resident kernels (single precision, interleaved or
// split complex) for rows of unit element stride and any pitch, and for
// column tiles (adjacent transforms of any element stride).
//
// A transform of N = R1*R2*...*Rp points is held by T threads, E = N/T
// complex values each, in registers.  Pass 1 reads global memory directly
// (element t + T*b + r*N/R1: consecutive threads read consecutive elements),
// the middle passes exchange through shared memory, and the last pass writes
// global memory directly (element t + T*b + r*N/Rp, again coalesced): the
// self-sorting Stockham order needs no digit-reversal pass, so every point is
// read from and written to HBM exactly once.  Shared memory is indexed
// i + (i >> 4), which makes every pass's stores and loads conflict-free for
// 8-byte elements.  Several transforms share a CTA when N is small.
#include <stdio.h>
#include <stdlib.h>

#include <vector>

#include "jv_kernels.cuh"

namespace jv {

template <int... Rs> struct RList;
template <int R0, int... Rs> struct RList<R0, Rs...> {
    static constexpr int first = R0;
    typedef RList<Rs...> rest;
};
template <> struct RList<> {};

__device__ __forceinline__ int padx(int i) { return i + (i >> 4); }

struct FastArgs {
    const float2 *in;   // transform v starts at in + off_in + v*vs_in, element n at + n*es_in
    float2 *out;
    long es_in, es_out; // element strides (1 for rows; the row pitch for column tiles)
    // split complex views (SPLIT instances): real / imaginary arrays, element
    // n of row v at [off + v*vs + n]
    const float *in_re, *in_im;
    float *out_re, *out_im;
    // output twiddle of the first step of a long transform (TW instances):
    // element k of transform g times W^(g*k) = tw_lo[m & tw_mask] * tw_hi[m >> tw_sh]
    const float2 *tw_lo, *tw_hi;
    unsigned tw_mask, tw_sh;
    // one pass of a large-radix Stockham transform of Nt = 2^k points (SP
    // instances; the kernel's N is the pass radix R): transform j reads
    // element n at j + n*Nt/R (es_in), multiplies it by W_Nt^(n*m*Nt/(Ns*R))
    // with m = j mod Ns, and writes output k at (j - m)*R + m + k*Ns
    unsigned sp_ns, sp_lgns, sp_twstride, sp_mask;
    long off_in, vs_in, off_out, vs_out;
    long nvec;
    int inv;
    int has_scale;
    float scale;
    const float2 *twp; // per-pass twiddles: pass p at its offset, entry r*Ns + m = exp(-2 pi i r m/(Ns R))
};

// twiddle and DFT of the thread's E/R butterflies of a radix-R pass; the
// pass's twiddle table is laid out [r][m] so a warp's loads are contiguous
template <int N, int T, int R, int E, int Ns>
__device__ __forceinline__ void fast_bfly(float2 (&v)[E], int t, const float2 *__restrict__ tp) {
    constexpr int B = E / R;
#pragma unroll
    for (int b = 0; b < B; b++) {
        if constexpr (Ns > 1) {
            int j = t + T * b;
            int m = j % Ns;
#pragma unroll
            for (int r = 1; r < R; r++) v[b * R + r] = cmul(v[b * R + r], __ldg(&tp[r * Ns + m]));
        }
        Dft<float2, R>::run(&v[b * R]);
    }
}

template <int N, int T, int E, int R>
__device__ __forceinline__ void load_pass(float2 (&v)[E], const float2 *s, int t) {
    constexpr int B = E / R;
#pragma unroll
    for (int b = 0; b < B; b++)
#pragma unroll
        for (int r = 0; r < R; r++) v[b * R + r] = s[padx(t + T * b + r * (N / R))];
}

template <int N, int T, int E, int R>
__device__ __forceinline__ void store_pass(const float2 (&v)[E], float2 *s, int t, int Ns) {
    constexpr int B = E / R;
#pragma unroll
    for (int b = 0; b < B; b++) {
        int j = t + T * b;
        int m = j % Ns;
        int base = (j - m) * R + m;
#pragma unroll
        for (int r = 0; r < R; r++) s[padx(base + r * Ns)] = v[b * R + r];
    }
}

// Passes after the first.  On entry shared memory holds the previous pass's output.
template <int N, int T, int E, int NsIn, int Off, typename L, bool SPLIT, bool COLS, bool TW, bool SP> struct Passes;

template <int N, int T, int E, int NsIn, int Off, int R0, int... Rs, bool SPLIT, bool COLS, bool TW, bool SP>
struct Passes<N, T, E, NsIn, Off, RList<R0, Rs...>, SPLIT, COLS, TW, SP> {
    static __device__ __forceinline__ void run(float2 (&v)[E], float2 *s, int t, const FastArgs &a, long row,
                                               bool live) {
        __syncthreads();
        load_pass<N, T, E, R0>(v, s, t);
        fast_bfly<N, T, R0, E, NsIn>(v, t, a.twp + Off);
        if constexpr (sizeof...(Rs) == 0) {
            // last pass: j < N/R0 = NsIn, so element j + r*NsIn -- coalesced stores
            if (live) {
                // base of the transform's outputs and the stride of output k:
                // rows (1, 32-bit offsets), column tiles (es_out), Stockham
                // passes ((row - m)*R + m + k*Ns)
                long ob = a.off_out + row * a.vs_out;
                long ks = COLS ? a.es_out : 1L;
                if constexpr (SP) {
                    const unsigned m = (unsigned)row & (a.sp_ns - 1u);
                    ob = a.off_out + (long)((unsigned)row >> a.sp_lgns) * ((long)a.sp_ns * N) + m;
                    ks = a.sp_ns;
                }
                float2 *o = a.out + ob;
                float *orr = a.out_re + ob, *oi = a.out_im + ob;
                constexpr int B = E / R0;
#pragma unroll
                for (int b = 0; b < B; b++) {
                    int j = t + T * b;
#pragma unroll
                    for (int r = 0; r < R0; r++) {
                        float2 c = v[b * R0 + r];
                        if constexpr (TW)
                            c = cmul(c, tw_two_level(a.tw_lo, a.tw_hi, a.tw_mask, a.tw_sh,
                                                     (unsigned)row * (unsigned)(j + r * NsIn)));
                        if (a.inv) c.y = -c.y;
                        if (a.has_scale) c = cscale(c, a.scale);
                        const int k = j + r * NsIn;
                        if constexpr (COLS) {
                            const long e = (long)k * ks;
                            if constexpr (SPLIT) {
                                orr[e] = c.x;
                                oi[e] = c.y;
                            } else {
                                o[e] = c;
                            }
                        } else {
                            if constexpr (SPLIT) {
                                orr[k] = c.x;
                                oi[k] = c.y;
                            } else {
                                o[k] = c;
                            }
                        }
                    }
                }
            }
        } else {
            __syncthreads();
            store_pass<N, T, E, R0>(v, s, t, NsIn);
            Passes<N, T, E, NsIn * R0, Off + R0 * NsIn, RList<Rs...>, SPLIT, COLS, TW, SP>::run(v, s, t, a, row, live);
        }
    }
};

// Rows (COLS false): RPC transforms per CTA, T consecutive threads per
// transform.  Column tiles (COLS true): RPC adjacent transforms per CTA with
// consecutive threads on adjacent transforms, so every load and store of a
// warp covers RPC neighbouring elements of each row it touches; each
// transform's shared-memory row has an odd pitch so the RPC rows fall in
// different banks.  CTAs of up to 512 threads are held to 64 registers so
// that 1024 threads share an SM (ptxas otherwise took 86-115 registers, and one
// or two CTAs per SM left a CTA's loads without other CTAs' passes to overlap);
// the Stockham passes are not: measured on 2^24 points, their 256-point
// passes took 69-85 us at 128 registers (23 % of warps active) and 98-119 us
// at 64 (47 %).
template <int N, int T, int RPC, typename L, bool SPLIT, bool COLS, bool TW, bool SP>
__global__ void __launch_bounds__(T *RPC, (T * RPC <= 512 && !SP) ? 1024 / (T * RPC) : 1) k_fast(const FastArgs pa) {
    constexpr int E = N / T;
    constexpr int R1 = L::first;
    constexpr int NP = N + N / 16 + (COLS ? 1 : 0);  // padded row in shared memory
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const FastArgs a = pa;
    const int t = COLS ? (int)threadIdx.x / RPC : (int)threadIdx.x % T;
    const int rl = COLS ? (int)threadIdx.x % RPC : (int)threadIdx.x / T;
    const long row = (long)blockIdx.x * RPC + rl;
    float2 *s = reinterpret_cast<float2 *>(smem_raw) + rl * NP;
    // rows past the end (last CTA only) recompute the last row and store nothing,
    // so every thread reaches every barrier
    const bool live = row < a.nvec;
    const long rowc = live ? row : a.nvec - 1;
    float2 v[E];
    // base pointers of the transform; rows index them with 32-bit offsets
    const long ib = a.off_in + rowc * a.vs_in;
    const float2 *inb = a.in + ib;
    const float *inr = a.in_re + ib, *ini = a.in_im + ib;
    constexpr int B1 = E / R1;
#pragma unroll
    for (int b = 0; b < B1; b++)
#pragma unroll
        for (int r = 0; r < R1; r++) {
            const int n = t + T * b + r * (N / R1);
            float2 c;
            if constexpr (COLS) {
                const long e = (long)n * a.es_in;
                if constexpr (SPLIT) c = make_float2(inr[e], ini[e]);
                else c = inb[e];
            } else {
                if constexpr (SPLIT) c = make_float2(inr[n], ini[n]);
                else c = inb[n];
            }
            if (a.inv) c.y = -c.y;
            if constexpr (SP) {
                // Stockham input twiddle W_Nt^(n*m*stride), n = element index
                const unsigned m = (unsigned)rowc & (a.sp_ns - 1u);
                if (m) {
                    const unsigned n = (unsigned)(t + T * b + r * (N / R1));
                    c = cmul(c, tw_two_level(a.tw_lo, a.tw_hi, a.tw_mask, a.tw_sh,
                                             (n * m * a.sp_twstride) & a.sp_mask));
                }
            }
            v[b * R1 + r] = c;
        }
    fast_bfly<N, T, R1, E, 1>(v, t, nullptr);
    store_pass<N, T, E, R1>(v, s, t, 1);
    if constexpr (SP) {
        if (a.sp_ns == 1) {
            // the first Stockham pass writes each transform's outputs
            // contiguously (j*R + k): the passes after the first radix take
            // the row mapping (T consecutive threads on one transform), so
            // the last one's stores are coalesced
            const int t2 = (int)threadIdx.x % T, rl2 = (int)threadIdx.x / T;
            const long row2 = (long)blockIdx.x * RPC + rl2;
            const bool live2 = row2 < a.nvec;
            Passes<N, T, E, R1, R1, typename L::rest, SPLIT, COLS, TW, SP>::run(
                v, reinterpret_cast<float2 *>(smem_raw) + rl2 * NP, t2, a, live2 ? row2 : a.nvec - 1, live2);
            return;
        }
    }
    Passes<N, T, E, R1, R1, typename L::rest, SPLIT, COLS, TW, SP>::run(v, s, t, a, rowc, live);
}

template <int N, int T, int RPC, typename L, bool SPLIT, bool COLS, bool TW = false, bool SP = false>
static bool launch_fast_n(const Job &j, cudaStream_t st) {
    FastArgs a;
    a.sp_ns = j.sp_ns;
    a.sp_lgns = j.sp_lgns;
    a.sp_twstride = j.sp_twstride;
    a.sp_mask = j.sp_mask;
    a.tw_lo = (const float2 *)j.tw_lo;
    a.tw_hi = (const float2 *)j.tw_hi;
    a.tw_mask = j.tw_mask;
    a.tw_sh = j.tw_sh;
    a.in = (const float2 *)j.cin.re;
    a.out = (float2 *)j.cout.re;
    a.es_in = j.cin.es;
    a.es_out = j.cout.es;
    a.in_re = (const float *)j.cin.re;
    a.in_im = (const float *)j.cin.im;
    a.out_re = (float *)j.cout.re;
    a.out_im = (float *)j.cout.im;
    a.off_in = j.cin.off;
    a.vs_in = j.cin.vs;
    a.off_out = j.cout.off;
    a.vs_out = j.cout.vs;
    a.nvec = j.nvec;
    a.inv = j.inv;
    a.has_scale = j.has_scale;
    a.scale = (float)j.scale;
    a.twp = (const float2 *)j.twp;
    if (!a.twp) return false;
    constexpr int NP = N + N / 16 + (COLS ? 1 : 0);
    size_t smem = (size_t)RPC * NP * sizeof(float2);
    static bool attr = false;
    if (!attr) {
        if (smem > 48 * 1024 &&
            !cuda_ok(cudaFuncSetAttribute(k_fast<N, T, RPC, L, SPLIT, COLS, TW, SP>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                     "cudaFuncSetAttribute"))
            return false;
        attr = true;
    }
    long grid = (j.nvec + RPC - 1) / RPC;
    k_fast<N, T, RPC, L, SPLIT, COLS, TW, SP><<<(unsigned)grid, T * RPC, smem, st>>>(a);
    count_launch();
    return cuda_ok(cudaGetLastError(), "k_fast launch");
}

// Radix list of the specialised kernel for length N (empty: none).
std::vector<int> fast_radices(long N) {
    switch (N) {
        case 64: return {16, 4};
        case 128: return {16, 8};
        case 256: return {16, 16};
        case 512: return {16, 16, 2};
        case 1000: return {10, 10, 10};
        case 1024: return {16, 16, 4};
        case 2048: return {16, 16, 8};
        case 4096: return {16, 16, 16};
        case 8192: return {16, 16, 16, 2};
        default: return {};
    }
}

// Rows: T threads per transform, RPC transforms per CTA.
template <bool SPLIT>
static bool launch_fast_rows(const Job &j, cudaStream_t st) {
    switch (j.N) {
        case 64: return launch_fast_n<64, 4, 64, RList<16, 4>, SPLIT, false>(j, st);
        case 128: return launch_fast_n<128, 8, 32, RList<16, 8>, SPLIT, false>(j, st);
        case 256: return launch_fast_n<256, 16, 16, RList<16, 16>, SPLIT, false>(j, st);
        case 512: return launch_fast_n<512, 32, 8, RList<16, 16, 2>, SPLIT, false>(j, st);
        case 1000: return launch_fast_n<1000, 100, 4, RList<10, 10, 10>, SPLIT, false>(j, st);
        case 1024: return launch_fast_n<1024, 64, 4, RList<16, 16, 4>, SPLIT, false>(j, st);
        case 2048: return launch_fast_n<2048, 128, 2, RList<16, 16, 8>, SPLIT, false>(j, st);
        case 4096: return launch_fast_n<4096, 256, 1, RList<16, 16, 16>, SPLIT, false>(j, st);
        case 8192: return launch_fast_n<8192, 512, 1, RList<16, 16, 16, 2>, SPLIT, false>(j, st);
        default: return false;
    }
}

// Column tiles: V adjacent transforms per CTA (V * 8 bytes of each row per
// warp access), shared memory about 70 KB per CTA for the long ones.
// Measured on 2^24 points (GB/s, against the shared-memory kernel's column
// tiles): 64 points 5624 (3664), 256: 5377 (4088), 512: 3478 (2220), 1024:
// 2927 (2472), 2048: 2059 (2000), 1000 x 4096: 2054 (1785).
template <bool SPLIT>
static bool launch_fast_cols(const Job &j, cudaStream_t st) {
    switch (j.N) {
        case 64: return launch_fast_n<64, 4, 64, RList<16, 4>, SPLIT, true>(j, st);
        case 128: return launch_fast_n<128, 8, 32, RList<16, 8>, SPLIT, true>(j, st);
        case 256: return launch_fast_n<256, 16, 16, RList<16, 16>, SPLIT, true>(j, st);
        case 512: return launch_fast_n<512, 32, 16, RList<16, 16, 2>, SPLIT, true>(j, st);
        case 1000: return launch_fast_n<1000, 100, 8, RList<10, 10, 10>, SPLIT, true>(j, st);
        case 1024: return launch_fast_n<1024, 64, 8, RList<16, 16, 4>, SPLIT, true>(j, st);
        case 2048: return launch_fast_n<2048, 128, 4, RList<16, 16, 8>, SPLIT, true>(j, st);
        // 4096 points: two columns per CTA measured slower (1689 GB/s) than the
        // shared-memory kernel's four (1841 GB/s); it keeps those
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

bool launch_fast_step_f32(const Job &j, cudaStream_t st) {
    if (j.kind != K_C2C || j.prec != P_F32 || j.nbatch != 1 || !fast_step_len(j.N) || !j.twp) return false;
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

// Specialised kernels: rows of unit element stride, or column tiles
// (adjacent transforms, any element stride), interleaved or split complex
// (both views alike), forward or inverse (conjugation folded into load and
// store), optional scale.
bool launch_fast_f32(const Job &j, cudaStream_t st) {
    if (j.no_fast) return false;
    if (j.kind != K_C2C || j.prec != P_F32) return false;
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
