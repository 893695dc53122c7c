// jv_fast.cuh -- the register-resident kernel (single precision): its
// template, shared by the row / column-tile / long-step / Stockham-pass
// launchers (jv_fast.cu) and the real-row launchers (jv_fast_real.cu).
//
// A transform of N = R1*R2*...*Rp points is held by T threads, E = N/T
// complex values each, in registers.  Pass 1 reads global memory directly
// (element t + T*b + r*N/R1: consecutive threads read consecutive elements),
// the middle passes exchange through shared memory, and the last pass writes
// global memory directly (element t + T*b + r*N/Rp, again coalesced): the
// self-sorting Stockham order needs no digit-reversal pass, so every point is
// read from and written to HBM exactly once.  Shared memory is indexed
// i + (i >> 4) (power-of-two passes conflict-free for 8-byte elements) with
// row pitches chosen per tile shape (fast_pitch).  Several transforms share a
// CTA when N is small.
//
// Real rows (RM = 1: R2C, RM = 2: C2R) hold the half-length complex
// transform: the R2C first pass reads x_{2n}, x_{2n+1} as one complex element
// and its last pass leaves Z_k in shared memory for the Hermitian split
// (X_k from Z_k and Z_{N-k}, c_VSIP_src/VI_rcfftmop_f_def.h:79-118); the C2R
// first pass forms Y_n from X_n and X_{N-n} (VI_crfftmop_f_def.h:58-110) and
// its last pass writes y_n as x_{2n}, x_{2n+1} (:121-124).
#pragma once

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

// Shared-memory index padding: one element per 16, or per 32 for the
// 1000-point (10 x 10 x 10) and 768-point (12 x 8 x 8) transforms, whose
// radix-10 and radix-12 strides collide less that way (2.6 and 1.75 wavefronts
// per 64-bit access on average become 1.7 and 1.5).
template <int N> constexpr int fast_pad_shift() { return (N == 1000 || N == 768) ? 5 : 4; }
template <int N> __device__ __forceinline__ int padx(int i) { return i + (i >> fast_pad_shift<N>()); }

// Padded pitch of a transform's row in shared memory.  Column tiles put
// 16/RPC transforms' elements t, t+1, ... and RPC columns in one half-warp's
// 64-bit access, so the RPC rows start 16/RPC elements apart modulo 16 (RPC <=
// 8) or one element apart: every access then hits 32 distinct banks (an odd
// pitch alone gave 2 wavefronts per access for 1024-point tiles of 8 columns
// and 4 for 2048-point tiles of 4).
template <int N, int RPC, bool COLS> constexpr int fast_pitch() {
    constexpr int base = N + (N >> fast_pad_shift<N>());
    if (!COLS) return base;
    if (RPC > 8) return base + 1;
    return base + (16 / RPC - base % 16 + 16) % 16;
}

struct FastArgs {
    const float2 *in;   // transform v starts at in + off_in + v*vs_in, element n at + n*es_in
    float2 *out;
    long es_in, es_out; // element strides (1 for rows; the row pitch for column tiles)
    // split complex views (SPLIT instances): real / imaginary arrays, element
    // n of row v at [off + v*vs + n]
    const float *in_re, *in_im;
    float *out_re, *out_im;
    // output twiddle of the first step of a long transform (TW instances):
    // element k of transform row of group y times W^(g*k), g = row*tw_ts +
    // y*tw_ys, = tw_lo[m & tw_mask] * tw_hi[m >> tw_sh]
    const float2 *tw_lo, *tw_hi;
    unsigned tw_mask, tw_sh, tw_ts, tw_ys;
    // column tiles (COLS instances): groups of nvec transforms along the
    // grid's y, bvs_in / bvs_out complex elements apart
    long bvs_in, bvs_out;
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
    const float2 *thalf; // real rows: exp(-+ i pi k/N), k <= N (R2C: minus, C2R: plus)
    // k-omega fusions (FXK): FX_TAPER -- real pair n of row v times (ts[2n],
    // ts[2n+1]) then arr[v], each product rounded, written back to the row
    // through wb; FX_POWER -- output k of transform v stored as (p, Im X) with
    // p = g_scale |X|^2, and p added to gram[v*g_vs + k*g_es]
    const float *tp_n, *tp_t;
    long tp_n_st, tp_t_st;
    float2 *wb;
    float *gram;
    long g_es, g_vs;
    float g_scale;
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
        for (int r = 0; r < R; r++) v[b * R + r] = s[padx<N>(t + T * b + r * (N / R))];
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
        for (int r = 0; r < R; r++) s[padx<N>(base + r * Ns)] = v[b * R + r];
    }
}

// R2C rows: the last pass's Z_k (k = j + r*Ns) to shared memory in natural
// order, then X_k = ((Z_k + conj Z_{N-k}) - i w_k (Z_k - conj Z_{N-k}))/2 for
// k = 0..N (Z_N = Z_0; w_k = exp(-i pi k/N)), the scale applied to Z first as
// the reference does (VI_rcfftmop_f_def.h:79-118).  The thread of pair
// (k, N-k), k = t + T*i <= N/2, reads Z_k and Z_{N-k} once and writes X_k and
// X_{N-k} (X_N for k = 0): ascending and descending coalesced stores when the
// output rows are contiguous; output element k at k*es_out (column-major
// spectra: adjacent rows' X_k are adjacent).
template <int N, int T, int E, int R>
__device__ __forceinline__ void r2c_finish(const float2 (&v)[E], float2 *s, int t, const FastArgs &a, long row,
                                           bool live, int Ns) {
    constexpr int B = E / R;
    __syncthreads();  // every thread has read the previous pass's output
#pragma unroll
    for (int b = 0; b < B; b++) {
        const int j = t + T * b;
#pragma unroll
        for (int r = 0; r < R; r++) s[padx<N>(j + r * Ns)] = v[b * R + r];
    }
    __syncthreads();
    if (!live) return;
    float2 *o = a.out + a.off_out + row * a.vs_out;
    constexpr int NPAIR = N / 2 + 1;
#pragma unroll
    for (int i = 0; i < (NPAIR + T - 1) / T; i++) {
        const int k = t + T * i;
        if (k >= NPAIR) break;
        const int nk = (k == 0) ? N : N - k;
        float2 zk = s[padx<N>(k)], zn = s[padx<N>(k == 0 ? 0 : N - k)];
        if (a.has_scale) {
            zk = cscale(zk, a.scale);
            zn = cscale(zn, a.scale);
        }
        const float2 w = __ldg(&a.thalf[k]), w2 = __ldg(&a.thalf[nk]);
        o[k * a.es_out] = make_float2(0.5f * (zn.x + zk.x + w.x * (zn.y + zk.y) + w.y * (zk.x - zn.x)),
                                      0.5f * (zk.y - zn.y + w.x * (zn.x - zk.x) + w.y * (zn.y + zk.y)));
        if (nk != k)
            o[nk * a.es_out] = make_float2(0.5f * (zk.x + zn.x + w2.x * (zk.y + zn.y) + w2.y * (zn.x - zk.x)),
                                           0.5f * (zn.y - zk.y + w2.x * (zk.x - zn.x) + w2.y * (zk.y + zn.y)));
    }
}

// Passes after the first.  On entry shared memory holds the previous pass's output.
template <int N, int T, int E, int NsIn, int Off, typename L, bool SPLIT, bool COLS, bool TW, bool SP, int RM,
          int FXK>
struct Passes;

template <int N, int T, int E, int NsIn, int Off, int R0, int... Rs, bool SPLIT, bool COLS, bool TW, bool SP, int RM,
          int FXK>
struct Passes<N, T, E, NsIn, Off, RList<R0, Rs...>, SPLIT, COLS, TW, SP, RM, FXK> {
    static __device__ __forceinline__ void run(float2 (&v)[E], float2 *s, int t, const FastArgs &a, long row,
                                               bool live) {
        __syncthreads();
        load_pass<N, T, E, R0>(v, s, t);
        fast_bfly<N, T, R0, E, NsIn>(v, t, a.twp + Off);
        if constexpr (sizeof...(Rs) == 0 && RM == 1) {
            r2c_finish<N, T, E, R0>(v, s, t, a, row, live, NsIn);
        } else if constexpr (sizeof...(Rs) == 0) {
            // last pass: j < N/R0 = NsIn, so element j + r*NsIn -- coalesced stores
            if (live) {
                // base of the transform's outputs and the stride of output k:
                // rows (1, 32-bit offsets), column tiles (es_out), Stockham
                // passes ((row - m)*R + m + k*Ns)
                long ob = a.off_out + row * a.vs_out;
                if constexpr (COLS) ob += (long)blockIdx.y * a.bvs_out;
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
                                                     ((unsigned)row * a.tw_ts + blockIdx.y * a.tw_ys) *
                                                         (unsigned)(j + r * NsIn)));
                        if (a.inv) c.y = -c.y;
                        if (a.has_scale) c = cscale(c, a.scale);
                        const int k = j + r * NsIn;
                        if constexpr ((FXK & FX_POWER) != 0) {
                            // p = |X|^2 (vsip_mcmagsq_f), p *= s (vsip_smmul_f),
                            // gram = p + gram (vsip_madd_f), rounded in that order
                            float p = add_rn(mul_rn(c.x, c.x), mul_rn(c.y, c.y));
                            p = mul_rn(a.g_scale, p);
                            float *g = a.gram + row * a.g_vs + (long)k * a.g_es;
                            *g = add_rn(p, *g);
                            c.x = p;
                        }
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
            Passes<N, T, E, NsIn * R0, Off + R0 * NsIn, RList<Rs...>, SPLIT, COLS, TW, SP, RM, FXK>::run(v, s, t, a,
                                                                                                      row, live);
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
template <int N, int T, int RPC, bool SP>
constexpr int fast_min_blocks() {
    // 1024 threads per SM (64 registers); 24 points per thread (768-point
    // rows) need more registers: 896 threads per SM (72 registers)
    return (T * RPC <= 512 && !SP) ? ((N / T > 16) ? 896 : 1024) / (T * RPC) : 1;
}

template <int N, int T, int RPC, typename L, bool SPLIT, bool COLS, bool TW, bool SP, int RM, int FXK>
__global__ void __launch_bounds__(T *RPC, fast_min_blocks<N, T, RPC, SP>()) k_fast(const FastArgs pa) {
    constexpr int E = N / T;
    constexpr int R1 = L::first;
    constexpr int NP = fast_pitch<N, RPC, COLS>();  // padded row in shared memory
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
    const long ib = a.off_in + rowc * a.vs_in + (COLS ? (long)blockIdx.y * a.bvs_in : 0L);
    const float2 *inb = a.in + ib;
    const float *inr = a.in_re + ib, *ini = a.in_im + ib;
    constexpr int B1 = E / R1;
#pragma unroll
    for (int b = 0; b < B1; b++)
#pragma unroll
        for (int r = 0; r < R1; r++) {
            const int n = t + T * b + r * (N / R1);
            float2 c;
            if constexpr (RM == 2) {
                // C2R: Y_n = X_n + conj X_{N-n} + i w_n (X_n - conj X_{N-n}) with
                // w_n = exp(+i pi n/N) (X_N at n = 0), conjugated below for the
                // forward passes; X_{N-n} is another thread's X_n (L1)
                const float2 f = __ldg(&inb[n]), bb = __ldg(&inb[N - n]);
                const float2 w = __ldg(&a.thalf[n]);
                c = make_float2(f.x + bb.x + w.y * (bb.x - f.x) - w.x * (f.y + bb.y),
                                f.y - bb.y - w.y * (f.y + bb.y) + w.x * (f.x - bb.x));
            } else if constexpr (COLS) {
                const long e = (long)n * a.es_in;
                if constexpr (SPLIT) c = make_float2(inr[e], ini[e]);
                else c = inb[e];
            } else {
                if constexpr (SPLIT) c = make_float2(inr[n], ini[n]);
                else c = inb[n];
            }
            if constexpr (RM == 1 && (FXK & FX_TAPER) != 0) {
                // kw.c: data = ts * data (VSIP_ROW), then data = arr * data (VSIP_COL)
                const float wt = a.tp_t[rowc * a.tp_t_st];
                c.x = mul_rn(mul_rn(a.tp_n[2L * n * a.tp_n_st], c.x), wt);
                c.y = mul_rn(mul_rn(a.tp_n[(2L * n + 1) * a.tp_n_st], c.y), wt);
                if (live) a.wb[ib + n] = c;
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
            Passes<N, T, E, R1, R1, typename L::rest, SPLIT, COLS, TW, SP, RM, FXK>::run(
                v, reinterpret_cast<float2 *>(smem_raw) + rl2 * NP, t2, a, live2 ? row2 : a.nvec - 1, live2);
            return;
        }
    }
    Passes<N, T, E, R1, R1, typename L::rest, SPLIT, COLS, TW, SP, RM, FXK>::run(v, s, t, a, rowc, live);
}

template <int N, int T, int RPC, typename L, bool SPLIT, bool COLS, bool TW = false, bool SP = false, int RM = 0,
          int FXK = 0>
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
    a.tw_ts = j.tw_ts;
    a.tw_ys = j.tw_ys;
    a.bvs_in = j.bvs_in;
    a.bvs_out = j.bvs_out;
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
    a.thalf = (const float2 *)j.thalf;
    if constexpr (RM == 1) {
        // R2C: the real input row read as N complex pairs (offset and pitch even)
        a.in = (const float2 *)j.rin.a;
        a.off_in = j.rin.off / 2;
        a.vs_in = j.rin.vs / 2;
        a.es_in = 1;
        a.inv = 0;
    } else if constexpr (RM == 2) {
        // C2R: the real output row written as N complex pairs, conjugated back
        a.out = (float2 *)j.rout.a;
        a.off_out = j.rout.off / 2;
        a.vs_out = j.rout.vs / 2;
        a.es_out = 1;
        a.inv = 1;
    }
    a.tp_n = (const float *)j.taper_n;
    a.tp_t = (const float *)j.taper_t;
    a.tp_n_st = j.taper_n_st;
    a.tp_t_st = j.taper_t_st;
    a.wb = const_cast<float2 *>(a.in);
    a.gram = (float *)j.gram;
    a.g_es = j.gram_es;
    a.g_vs = j.gram_vs;
    a.g_scale = (float)j.gram_scale;
    if (!a.twp || (RM != 0 && !a.thalf)) return false;
    if ((FXK & FX_TAPER) != 0 && (!a.tp_n || !a.tp_t || !j.taper_back)) return false;
    if ((FXK & FX_POWER) != 0 && !a.gram) return false;
    constexpr int NP = fast_pitch<N, RPC, COLS>();
    size_t smem = (size_t)RPC * NP * sizeof(float2);
    static std::atomic<bool> attr{false};  // set once; concurrent first calls both set it
    if (!attr) {
        if (smem > 48 * 1024 &&
            !cuda_ok(cudaFuncSetAttribute(k_fast<N, T, RPC, L, SPLIT, COLS, TW, SP, RM, FXK>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                     "cudaFuncSetAttribute"))
            return false;
        attr = true;
    }
    long grid = (j.nvec + RPC - 1) / RPC;
    // groups along y: column-tile steps of a long transform (at most 65535)
    const unsigned gy = COLS ? (unsigned)j.nbatch : 1u;
    if (gy < 1 || gy > 65535u) return false;
    k_fast<N, T, RPC, L, SPLIT, COLS, TW, SP, RM, FXK><<<dim3((unsigned)grid, gy), T * RPC, smem, st>>>(a);
    count_launch();
    return cuda_ok(cudaGetLastError(), "k_fast launch");
}

}  // namespace jv
