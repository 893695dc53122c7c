// jv_fast_dd.cu -- the FP64 form of the row kernel: complex-double rows
// transformed in double-float arithmetic (jv_dd.cuh) on the FP32 pipes.
//
// GB300's FP64 rate is a small fraction of its FP32 rate, and the plain
// double-precision kernels are bound by it (about 60 FP64 operations per
// point for 4096-point rows).  Here each row is read as doubles, shifted by a
// power of two so that its largest element lies in [1, 2) (the shift is the
// row's largest exponent, found with a shared-memory max over the row's
// threads), split into hi + lo floats on the integer pipe, transformed with
// self-sorting radix-8/4/2 Stockham passes held in registers (E = 8 points per
// thread, exchanges through padded shared memory, per-pass [r][m] twiddle
// tables in double-float), and written back as hi + lo shifted back.  The
// result carries about 48 significant bits (unit roundoff 2^-48) instead of
// 53: an opt-in form (JVSIP_FORM_DF64) for 64-point to 8192-point rows.
#include <stdio.h>

#include <vector>

#include "jv_dd.cuh"
#include "jv_kernels.cuh"

namespace jv {

template <int... Rs> struct DRList;
template <int R0, int... Rs> struct DRList<R0, Rs...> {
    static constexpr int first = R0;
    typedef DRList<Rs...> rest;
};
template <> struct DRList<> {};

__device__ __forceinline__ int padd(int i) { return i + (i >> 4); }

struct FastDDArgs {
    const double2 *in;  // row v starts at in + off_in + v*vs_in (unit element stride)
    double2 *out;
    long off_in, vs_in, off_out, vs_out;
    long nvec;
    int inv;
    int has_scale;
    dd scale;
    const cdd *tw;      // per-pass twiddles: pass p at its offset, entry r*Ns + m = exp(-2 pi i r m/(Ns R))
};

template <int T, int R, int E, int Ns>
__device__ __forceinline__ void dd_bfly(cdd (&v)[E], int t, const cdd *__restrict__ tp) {
    constexpr int B = E / R;
#pragma unroll
    for (int b = 0; b < B; b++) {
        if constexpr (Ns > 1) {
            const int j = t + T * b;
            const int m = j % Ns;
#pragma unroll
            for (int r = 1; r < R; r++) v[b * R + r] = cmul(v[b * R + r], tp[r * Ns + m]);
        }
        Dft<cdd, R>::run(&v[b * R]);
    }
}

template <int N, int T, int E, int R>
__device__ __forceinline__ void dd_load_pass(cdd (&v)[E], const cdd *s, int t) {
    constexpr int B = E / R;
#pragma unroll
    for (int b = 0; b < B; b++)
#pragma unroll
        for (int r = 0; r < R; r++) v[b * R + r] = s[padd(t + T * b + r * (N / R))];
}

template <int N, int T, int E, int R>
__device__ __forceinline__ void dd_store_pass(const cdd (&v)[E], cdd *s, int t, int Ns) {
    constexpr int B = E / R;
#pragma unroll
    for (int b = 0; b < B; b++) {
        const int j = t + T * b;
        const int m = j % Ns;
        const int base = (j - m) * R + m;
#pragma unroll
        for (int r = 0; r < R; r++) s[padd(base + r * Ns)] = v[b * R + r];
    }
}

template <int N, int T, int E, int NsIn, int Off, typename L> struct DDPasses;

template <int N, int T, int E, int NsIn, int Off, int R0, int... Rs>
struct DDPasses<N, T, E, NsIn, Off, DRList<R0, Rs...>> {
    static __device__ __forceinline__ void run(cdd (&v)[E], cdd *s, int t, const FastDDArgs &a, long row, bool live,
                                               int sh) {
        __syncthreads();
        dd_load_pass<N, T, E, R0>(v, s, t);
        dd_bfly<T, R0, E, NsIn>(v, t, a.tw + Off);
        if constexpr (sizeof...(Rs) == 0) {
            // last pass: element j + r*NsIn, coalesced stores of doubles
            if (live) {
                double2 *o = a.out + a.off_out + row * a.vs_out;
                constexpr int B = E / R0;
#pragma unroll
                for (int b = 0; b < B; b++) {
                    const int j = t + T * b;
#pragma unroll
                    for (int r = 0; r < R0; r++) {
                        cdd c = v[b * R0 + r];
                        if (a.inv) c.y = -c.y;
                        if (a.has_scale) {
                            c.x *= a.scale;
                            c.y *= a.scale;
                        }
                        o[j + r * NsIn] = make_double2(dd_to_double(c.x, sh), dd_to_double(c.y, sh));
                    }
                }
            }
        } else {
            __syncthreads();
            dd_store_pass<N, T, E, R0>(v, s, t, NsIn);
            DDPasses<N, T, E, NsIn * R0, Off + R0 * NsIn, DRList<Rs...>>::run(v, s, t, a, row, live, sh);
        }
    }
};

template <int N, int T, int RPC, typename L>
__global__ void __launch_bounds__(T *RPC) k_fast_dd(const FastDDArgs pa) {
    constexpr int E = N / T;
    constexpr int R1 = L::first;
    constexpr int NP = N + N / 16;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int rowexp[RPC];
    const FastDDArgs a = pa;
    const int t = threadIdx.x % T;
    const int rl = threadIdx.x / T;
    const long row = (long)blockIdx.x * RPC + rl;
    cdd *s = reinterpret_cast<cdd *>(smem_raw) + rl * NP;
    const bool live = row < a.nvec;
    const long rowc = live ? row : a.nvec - 1;
    if (t == 0) rowexp[rl] = 0;
    // the row's doubles, and the largest biased exponent among them
    double2 x[E];
    const double2 *in = a.in + a.off_in + rowc * a.vs_in;
    constexpr int B1 = E / R1;
    int emax = 0;
#pragma unroll
    for (int b = 0; b < B1; b++)
#pragma unroll
        for (int r = 0; r < R1; r++) {
            const double2 c = in[t + T * b + r * (N / R1)];
            x[b * R1 + r] = c;
            emax = max(emax, max(dd_exp_of(c.x), dd_exp_of(c.y)));
        }
    __syncthreads();
    atomicMax(&rowexp[rl], emax);
    __syncthreads();
    // shift so the largest element lies in [1, 2); an all-zero row keeps 0
    const int sh = rowexp[rl] == 0 ? 0 : rowexp[rl] - 1023;
    cdd v[E];
#pragma unroll
    for (int i = 0; i < E; i++) {
        v[i].x = dd_from_double(x[i].x, sh);
        v[i].y = dd_from_double(x[i].y, sh);
        if (a.inv) v[i].y = -v[i].y;
    }
    dd_bfly<T, R1, E, 1>(v, t, nullptr);
    dd_store_pass<N, T, E, R1>(v, s, t, 1);
    DDPasses<N, T, E, R1, R1, typename L::rest>::run(v, s, t, a, rowc, live, sh);
}

template <int N, int T, int RPC, typename L>
static bool launch_dd_n(const Job &j, cudaStream_t st) {
    FastDDArgs a;
    a.in = (const double2 *)j.cin.re;
    a.out = (double2 *)j.cout.re;
    a.off_in = j.cin.off;
    a.vs_in = j.cin.vs;
    a.off_out = j.cout.off;
    a.vs_out = j.cout.vs;
    a.nvec = j.nvec;
    a.inv = j.inv;
    a.has_scale = j.has_scale;
    a.scale = dd(j.scale);
    a.tw = (const cdd *)j.twdd;
    if (!a.tw) return false;
    constexpr int NP = N + N / 16;
    const size_t smem = (size_t)RPC * NP * sizeof(cdd);
    static std::atomic<bool> attr{false};  // set once; concurrent first calls both set it
    if (!attr) {
        if (smem > 48 * 1024 &&
            !cuda_ok(cudaFuncSetAttribute(k_fast_dd<N, T, RPC, L>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)smem),
                     "cudaFuncSetAttribute"))
            return false;
        attr = true;
    }
    const long grid = (j.nvec + RPC - 1) / RPC;
    k_fast_dd<N, T, RPC, L><<<(unsigned)grid, T * RPC, smem, st>>>(a);
    count_launch();
    return cuda_ok(cudaGetLastError(), "k_fast_dd launch");
}

// Radix list of the FP64 form for length N (empty: the form does not take N).
std::vector<int> dd_radices(long N) {
    switch (N) {
        case 64: return {8, 8};
        case 128: return {8, 8, 2};
        case 256: return {8, 8, 4};
        case 512: return {8, 8, 8};
        case 1024: return {8, 8, 8, 2};
        case 2048: return {8, 8, 8, 4};
        case 4096: return {8, 8, 8, 8};
        case 8192: return {8, 8, 8, 8, 2};
        default: return {};
    }
}

// The FP64 form: complex-double rows of unit element stride, interleaved,
// 16-byte aligned, rows not overlapping; false when the call does not qualify.
bool launch_fast_dd(const Job &j, cudaStream_t st) {
    if (j.kind != K_C2C || j.prec != P_F64) return false;
    const CView &ci = j.cin, &co = j.cout;
    if (ci.cst != 2 || co.cst != 2 || ci.es != 1 || co.es != 1) return false;
    if ((const double *)ci.im != (const double *)ci.re + 1 || (const double *)co.im != (const double *)co.re + 1)
        return false;
    if (((uintptr_t)ci.re % 16) || ((uintptr_t)co.re % 16)) return false;
    if (j.nvec <= 0 || j.nvec > 0x7fffffffL) return false;
    if (j.nvec > 1 && (labs(ci.vs) < j.N || labs(co.vs) < j.N)) return false;
    switch (j.N) {
        case 64: return launch_dd_n<64, 8, 64, DRList<8, 8>>(j, st);
        case 128: return launch_dd_n<128, 16, 32, DRList<8, 8, 2>>(j, st);
        case 256: return launch_dd_n<256, 32, 16, DRList<8, 8, 4>>(j, st);
        case 512: return launch_dd_n<512, 64, 8, DRList<8, 8, 8>>(j, st);
        case 1024: return launch_dd_n<1024, 128, 4, DRList<8, 8, 8, 2>>(j, st);
        case 2048: return launch_dd_n<2048, 256, 2, DRList<8, 8, 8, 4>>(j, st);
        case 4096: return launch_dd_n<4096, 512, 1, DRList<8, 8, 8, 8>>(j, st);
        case 8192: return launch_dd_n<8192, 1024, 1, DRList<8, 8, 8, 8, 2>>(j, st);
        default: return false;
    }
}

}  // namespace jv
