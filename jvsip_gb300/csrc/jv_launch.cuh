// jv_launch.cuh -- host-side launchers of the general kernels, written once
// for both precisions and instantiated in jv_kern_f32.cu / jv_kern_f64.cu.
#pragma once

#include <stdio.h>

#include <algorithm>

#include "jv_kernels.cuh"

namespace jv {

// Two register budgets of the shared-memory kernel per precision: EMAX complex
// values a thread keeps per radix pass and the block size bound MAXT.  The
// small variant serves transforms of up to EMAX*MAXT/2 elements per CTA
// without spilling; the large one reaches EMAX*MAXT elements.
template <typename T> struct KCfg;
template <> struct KCfg<float> {
    static constexpr int EMAX_S = 8, MAXT_S = 1024, EMAX_L = 16, MAXT_L = 1024;
};
template <> struct KCfg<double> {
    static constexpr int EMAX_S = 8, MAXT_S = 512, EMAX_L = 16, MAXT_L = 512;
};

template <typename T>
static CAcc<T> cacc(const CView &v) {
    CAcc<T> a;
    a.re = (const T *)v.re;
    a.im = (const T *)v.im;
    a.cst = v.cst;
    a.off = v.off;
    a.es = v.es;
    a.vs = v.vs;
    a.vec = (v.cst == 2) && ((const T *)v.im == (const T *)v.re + 1) &&
            (((uintptr_t)v.re % (2 * sizeof(T))) == 0);
    return a;
}
template <typename T>
static CSto<T> csto(const CView &v) {
    CSto<T> a;
    a.re = (T *)v.re;
    a.im = (T *)v.im;
    a.cst = v.cst;
    a.off = v.off;
    a.es = v.es;
    a.vs = v.vs;
    a.vec = (v.cst == 2) && ((T *)v.im == (T *)v.re + 1) && (((uintptr_t)v.re % (2 * sizeof(T))) == 0);
    return a;
}
template <typename T>
static RAcc<T> racc(const RView &v) {
    RAcc<T> a;
    a.a = (const T *)v.a;
    a.rst = v.rst;
    a.off = v.off;
    a.es = v.es;
    a.vs = v.vs;
    return a;
}
template <typename T>
static RSto<T> rsto(const RView &v) {
    RSto<T> a;
    a.a = (T *)v.a;
    a.rst = v.rst;
    a.off = v.off;
    a.es = v.es;
    a.vs = v.vs;
    return a;
}

static inline long labs_(long x) { return x < 0 ? -x : x; }

// shared memory kept out of the dynamic allocation for the kernel's own
// static variables (the TMA barrier)
constexpr size_t kStaticSmem = 1024;

// cuTensorMapEncodeTiled from the driver, looked up once
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
inline EncodeTiledFn encode_tiled() {
    // initialised once, thread-safely, on the first call
    static const EncodeTiledFn fn = []() -> EncodeTiledFn {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            return (EncodeTiledFn)f;
        cudaGetLastError();
        return nullptr;
    }();
    return fn;
}

// TMA staging of the c2c column tiles (transforms adjacent in memory, vpb of
// them per tile): the view as a 2-D tensor of scalars, x = 2*transform (+ re /
// im), y = element, boxes of 2*vpb x rows.  Requires a 16-byte aligned start,
// a row pitch of a multiple of 16 bytes, an even vpb (so every tile's x is a
// multiple of 16 bytes) and boxes that fit the tile's shared memory; returns
// false (plain loads) otherwise.
template <typename T>
static bool tma_columns(SmemArgs<T> &a, const Job &j, long vpb, long ld) {
    a.tma = 0;
    const CView &v = j.cin;
    // automatic: long transforms only (measured on GB300: columns of 1536 and
    // 4096 points 5-9 % faster with TMA boxes, 1000 points and shorter 10-30 %
    // slower than the first pass's own coalesced loads)
    const bool want = j.tma_columns == 1 || (j.tma_columns < 0 && j.N >= 1536);
    if (!want || j.kind != K_C2C || !a.vec_fast || a.ld_rows || !a.cin.vec || !a.cout.vec || j.npass < 2 ||
        j.nbatch > 1)
        return false;
    if (v.vs != 1 || v.es <= 0 || vpb % 2 != 0 || 2 * vpb > 256) return false;
    const T *base = (const T *)v.re + 2 * v.off;
    if (((uintptr_t)base % 16) || ((2 * v.es * (long)sizeof(T)) % 16)) return false;
    const long N = j.N;
    const long q = std::max(1L, 128L / (vpb * 2 * (long)sizeof(T)));  // rows keeping each box 128-byte aligned
    const long nb = (N + 255) / 256;
    long rows = (N + nb - 1) / nb;
    rows = (rows + q - 1) / q * q;
    if (rows > 256 || nb * rows > ld) return false;
    EncodeTiledFn enc = encode_tiled();
    if (!enc) return false;
    int *status = kernel_status();
    if (!status) return false;
    cuuint64_t dims[2] = {(cuuint64_t)(2 * j.nvec), (cuuint64_t)N};
    cuuint64_t strides[1] = {(cuuint64_t)(2 * v.es * (long)sizeof(T))};
    cuuint32_t box[2] = {(cuuint32_t)(2 * vpb), (cuuint32_t)rows};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = enc(&a.tmap, sizeof(T) == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2,
                     (void *)base, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                     CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return false;
    a.tma = 1;
    a.tma_boxes = (int)nb;
    a.tma_rows = (int)rows;
    a.tma_bytes = (unsigned)(nb * rows * vpb * 2 * sizeof(T));
    a.tma_expire = test_wait_expiry() ? 1 : 0;
    a.status = status;
    return true;
}

template <typename T>
long smem_len_limit(int kind) {
    Device *d = device();
    size_t cap = d ? d->smem_optin - kStaticSmem : 48 * 1024;
    long byfit = (long)(cap / (2 * sizeof(T))) - 2;
    long bythreads = (long)KCfg<T>::EMAX_L * KCfg<T>::MAXT_L;
    long lim = byfit < bythreads ? byfit : bythreads;
    (void)kind;
    return lim;
}

// Pass counts per codelet (order of kRadixList) packed 4 bits each; false if
// a radix is not a codelet or a count does not fit.
inline bool pack_passes(const int *radix, int n, unsigned long long *out) {
    int cnt[kRadices] = {0};
    for (int i = 0; i < n; i++) {
        int r = 0;
        while (r < kRadices && kRadixList[r] != radix[i]) r++;
        if (r == kRadices || ++cnt[r] > 15) return false;
    }
    // the plan lists its radices in the kernels' loop order (largest first)
    for (int i = 1; i < n; i++)
        if (radix[i] > radix[i - 1]) return false;
    unsigned long long v = 0;
    for (int r = 0; r < kRadices; r++) v |= (unsigned long long)cnt[r] << (4 * r);
    *out = v;
    return true;
}
inline bool pack_passes(const std::vector<int> &radix, unsigned long long *out) {
    return pack_passes(radix.data(), (int)radix.size(), out);
}

// Threads needed so that every pass fits: a thread holds pass_k(EMAX, R)
// butterflies of radix R.
template <int EMAX>
static long threads_needed(const Job &j, long elems) {
    long need = 32;
    for (int i = 0; i < j.npass; i++) {
        long R = j.radix[i];
        long K = pass_k(EMAX, (int)R);
        long t = (elems / R + K - 1) / K;
        if (t > need) need = t;
    }
    return ((need + 31) / 32) * 32;
}

template <typename T, int KIND, int EMAX, int MAXT>
static bool launch_smem_v(SmemArgs<T> &a, const Job &j, long vpb, long ld, cudaStream_t st) {
    typedef typename cplx_t<T>::t C;
    Device *d = device();
    long nthr = threads_needed<EMAX>(j, vpb * j.N);
    if (nthr < 64) nthr = 64;
    if (nthr > MAXT) {
        set_error(E_UNSUPPORTED, "transform too large for the shared-memory kernel");
        return false;
    }
    a.vpb = (int)vpb;
    a.mvpb = magic_host((unsigned long)vpb);
    a.ld = (int)ld;
    tma_columns<T>(a, j, vpb, ld);
    {
        const long Lin = j.N + (j.kind == K_C2R ? 1 : 0), Lout = j.N + (j.kind == K_R2C ? 1 : 0);
        a.win = walk_const(a.vec_fast ? vpb : Lin, nthr);
        a.wout = walk_const(a.vec_fast ? vpb : Lout, nthr);
    }
    size_t smem = (size_t)vpb * ld * sizeof(C);
    static std::atomic<bool> attr_set{false};  // set once; concurrent first calls both set it
    if (!attr_set) {
        if (!cuda_ok(cudaFuncSetAttribute(k_smem<T, KIND, EMAX, MAXT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)(d->smem_optin - kStaticSmem)),
                     "cudaFuncSetAttribute"))
            return false;
        attr_set = true;
    }
    long grid = (j.nvec + vpb - 1) / vpb;
    if (grid > 0x7fffffffL) {
        set_error(E_UNSUPPORTED, "too many transforms for one launch");
        return false;
    }
    // groups along y, at most 65535 per launch
    for (long y0 = 0; y0 < j.nbatch; y0 += 65535) {
        const long ny = std::min(65535L, j.nbatch - y0);
        SmemArgs<T> b = a;
        b.cin.off += y0 * a.bvs_in;
        b.cout.off += y0 * a.bvs_out;
        b.y0 = y0;
        k_smem<T, KIND, EMAX, MAXT><<<dim3((unsigned)grid, (unsigned)ny), (unsigned)nthr, smem, st>>>(b);
        count_launch();
        if (!cuda_ok(cudaGetLastError(), "k_smem launch")) return false;
    }
    return true;
}

// The shared-memory kernel for transform kind KIND (one instantiation per
// kind keeps each kind's register allocation to its own code).
template <typename T, int KIND>
bool launch_smem_t(const Job &j, cudaStream_t st) {
    typedef typename cplx_t<T>::t C;
    typedef KCfg<T> K;
    Device *d = device();
    if (!d) return false;
    if (j.nvec <= 0 || j.N <= 0) return true;
    SmemArgs<T> a;
    memset(&a, 0, sizeof(a));
    a.kind = j.kind;
    a.N = (int)j.N;
    a.nvec = j.nvec;
    a.inv = j.inv;
    a.has_scale = j.has_scale;
    a.scale = (T)j.scale;
    if (!pack_passes(j.radix, j.npass, &a.passes) || !j.pc) {
        set_error(E_UNSUPPORTED, "pass schedule not handled by the shared-memory kernel");
        return false;
    }
    a.pc = (const uint4 *)j.pc;
    a.cin = cacc<T>(j.cin);
    a.cout = csto<T>(j.cout);
    a.rin = racc<T>(j.rin);
    a.rout = rsto<T>(j.rout);
    a.tw = (const C *)j.tw;
    a.thalf = (const C *)j.thalf;
    // global access mapping: when consecutive transforms are adjacent in memory
    // (column transforms of a row-major matrix) consecutive threads take
    // consecutive transforms, otherwise consecutive elements of one transform.
    long es_in = (j.kind == K_R2C) ? j.rin.es : j.cin.es, vs_in = (j.kind == K_R2C) ? j.rin.vs : j.cin.vs;
    long es_out = (j.kind == K_C2R) ? j.rout.es : j.cout.es, vs_out = (j.kind == K_C2R) ? j.rout.vs : j.cout.vs;
    bool vf_in = labs_(vs_in) == 1 && labs_(es_in) != 1;
    bool vf_out = labs_(vs_out) == 1 && labs_(es_out) != 1;
    a.vec_fast = (vf_in || vf_out) ? 1 : 0;
    // a row-contiguous side of a column-type tile keeps the element-fastest mapping
    a.ld_rows = (a.vec_fast && !vf_in && labs_(es_in) == 1) ? 1 : 0;
    a.st_rows = (a.vec_fast && !vf_out && labs_(es_out) == 1) ? 1 : 0;
    a.conj_in = j.conj_in < 0 ? j.inv : j.conj_in;
    a.conj_out = j.conj_out < 0 ? j.inv : j.conj_out;
    a.bvs_in = j.bvs_in;
    a.bvs_out = j.bvs_out;
    a.tw_lo = (const C *)j.tw_lo;
    a.tw_hi = (const C *)j.tw_hi;
    a.tw_mask = j.tw_mask;
    a.tw_sh = j.tw_sh;
    a.tw_ts = j.tw_ts;
    a.tw_ys = j.tw_ys;
    if ((j.nbatch > 1 || j.tw_lo || a.conj_in != j.inv || a.conj_out != j.inv) &&
        !(j.kind == K_C2C && a.cin.vec && a.cout.vec && j.npass > 0)) {
        set_error(E_UNSUPPORTED, "long-transform step on a view the fused c2c tile does not take");
        return false;
    }
    {
        // the real side of R2C (input) / C2R (output) read or written as complex
        // pairs by the first / last pass with consecutive threads on consecutive
        // elements: the real rows must not be the column-type side of the tile
        const RView &rv = (j.kind == K_R2C) ? j.rin : j.rout;
        const bool real_rows = (j.kind == K_R2C) ? !vf_in : !vf_out;
        a.real_pairs = (j.kind != K_C2C && real_rows && rv.rst == 1 && rv.es == 1 && rv.off % 2 == 0 &&
                        rv.vs % 2 == 0 && rv.vs > 0 && ((uintptr_t)rv.a % (2 * sizeof(T))) == 0)
                           ? 1
                           : 0;
    }
    // the k-omega pipeline's tapers and power accumulator (their instances only)
    a.tp_n = (const T *)j.taper_n;
    a.tp_n_st = j.taper_n_st;
    a.tp_t = (const T *)j.taper_t;
    a.tp_t_st = j.taper_t_st;
    a.tp_back = j.taper_back;
    a.gram = (T *)j.gram;
    a.g_es = j.gram_es;
    a.g_vs = j.gram_vs;
    a.g_scale = (T)j.gram_scale;
    // the pipeline instances run only on their fused paths (the view walkers
    // know neither tapers nor the power store)
    if (KIND == KX_R2C_TAPER && !a.real_pairs) {
        set_error(E_UNSUPPORTED, "tapered R2C needs real rows of unit stride, even offset and pitch");
        return false;
    }
    if (KIND == KX_C2C_SPLIT && !(a.cin.cst == 1 && a.cout.cst == 1)) {
        set_error(E_UNSUPPORTED, "split instance on interleaved views");
        return false;
    }
    if (KIND == KX_C2C_POWER && !(a.cin.vec && a.cout.vec)) {
        set_error(E_UNSUPPORTED, "power columns need an interleaved spectrum");
        return false;
    }
    const long N = j.N;
    // shared-memory rows are indexed i + i/16 (conflict-free Stockham passes)
    const long need = N + (j.kind == K_C2R ? 1 : 0);
    long ld = (need - 1) + (need - 1) / 16 + 1;
    a.twg = (const C *)j.twg;
    if (!a.twg) {
        set_error(E_ARG, "plan has no per-pass twiddle tables");
        return false;
    }
    const long elem_cap = (long)K::EMAX_L * K::MAXT_L;
    long vpb;
    if (a.vec_fast) {
        // 16 (f32) or 8 (f64) adjacent transforms: 128-byte rows of the tile;
        // fewer (down to one 32-byte sector) while the grid would leave SMs
        // with under four CTAs
        vpb = (sizeof(T) == 4) ? 16 : 8;
        const long minv = 32 / (long)sizeof(C);
        while (vpb > minv && (j.nvec + vpb - 1) / vpb * j.nbatch < 4L * d->sms) vpb /= 2;
        if (ld % 2 == 0) ld += 1;
    } else {
        long target = (sizeof(T) == 4) ? 2048 : 1024;
        vpb = target / N;
        if (vpb < 1) vpb = 1;
    }
    if (j.tuned_vpb > 0) vpb = j.tuned_vpb;  // the autotuner's transforms per CTA (bounded below)
    size_t cap = d->smem_optin - kStaticSmem;
    while (vpb > 1 && ((size_t)vpb * ld * sizeof(C) > cap || vpb * N > elem_cap ||
                       threads_needed<K::EMAX_L>(j, vpb * N) > K::MAXT_L))
        vpb--;
    if (vpb > j.nvec) vpb = j.nvec;
    if ((size_t)vpb * ld * sizeof(C) > cap || vpb * N > elem_cap) {
        set_error(E_UNSUPPORTED, "length too large for the shared-memory kernel");
        return false;
    }
    // 8 values per thread and pass when the threads suffice, else 16 (the
    // autotuner may ask for 16 where 8 would fit)
    if (j.tuned_emax != K::EMAX_L && threads_needed<K::EMAX_S>(j, vpb * N) <= K::MAXT_S)
        return launch_smem_v<T, KIND, K::EMAX_S, K::MAXT_S>(a, j, vpb, ld, st);
    return launch_smem_v<T, KIND, K::EMAX_L, K::MAXT_L>(a, j, vpb, ld, st);
}

template <typename T>
static CView dense_view(void *buf, long N) {
    CView v;
    v.re = buf;
    v.im = (T *)buf + 1;
    v.cst = 2;
    v.off = 0;
    v.es = 1;
    v.vs = N;
    return v;
}

template <typename T>
static bool gpass(const GPassArgs<T> &a, cudaStream_t st) {
    Device *d = device();
    long total = gpass_items(a.nvec, a.N, a.R);
    long grid = (total + 255) / 256;
    long gmax = (long)d->sms * 32;
    if (grid > gmax) grid = gmax;
    if (grid < 1) grid = 1;
    const unsigned g = (unsigned)grid;
    typedef typename cplx_t<T>::t C;
    // the first pass (Ns = 1) stages its outputs in shared memory when the
    // staging and the slots' indices (256 x (8 + 4) bytes of static shared
    // memory) fit the default 48 KB (coalesced stores)
    switch (a.R) {
#define JV_GPASS_R(R)                                                                               \
    case R:                                                                                         \
        if (a.Ns == 1 && 256 * gpass_stage_pitch<R>() * sizeof(C) + 256 * 12 <= 48 * 1024)          \
            k_gpass_r1<T, R><<<g, 256, 256 * gpass_stage_pitch<R>() * sizeof(C), st>>>(a);          \
        else                                                                                        \
            k_gpass_r<T, R><<<g, 256, 0, st>>>(a);                                                  \
        break;
        JV_GPASS_R(2) JV_GPASS_R(3) JV_GPASS_R(4) JV_GPASS_R(5) JV_GPASS_R(6) JV_GPASS_R(7) JV_GPASS_R(8)
        JV_GPASS_R(9) JV_GPASS_R(10) JV_GPASS_R(12) JV_GPASS_R(14) JV_GPASS_R(15) JV_GPASS_R(16)
        JV_GPASS_R(11) JV_GPASS_R(13) JV_GPASS_R(17) JV_GPASS_R(19) JV_GPASS_R(23)
#undef JV_GPASS_R
        default: k_gpass<T><<<g, 256, 0, st>>>(a); break;  // primes above 23: direct sums
    }
    count_launch();
    return cuda_ok(cudaGetLastError(), "k_gpass launch");
}

template <typename T>
static unsigned grid_for(long total) {
    Device *d = device();
    long g = (total + 255) / 256;
    long gmax = (long)d->sms * 32;
    if (g > gmax) g = gmax;
    if (g < 1) g = 1;
    return (unsigned)g;
}

// Helper kernels of the real long transforms (two-step path).
template <typename T>
bool launch_r2c_pairs_t(void *z, long es, long vs, long N, long nvec, int has_scale, double scale,
                        const void *thalf, cudaStream_t st) {
    typedef typename cplx_t<T>::t C;
    PairSplitArgs<T> a;
    a.z = (C *)z;
    a.es = es;
    a.vs = vs;
    a.N = (int)N;
    a.nvec = nvec;
    a.has_scale = has_scale;
    a.scale = (T)scale;
    a.thalf = (const C *)thalf;
    k_r2c_split_pairs<T><<<grid_for<T>(nvec * (N / 2 + 1)), 256, 0, st>>>(a);
    count_launch();
    return cuda_ok(cudaGetLastError(), "k_r2c_split_pairs launch");
}

template <typename T>
bool launch_c2r_unsplit_t(const Job &j, void *ydst, cudaStream_t st) {
    typedef typename cplx_t<T>::t C;
    SplitArgs<T> s;
    memset(&s, 0, sizeof(s));
    s.N = (int)j.N;
    s.nvec = j.nvec;
    s.zin = cacc<T>(j.cin);
    s.ydst = (C *)ydst;
    s.thalf = (const C *)j.thalf;
    k_c2r_unsplit<T><<<grid_for<T>(j.nvec * j.N), 256, 0, st>>>(s);
    count_launch();
    return cuda_ok(cudaGetLastError(), "k_c2r_unsplit launch");
}

template <typename T>
bool launch_c2r_unpack_t(const Job &j, const void *y, cudaStream_t st) {
    typedef typename cplx_t<T>::t C;
    UnpackArgs<T> u;
    memset(&u, 0, sizeof(u));
    u.N = (int)j.N;
    u.nvec = j.nvec;
    u.has_scale = j.has_scale;
    u.scale = (T)j.scale;
    u.y = (const C *)y;
    u.xout = rsto<T>(j.rout);
    k_c2r_unpack<T><<<grid_for<T>(j.nvec * j.N), 256, 0, st>>>(u);
    count_launch();
    return cuda_ok(cudaGetLastError(), "k_c2r_unpack launch");
}

// Global-memory path: one launch per radix pass, dense scratch between passes.
template <typename T>
bool launch_global_t(const Job &j, cudaStream_t st) {
    typedef typename cplx_t<T>::t C;
    if (j.nvec <= 0 || j.N <= 0) return true;
    const long N = j.N;
    const size_t bytes = (size_t)j.nvec * N * sizeof(C);
    void *A = dmalloc(bytes), *B = dmalloc(bytes);
    if (!A || !B) {
        dfree(A);
        dfree(B);
        return false;
    }
    bool ok = true;
    GPassArgs<T> g;
    memset(&g, 0, sizeof(g));
    g.N = (int)N;
    g.nvec = j.nvec;
    g.tw = (const C *)j.tw;
    void *cur = A, *nxt = B;
    if (j.kind == K_C2C) {
        const int np = j.npass;
        if (np == 0) {
            // length-1 transform: a radix-1 pass is a copy with scale
            GPassArgs<T> a = g;
            a.R = 1;
            a.Ns = 1;
            a.src = cacc<T>(j.cin);
            a.dst = csto<T>(j.cout);
            a.has_scale = j.has_scale;
            a.scale = (T)j.scale;
            ok = gpass<T>(a, st);
        }
        int Ns = 1;
        for (int p = 0; p < np && ok; p++) {
            GPassArgs<T> a = g;
            a.R = j.radix[p];
            a.Ns = Ns;
            bool first = (p == 0), last = (p == np - 1);
            a.src = first ? cacc<T>(j.cin) : cacc<T>(dense_view<T>(cur, N));
            a.conj_in = first && j.inv;
            bool to_out = last && !(j.inplace && np == 1);
            if (to_out) {
                a.dst = csto<T>(j.cout);
                a.conj_out = j.inv;
                a.has_scale = j.has_scale;
                a.scale = (T)j.scale;
            } else {
                a.dst = csto<T>(dense_view<T>(first ? cur : nxt, N));
            }
            ok = gpass<T>(a, st);
            if (!first) {
                void *t = cur;
                cur = nxt;
                nxt = t;
            }
            Ns *= j.radix[p];
        }
        if (ok && j.inplace && np == 1) {
            // single pass in place: the pass wrote scratch, a radix-1 copy finishes
            GPassArgs<T> a = g;
            a.R = 1;
            a.Ns = 1;
            a.src = cacc<T>(dense_view<T>(cur, N));
            a.dst = csto<T>(j.cout);
            a.conj_out = j.inv;
            a.has_scale = j.has_scale;
            a.scale = (T)j.scale;
            ok = gpass<T>(a, st);
        }
    } else if (j.kind == K_R2C) {
        int Ns = 1;
        for (int p = 0; p < j.npass && ok; p++) {
            GPassArgs<T> a = g;
            a.R = j.radix[p];
            a.Ns = Ns;
            if (p == 0) {
                a.src_real = 1;
                a.rsrc = racc<T>(j.rin);
                a.dst = csto<T>(dense_view<T>(cur, N));
            } else {
                a.src = cacc<T>(dense_view<T>(cur, N));
                a.dst = csto<T>(dense_view<T>(nxt, N));
            }
            ok = gpass<T>(a, st);
            if (p > 0) {
                void *t = cur;
                cur = nxt;
                nxt = t;
            }
            Ns *= j.radix[p];
        }
        if (ok && j.npass == 0) {  // MN = 1: pack only
            GPassArgs<T> a = g;
            a.R = 1;
            a.Ns = 1;
            a.src_real = 1;
            a.rsrc = racc<T>(j.rin);
            a.dst = csto<T>(dense_view<T>(cur, N));
            ok = gpass<T>(a, st);
        }
        if (ok) {
            SplitArgs<T> s;
            memset(&s, 0, sizeof(s));
            s.N = (int)N;
            s.nvec = j.nvec;
            s.has_scale = j.has_scale;
            s.scale = (T)j.scale;
            s.zsrc = (const C *)cur;
            s.xout = csto<T>(j.cout);
            s.thalf = (const C *)j.thalf;
            k_r2c_split<T><<<grid_for<T>(j.nvec * (N + 1)), 256, 0, st>>>(s);
            count_launch();
            ok = cuda_ok(cudaGetLastError(), "k_r2c_split launch");
        }
    } else {
        SplitArgs<T> s;
        memset(&s, 0, sizeof(s));
        s.N = (int)N;
        s.nvec = j.nvec;
        s.zin = cacc<T>(j.cin);
        s.ydst = (C *)cur;
        s.thalf = (const C *)j.thalf;
        k_c2r_unsplit<T><<<grid_for<T>(j.nvec * N), 256, 0, st>>>(s);
        count_launch();
        ok = cuda_ok(cudaGetLastError(), "k_c2r_unsplit launch");
        int Ns = 1;
        for (int p = 0; p < j.npass && ok; p++) {
            GPassArgs<T> a = g;
            a.R = j.radix[p];
            a.Ns = Ns;
            a.src = cacc<T>(dense_view<T>(cur, N));
            a.dst = csto<T>(dense_view<T>(nxt, N));
            ok = gpass<T>(a, st);
            void *t = cur;
            cur = nxt;
            nxt = t;
            Ns *= j.radix[p];
        }
        if (ok) {
            UnpackArgs<T> u;
            memset(&u, 0, sizeof(u));
            u.N = (int)N;
            u.nvec = j.nvec;
            u.has_scale = j.has_scale;
            u.scale = (T)j.scale;
            u.y = (const C *)cur;
            u.xout = rsto<T>(j.rout);
            k_c2r_unpack<T><<<grid_for<T>(j.nvec * N), 256, 0, st>>>(u);
            count_launch();
            ok = cuda_ok(cudaGetLastError(), "k_c2r_unpack launch");
        }
    }
    // scratch goes back to the pool; reuse is ordered on the library stream
    dfree(A);
    dfree(B);
    return ok;
}

}  // namespace jv
