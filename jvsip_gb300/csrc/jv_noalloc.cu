// jv_noalloc.cu -- a complex-to-complex multiple FFT that allocates nothing.
//
// Some callers cannot allocate device memory at the moment they need a
// transform: real-time or interrupt-driven threads that must not block in the
// driver's allocator, and applications whose device memory is reserved in
// full up front by another framework.
// jvsip_ccfftm_noalloc_f serves them.  It runs the library's multi-pass
// global-memory transform -- the path used for lengths with prime factors
// above 7 or lengths too long for shared memory -- with the two intermediate
// buffers that path needs taken from one fixed array in device memory that is
// part of the library image, instead of from the allocator.
//
// The caller passes device pointers to the input and output and a plan made
// beforehand (plan creation allocates; this call does not).  The array holds
// at most JV_NOALLOC_MAX complex points per buffer, so mN * MN of the plan must
// not exceed it; larger calls are rejected with an error.  The array lives on
// every GPU that loads the library until the process exits.  Its address on
// the library's device is looked up once, by the first call (which makes that
// device current for the lookup).  Every call uses the
// same array and it keeps the last call's contents; nothing in it has to start
// at zero because every pass writes all the scratch it later reads.  Calls are
// issued on the library's stream, so calls from this library are ordered;
// calls that overlap on the GPU by other means (another process-wide stream
// using the same library instance concurrently) would race on the array.
#include <mutex>

#include "jv_launch.cuh"

namespace jv {

constexpr long JV_NOALLOC_MAX = 1L << 20;   // complex points per scratch buffer (8 MiB)

// two scratch buffers of JV_NOALLOC_MAX float2 each: 16 MiB per device
static __device__ __align__(256) float2 g_noalloc_scratch[2 * JV_NOALLOC_MAX];

static std::mutex g_na_mu;
static float2 *g_na_addr = nullptr;  // device address of the array on the library's device

// Device address of the scratch array on the library's device, looked up on
// the first call with that device made current for the lookup (the library
// runs all its work on one device, Device::id, and its stream).
static float2 *noalloc_scratch(const Device *d) {
    std::lock_guard<std::mutex> lk(g_na_mu);
    if (g_na_addr) return g_na_addr;
    int cur = -1;
    if (!cuda_ok(cudaGetDevice(&cur), "cudaGetDevice")) return nullptr;
    if (cur != d->id && !cuda_ok(cudaSetDevice(d->id), "cudaSetDevice to the library's device")) return nullptr;
    void *ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (cur != d->id) cudaSetDevice(cur);
    if (e != cudaSuccess || !ptr) {
        set_error(E_CUDA, std::string("cudaGetSymbolAddress of the fixed scratch: ") + cudaGetErrorString(e));
        return nullptr;
    }
    g_na_addr = (float2 *)ptr;
    return g_na_addr;
}

}  // namespace jv

using namespace jv;

extern "C" int jvsip_ccfftm_noalloc_f(const vsip_fftm_f *plan, const void *x, long x_pitch, void *y, long y_pitch) {
    Plan *p = plan_of(plan);
    if (!p || p->prec != P_F32 || (p->type != JV_CCFFTOP && p->type != JV_CCFFTIP)) {
        set_error(E_ARG, "jvsip_ccfftm_noalloc_f: needs a complex-to-complex single-precision plan");
        return E_ARG;
    }
    if (!x || !y || ((uintptr_t)x % 8) || ((uintptr_t)y % 8)) {
        set_error(E_ARG, "jvsip_ccfftm_noalloc_f: input and output must be 8-byte aligned device pointers");
        return E_ARG;
    }
    const long N = p->MN, nv = p->mN;
    // pitch: distance between consecutive transforms (ROW plans) or between
    // consecutive points of a transform (COL plans), in complex elements
    const long need = (p->major == 0) ? N : nv;
    if (x_pitch < need || y_pitch < need) {
        set_error(E_ARG, p->major == 0 ? "jvsip_ccfftm_noalloc_f: row pitch smaller than the row (VSIP_ROW plan)"
                                       : "jvsip_ccfftm_noalloc_f: column pitch smaller than the number of columns "
                                         "(VSIP_COL plan)");
        return E_ARG;
    }
    {
        // the passes read x while writing y: the two may be one buffer
        // (in place) but must not overlap otherwise
        const uintptr_t xb = (uintptr_t)x, yb = (uintptr_t)y;
        const long span_x = (p->major == 0 ? (nv - 1) * x_pitch + N : (N - 1) * x_pitch + nv);
        const long span_y = (p->major == 0 ? (nv - 1) * y_pitch + N : (N - 1) * y_pitch + nv);
        const uintptr_t xe = xb + (uintptr_t)span_x * 8, ye = yb + (uintptr_t)span_y * 8;
        if (xb != yb && N > 0 && nv > 0 && xb < ye && yb < xe) {
            set_error(E_ARG, "jvsip_ccfftm_noalloc_f: input and output overlap without being the same buffer");
            return E_ARG;
        }
    }
    if (N * nv > JV_NOALLOC_MAX) {
        set_error(E_ARG, "jvsip_ccfftm_noalloc_f: mN*MN exceeds the fixed scratch of 1048576 complex points");
        return E_ARG;
    }
    Device *d = device();
    if (!d) return E_NODEVICE;
    float2 *sc = noalloc_scratch(d);
    if (!sc) return jvsip_gpu_last_error();
    if (N <= 0 || nv <= 0) return 0;

    CView cin, cout;
    cin.re = (void *)x;
    cin.im = (float *)x + 1;
    cin.cst = 2;
    cin.off = 0;
    cout.re = y;
    cout.im = (float *)y + 1;
    cout.cst = 2;
    cout.off = 0;
    if (p->major == 0) {
        cin.es = 1;
        cin.vs = x_pitch;
        cout.es = 1;
        cout.vs = y_pitch;
    } else {
        cin.es = x_pitch;
        cin.vs = 1;
        cout.es = y_pitch;
        cout.vs = 1;
    }
    const bool inplace = (x == (const void *)y);
    const int inv = (p->dir == 1) ? 1 : 0;
    const bool has_scale = (p->scale != 1.0);
    const int np = (int)p->radix.size();
    cudaStream_t st = d->stream;

    GPassArgs<float> g;
    memset(&g, 0, sizeof(g));
    g.N = (int)N;
    g.nvec = nv;
    g.tw = (const float2 *)p->d_tw;
    void *cur = sc, *nxt = sc + JV_NOALLOC_MAX;
    bool ok = true;
    if (np == 0) {  // length 1: a radix-1 pass is a copy with scale
        GPassArgs<float> a = g;
        a.R = 1;
        a.Ns = 1;
        a.src = cacc<float>(cin);
        a.dst = csto<float>(cout);
        a.has_scale = has_scale;
        a.scale = (float)p->scale;
        ok = gpass<float>(a, st);
    }
    int Ns = 1;
    for (int q = 0; q < np && ok; q++) {
        GPassArgs<float> a = g;
        a.R = p->radix[q];
        a.Ns = Ns;
        bool first = (q == 0), last = (q == np - 1);
        a.src = first ? cacc<float>(cin) : cacc<float>(dense_view<float>(cur, N));
        a.conj_in = first && inv;
        if (last && !(inplace && np == 1)) {
            a.dst = csto<float>(cout);
            a.conj_out = inv;
            a.has_scale = has_scale;
            a.scale = (float)p->scale;
        } else {
            a.dst = csto<float>(dense_view<float>(first ? cur : nxt, N));
        }
        ok = gpass<float>(a, st);
        if (!first) {
            void *t = cur;
            cur = nxt;
            nxt = t;
        }
        Ns *= p->radix[q];
    }
    if (ok && inplace && np == 1) {
        GPassArgs<float> a = g;
        a.R = 1;
        a.Ns = 1;
        a.src = cacc<float>(dense_view<float>(cur, N));
        a.dst = csto<float>(cout);
        a.conj_out = inv;
        a.has_scale = has_scale;
        a.scale = (float)p->scale;
        ok = gpass<float>(a, st);
    }
    return ok ? 0 : jvsip_gpu_last_error();
}
