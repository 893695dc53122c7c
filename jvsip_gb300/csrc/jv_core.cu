// jv_core.cu -- error state, device context, device memory pool, block
// residency and the VSIPL block/view calls of the fftm boundary.
//
// The block and view calls keep the reference's semantics and object layouts
// (c_VSIP_src/VI_cblockbind_f_di.h, VI_cblockadmit_f_di.h:16-29,
// VI_cblockrelease_f_di.h:16-34, VI_cblockdestroy_f_di.h, vsip_blockbind_f.c,
// vsip_blockadmit_f.c, vsip_blockrelease_f.c, vsip_blockdestroy_f.c,
// vsip_cmbind_f.c, vsip_cmcreate_f.c, vsip_cmdestroy_f.c) and add device
// residency: admission creates a device mirror of a user block (uploaded when
// `update` is true), release downloads it (when `update` is true) and frees it.
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <atomic>
#include <map>
#include <unordered_map>
#include <unordered_set>

#include "jv_core.h"

namespace jv {

// ------------------------------------------------------------------ errors
static thread_local int t_err = 0;
static thread_local std::string t_msg;

void set_error(int code, const std::string &msg) {
    t_err = code;
    t_msg = msg;
    if (getenv("JVSIP_GPU_VERBOSE")) fprintf(stderr, "jvsip_gpu: error %d: %s\n", code, msg.c_str());
}

bool cuda_ok(cudaError_t e, const char *what) {
    if (e == cudaSuccess) return true;
    set_error(e == cudaErrorMemoryAllocation ? E_ALLOC : E_CUDA,
              std::string(what) + ": " + cudaGetErrorString(e));
    return false;
}

// ------------------------------------------------------------------ device
static std::mutex g_dev_mu;
static Device g_dev;
static bool g_dev_tried = false;

Device *device() {
    std::lock_guard<std::mutex> lk(g_dev_mu);
    if (g_dev.id >= 0) return &g_dev;
    if (g_dev_tried) {
        set_error(E_NODEVICE, "no usable CUDA device");
        return nullptr;
    }
    g_dev_tried = true;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        set_error(E_NODEVICE, "no usable CUDA device");
        return nullptr;
    }
    int id = 0;
    if (!cuda_ok(cudaGetDevice(&id), "cudaGetDevice")) return nullptr;
    cudaDeviceProp prop;
    if (!cuda_ok(cudaGetDeviceProperties(&prop, id), "cudaGetDeviceProperties")) return nullptr;
    Device d;
    d.id = id;
    d.sms = prop.multiProcessorCount;
    d.smem_optin = prop.sharedMemPerBlockOptin;
    if (!cuda_ok(cudaStreamCreateWithFlags(&d.stream, cudaStreamNonBlocking), "cudaStreamCreate") ||
        !cuda_ok(cudaStreamCreateWithFlags(&d.h2d, cudaStreamNonBlocking), "cudaStreamCreate") ||
        !cuda_ok(cudaStreamCreateWithFlags(&d.d2h, cudaStreamNonBlocking), "cudaStreamCreate"))
        return nullptr;
    for (int i = 0; i < 128; i++)
        if (!cuda_ok(cudaEventCreateWithFlags(&d.ev[i], cudaEventDisableTiming), "cudaEventCreate")) return nullptr;
    g_dev = d;
    return &g_dev;
}

// ------------------------------------------------------------------ launch counter
static std::atomic<unsigned long long> g_launches{0};
void count_launch(unsigned n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
void count_launch_undo(unsigned long long n) { g_launches.fetch_sub(n, std::memory_order_relaxed); }

// Device status word of the kernels that wait on asynchronous copies (the
// TMA-staged column tiles): set to 1 when a bounded wait expired.
static std::mutex g_ks_mu;
static int *g_ks = nullptr;
int *kernel_status() {
    std::lock_guard<std::mutex> lk(g_ks_mu);
    if (!g_ks) {
        g_ks = (int *)dmalloc(sizeof(int));
        if (g_ks && cudaMemset(g_ks, 0, sizeof(int)) != cudaSuccess) g_ks = nullptr;
    }
    return g_ks;
}
// Test hook of the bounded waits (jvsip_gpu_test_wait_expiry).
static std::atomic<int> g_test_expiry{0};
bool test_wait_expiry() { return g_test_expiry.load(std::memory_order_relaxed) != 0; }
void set_test_wait_expiry(int on) { g_test_expiry.store(on ? 1 : 0, std::memory_order_relaxed); }

int kernel_status_check(cudaStream_t st) {
    std::lock_guard<std::mutex> lk(g_ks_mu);
    if (!g_ks) return 0;
    int h = 0;
    if (cudaMemcpyAsync(&h, g_ks, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return E_CUDA;
    if (h) {
        cudaMemsetAsync(g_ks, 0, sizeof(int), st);
        set_error(E_DEVICE, "a bounded wait for an asynchronous tile copy expired");
        return E_DEVICE;
    }
    return 0;
}


// ------------------------------------------------------------------ memory pool
static std::mutex g_pool_mu;
static std::multimap<size_t, void *> g_free;       // size -> buffer
static std::unordered_map<void *, size_t> g_live;  // buffer -> size

static size_t size_class(size_t b) {
    // 2 MiB granularity above 2 MiB, powers of two below
    if (b <= 256) return 256;
    if (b < (2u << 20)) {
        size_t c = 256;
        while (c < b) c <<= 1;
        return c;
    }
    return (b + (2u << 20) - 1) & ~((size_t)(2u << 20) - 1);
}

void *dmalloc(size_t bytes) {
    if (!device()) return nullptr;
    size_t c = size_class(bytes ? bytes : 1);
    {
        std::lock_guard<std::mutex> lk(g_pool_mu);
        auto it = g_free.find(c);
        if (it != g_free.end()) {
            void *p = it->second;
            g_free.erase(it);
            g_live[p] = c;
            return p;
        }
    }
    void *p = nullptr;
    cudaError_t e = cudaMalloc(&p, c);
    if (e == cudaErrorMemoryAllocation) {
        cudaGetLastError();
        pool_trim();
        e = cudaMalloc(&p, c);
    }
    if (!cuda_ok(e, "cudaMalloc")) return nullptr;
    std::lock_guard<std::mutex> lk(g_pool_mu);
    g_live[p] = c;
    return p;
}

void dfree(void *p) {
    if (!p) return;
    std::lock_guard<std::mutex> lk(g_pool_mu);
    auto it = g_live.find(p);
    if (it == g_live.end()) return;
    g_free.emplace(it->second, p);
    g_live.erase(it);
}

void pool_trim() {
    std::lock_guard<std::mutex> lk(g_pool_mu);
    if (g_dev.stream) cudaStreamSynchronize(g_dev.stream);
    for (auto &kv : g_free) cudaFree(kv.second);
    g_free.clear();
}

// ------------------------------------------------------------------ pinned host arrays
static std::mutex g_pin_mu;
static std::unordered_set<const void *> g_pinned;

void *host_alloc(size_t bytes) {
    void *p = nullptr;
    if (getenv("JVSIP_GPU_NO_PINNED") == nullptr && device()) {
        if (cudaMallocHost(&p, bytes ? bytes : 1) == cudaSuccess) {
            std::lock_guard<std::mutex> lk(g_pin_mu);
            g_pinned.insert(p);
            return p;
        }
        cudaGetLastError();
    }
    return malloc(bytes ? bytes : 1);
}

bool pinned_owned(const void *p) {
    std::lock_guard<std::mutex> lk(g_pin_mu);
    return g_pinned.count(p) != 0;
}

void host_free(void *p) {
    if (!p) return;
    {
        std::lock_guard<std::mutex> lk(g_pin_mu);
        auto it = g_pinned.find(p);
        if (it != g_pinned.end()) {
            g_pinned.erase(it);
            cudaFreeHost(p);
            return;
        }
    }
    free(p);
}

// ------------------------------------------------------------------ residency table
static std::mutex g_mir_mu;
static std::unordered_map<const void *, Mirror> g_mirrors;

Mirror *mirror_find(const void *block) {
    std::lock_guard<std::mutex> lk(g_mir_mu);
    auto it = g_mirrors.find(block);
    return it == g_mirrors.end() ? nullptr : &it->second;
}

Mirror *mirror_create(const void *block, size_t bytes, bool split) {
    Mirror m;
    m.bytes = bytes;
    m.d = dmalloc(bytes);
    if (!m.d) return nullptr;
    if (split) {
        m.d_im = dmalloc(bytes);
        if (!m.d_im) {
            dfree(m.d);
            return nullptr;
        }
    }
    std::lock_guard<std::mutex> lk(g_mir_mu);
    auto &slot = g_mirrors[block];
    slot = m;
    return &slot;
}

void mirror_drop(const void *block) {
    Mirror m;
    {
        std::lock_guard<std::mutex> lk(g_mir_mu);
        auto it = g_mirrors.find(block);
        if (it == g_mirrors.end()) return;
        m = it->second;
        g_mirrors.erase(it);
    }
    Device *d = device();
    if (d) cudaStreamSynchronize(d->stream);  // no queued kernel may still use it
    dfree(m.d);
    dfree(m.d_im);
}

}  // namespace jv

using namespace jv;

// ====================================================================== C ABI
extern "C" {

int jvsip_gpu_last_error(void) { return t_err; }
const char *jvsip_gpu_last_error_string(void) { return t_msg.c_str(); }
void jvsip_gpu_clear_error(void) {
    t_err = 0;
    t_msg.clear();
}

int jvsip_gpu_test_wait_expiry(int on) {
    jv::set_test_wait_expiry(on);
    return 0;
}

int jvsip_gpu_synchronize(void) {
    Device *d = device();
    if (!d) return E_NODEVICE;
    if (!cuda_ok(cudaStreamSynchronize(d->stream), "cudaStreamSynchronize")) return E_CUDA;
    const int k = jv::kernel_status_check(d->stream);
    const int sp = split_status_check(d->stream);
    return k ? k : sp;
}

int vsip_init(void *ptr) {
    (void)ptr;
    device();  // bring the device up early; absence is not an error for VSIPL itself
    return 0;
}

int vsip_finalize(void *ptr) {
    (void)ptr;
    Device *d = device();
    if (d) cudaStreamSynchronize(d->stream);
    return 0;
}

}  // extern "C"

// ---------------------------------------------------------------- typed block / view calls
// The body is written once for both precisions.
#define JV_BLOCK_API(SFX, T, CT)                                                                    \
    extern "C" vsip_block_##SFX *vsip_blockbind_##SFX(T *const p, vsip_length N, vsip_memory_hint h) { \
        vsip_block_##SFX *b = (vsip_block_##SFX *)malloc(sizeof(*b));                                \
        if (!b) return NULL;                                                                         \
        b->kind = JV_USER_BLOCK;                                                                     \
        b->admit = JV_RELEASED_BLOCK;                                                                \
        b->markings = JV_VALID_OBJECT;                                                               \
        b->array = p;                                                                                \
        b->rstride = 1;                                                                              \
        b->size = N;                                                                                 \
        b->bindings = 0;                                                                             \
        b->hint = h;                                                                                 \
        b->parent = NULL;                                                                            \
        b->update = 0;                                                                               \
        return b;                                                                                    \
    }                                                                                                \
    extern "C" vsip_block_##SFX *vsip_blockcreate_##SFX(vsip_length N, vsip_memory_hint h) {        \
        vsip_block_##SFX *b = (vsip_block_##SFX *)malloc(sizeof(*b));                                \
        if (!b) return NULL;                                                                         \
        b->array = (T *)host_alloc(N * sizeof(T));                                                   \
        if (!b->array) {                                                                             \
            free(b);                                                                                 \
            return NULL;                                                                             \
        }                                                                                            \
        b->kind = JV_VSIPL_BLOCK;                                                                    \
        b->admit = JV_ADMITTED_BLOCK;                                                                \
        b->markings = JV_VALID_OBJECT;                                                               \
        b->size = N;                                                                                 \
        b->rstride = 1;                                                                              \
        b->bindings = 0;                                                                             \
        b->hint = h;                                                                                 \
        b->parent = NULL;                                                                            \
        b->update = 0;                                                                               \
        return b;                                                                                    \
    }                                                                                                \
    extern "C" int vsip_blockadmit_##SFX(vsip_block_##SFX *b, vsip_scalar_bl update) {              \
        if (!b || b->array == NULL || b->kind != JV_USER_BLOCK) return 1;                            \
        b->admit = JV_ADMITTED_BLOCK;                                                                \
        size_t bytes = b->size * (size_t)(b->rstride > 0 ? b->rstride : 1) * sizeof(T);              \
        Mirror *m = mirror_find(b);                                                                  \
        if (!m) m = mirror_create(b, bytes, false);                                                  \
        if (m && update) {                                                                           \
            Device *d = device();                                                                    \
            if (!cuda_ok(cudaMemcpyAsync(m->d, b->array, bytes, cudaMemcpyHostToDevice, d->stream),  \
                         "admit upload"))                                                            \
                return 1;                                                                            \
            cudaStreamSynchronize(d->stream);                                                        \
        }                                                                                            \
        if (m) m->device_newer = false;                                                              \
        return 0;                                                                                    \
    }                                                                                                \
    extern "C" T *vsip_blockrelease_##SFX(vsip_block_##SFX *b, vsip_scalar_bl update) {             \
        if (!b || b->kind != JV_USER_BLOCK) return NULL;                                             \
        Mirror *m = mirror_find(b);                                                                  \
        if (m) {                                                                                     \
            if (update && m->device_newer) {                                                         \
                Device *d = device();                                                                \
                cuda_ok(cudaMemcpyAsync(b->array, m->d, m->bytes, cudaMemcpyDeviceToHost, d->stream),\
                        "release download");                                                         \
                cudaStreamSynchronize(d->stream);                                                    \
            }                                                                                        \
            mirror_drop(b);                                                                          \
        }                                                                                            \
        b->update = update;                                                                          \
        b->admit = JV_RELEASED_BLOCK;                                                                \
        return b->array;                                                                             \
    }                                                                                                \
    extern "C" void vsip_blockdestroy_##SFX(vsip_block_##SFX *b) {                                  \
        if (!b || b->kind == JV_DERIVED_BLOCK) return;                                               \
        mirror_drop(b);                                                                              \
        b->markings = JV_FREED_OBJECT;                                                               \
        if (b->kind == JV_VSIPL_BLOCK) host_free(b->array);                                          \
        free(b);                                                                                     \
    }                                                                                                \
    extern "C" int jvsip_blocksync_##SFX(vsip_block_##SFX *b) {                                     \
        Mirror *m = b ? mirror_find(b) : nullptr;                                                    \
        if (!m) return 0;                                                                            \
        if (m->device_newer) {                                                                       \
            Device *d = device();                                                                    \
            if (!cuda_ok(cudaMemcpyAsync(b->array, m->d, m->bytes, cudaMemcpyDeviceToHost, d->stream),\
                         "sync download"))                                                           \
                return E_CUDA;                                                                       \
            cudaStreamSynchronize(d->stream);                                                        \
            m->device_newer = false;                                                                 \
        }                                                                                            \
        return 0;                                                                                    \
    }                                                                                                \
    /* complex blocks */                                                                             \
    static vsip_cblock_##SFX *jv_cblock_new_##SFX(T *Rp, T *Ip, vsip_length N, vsip_memory_hint h,  \
                                                  int kind) {                                        \
        vsip_cblock_##SFX *b = (vsip_cblock_##SFX *)calloc(1, sizeof(*b));                           \
        if (!b) return NULL;                                                                         \
        b->hint = h;                                                                                 \
        b->size = N;                                                                                 \
        b->kind = kind;                                                                              \
        b->admit = (kind == JV_USER_BLOCK) ? JV_RELEASED_BLOCK : JV_ADMITTED_BLOCK;                  \
        b->markings = JV_VALID_OBJECT;                                                               \
        b->bindings = 0;                                                                             \
        b->R = (vsip_block_##SFX *)calloc(1, sizeof(vsip_block_##SFX));                              \
        b->I = (vsip_block_##SFX *)calloc(1, sizeof(vsip_block_##SFX));                              \
        if (!b->R || !b->I) {                                                                        \
            free(b->R);                                                                              \
            free(b->I);                                                                              \
            free(b);                                                                                 \
            return NULL;                                                                             \
        }                                                                                            \
        vsip_block_##SFX *parts[2] = {b->R, b->I};                                                   \
        for (int q = 0; q < 2; q++) {                                                                \
            parts[q]->kind = JV_DERIVED_BLOCK;                                                       \
            parts[q]->admit = b->admit;                                                              \
            parts[q]->markings = JV_VALID_OBJECT;                                                    \
            parts[q]->size = N;                                                                      \
            parts[q]->hint = h;                                                                      \
            parts[q]->parent = b;                                                                    \
        }                                                                                            \
        if (Ip == NULL) { /* interleaved */                                                          \
            b->cstride = 2;                                                                          \
            b->R->array = Rp;                                                                        \
            b->I->array = Rp + 1;                                                                    \
            b->R->rstride = b->I->rstride = 2;                                                       \
        } else {                                                                                     \
            b->cstride = 1;                                                                          \
            b->R->array = Rp;                                                                        \
            b->I->array = Ip;                                                                        \
            b->R->rstride = b->I->rstride = 1;                                                       \
        }                                                                                            \
        b->a_zero.r = 0; b->a_zero.i = 0; b->a_one.r = 1; b->a_one.i = 0;                            \
        b->a_imag_one.r = 0; b->a_imag_one.i = 1; b->a_scalar.r = 0; b->a_scalar.i = 0;              \
        return b;                                                                                    \
    }                                                                                                \
    extern "C" vsip_cblock_##SFX *vsip_cblockbind_##SFX(T *const Rp, T *const Ip, vsip_length N,    \
                                                      vsip_memory_hint h) {                          \
        return jv_cblock_new_##SFX(Rp, Ip, N, h, JV_USER_BLOCK);                                     \
    }                                                                                                \
    extern "C" vsip_cblock_##SFX *vsip_cblockcreate_##SFX(vsip_length N, vsip_memory_hint h) {      \
        T *a = (T *)host_alloc(2 * N * sizeof(T));                                                   \
        if (!a) return NULL;                                                                         \
        vsip_cblock_##SFX *b = jv_cblock_new_##SFX(a, NULL, N, h, JV_VSIPL_BLOCK);                   \
        if (!b) host_free(a);                                                                        \
        return b;                                                                                    \
    }                                                                                                \
    extern "C" int vsip_cblockadmit_##SFX(vsip_cblock_##SFX *b, vsip_scalar_bl update) {            \
        if (!b || b->R->array == NULL || b->kind != JV_USER_BLOCK) return 1;                         \
        b->admit = b->R->admit = b->I->admit = JV_ADMITTED_BLOCK;                                    \
        b->a_scalar.r = 0; b->a_scalar.i = 0; b->a_zero.r = 0; b->a_zero.i = 0;                      \
        b->a_one.r = 1; b->a_one.i = 0; b->a_imag_one.r = 0; b->a_imag_one.i = 1;                    \
        bool split = (b->cstride == 1);                                                              \
        size_t bytes = (split ? 1 : 2) * b->size * sizeof(T);                                        \
        Mirror *m = mirror_find(b);                                                                  \
        if (!m) m = mirror_create(b, bytes, split);                                                  \
        if (m && update) {                                                                           \
            Device *d = device();                                                                    \
            bool ok = cuda_ok(cudaMemcpyAsync(m->d, b->R->array, bytes, cudaMemcpyHostToDevice,      \
                                              d->stream), "admit upload");                           \
            if (ok && split)                                                                         \
                ok = cuda_ok(cudaMemcpyAsync(m->d_im, b->I->array, bytes, cudaMemcpyHostToDevice,    \
                                             d->stream), "admit upload");                            \
            cudaStreamSynchronize(d->stream);                                                        \
            if (!ok) return 1;                                                                       \
        }                                                                                            \
        if (m) m->device_newer = false;                                                              \
        return 0;                                                                                    \
    }                                                                                                \
    extern "C" int jvsip_cblocksync_##SFX(vsip_cblock_##SFX *b) {                                   \
        Mirror *m = b ? mirror_find(b) : nullptr;                                                    \
        if (!m) return 0;                                                                            \
        if (m->device_newer) {                                                                       \
            Device *d = device();                                                                    \
            bool ok = cuda_ok(cudaMemcpyAsync(b->R->array, m->d, m->bytes, cudaMemcpyDeviceToHost,  \
                                              d->stream), "sync download");                          \
            if (ok && m->d_im)                                                                       \
                ok = cuda_ok(cudaMemcpyAsync(b->I->array, m->d_im, m->bytes,                         \
                                             cudaMemcpyDeviceToHost, d->stream), "sync download");   \
            cudaStreamSynchronize(d->stream);                                                        \
            if (!ok) return E_CUDA;                                                                  \
            m->device_newer = false;                                                                 \
        }                                                                                            \
        return 0;                                                                                    \
    }                                                                                                \
    extern "C" void vsip_cblockrelease_##SFX(vsip_cblock_##SFX *b, vsip_scalar_bl update, T **Rp,   \
                                             T **Ip) {                                               \
        if (b) b->update = update;                                                                   \
        if (!b || b->kind != JV_USER_BLOCK) {                                                        \
            if (Rp) *Rp = NULL;                                                                      \
            if (Ip) *Ip = NULL;                                                                      \
            return;                                                                                  \
        }                                                                                            \
        if (mirror_find(b)) {                                                                        \
            if (update) jvsip_cblocksync_##SFX(b);                                                   \
            mirror_drop(b);                                                                          \
        }                                                                                            \
        b->admit = b->R->admit = b->I->admit = JV_RELEASED_BLOCK;                                    \
        if (Rp) *Rp = b->R->array;                                                                   \
        if (Ip) *Ip = (b->cstride == 1) ? b->I->array : NULL;                                        \
    }                                                                                                \
    extern "C" void vsip_cblockdestroy_##SFX(vsip_cblock_##SFX *b) {                                \
        if (!b) return;                                                                              \
        mirror_drop(b);                                                                              \
        b->markings = b->R->markings = b->I->markings = JV_FREED_OBJECT;                             \
        if (b->kind == JV_VSIPL_BLOCK) host_free(b->R->array);                                       \
        free(b->R);                                                                                  \
        free(b->I);                                                                                  \
        free(b);                                                                                     \
    }                                                                                                \
    /* views */                                                                                      \
    extern "C" vsip_cmview_##SFX *vsip_cmbind_##SFX(const vsip_cblock_##SFX *b, vsip_offset o,      \
                                                  vsip_stride cs, vsip_length cl, vsip_stride rs,    \
                                                  vsip_length rl) {                                  \
        vsip_cmview_##SFX *v = (vsip_cmview_##SFX *)malloc(sizeof(*v));                              \
        if (!v) return NULL;                                                                         \
        v->block = (vsip_cblock_##SFX *)b;                                                           \
        v->offset = o;                                                                               \
        v->row_stride = rs;                                                                          \
        v->col_stride = cs;                                                                          \
        v->row_length = rl;                                                                          \
        v->col_length = cl;                                                                          \
        v->markings = JV_VALID_OBJECT;                                                               \
        return v;                                                                                    \
    }                                                                                                \
    extern "C" vsip_mview_##SFX *vsip_mbind_##SFX(const vsip_block_##SFX *b, vsip_offset o,         \
                                                vsip_stride cs, vsip_length cl, vsip_stride rs,      \
                                                vsip_length rl) {                                    \
        vsip_mview_##SFX *v = (vsip_mview_##SFX *)malloc(sizeof(*v));                                \
        if (!v) return NULL;                                                                         \
        v->block = (vsip_block_##SFX *)b;                                                            \
        v->offset = o;                                                                               \
        v->row_stride = rs;                                                                          \
        v->col_stride = cs;                                                                          \
        v->row_length = rl;                                                                          \
        v->col_length = cl;                                                                          \
        v->markings = JV_VALID_OBJECT;                                                               \
        return v;                                                                                    \
    }                                                                                                \
    extern "C" vsip_cmview_##SFX *vsip_cmcreate_##SFX(vsip_length m, vsip_length n, vsip_major rc,  \
                                                    vsip_memory_hint h) {                            \
        vsip_cblock_##SFX *b = vsip_cblockcreate_##SFX(m * n, h);                                    \
        if (!b) return NULL;                                                                         \
        vsip_cmview_##SFX *v = (rc == VSIP_ROW) ? vsip_cmbind_##SFX(b, 0, (vsip_stride)n, m, 1, n)   \
                                                : vsip_cmbind_##SFX(b, 0, 1, m, (vsip_stride)m, n);  \
        if (!v) vsip_cblockdestroy_##SFX(b);                                                         \
        return v;                                                                                    \
    }                                                                                                \
    extern "C" vsip_mview_##SFX *vsip_mcreate_##SFX(vsip_length m, vsip_length n, vsip_major rc,    \
                                                  vsip_memory_hint h) {                              \
        vsip_block_##SFX *b = vsip_blockcreate_##SFX(m * n, h);                                      \
        if (!b) return NULL;                                                                         \
        vsip_mview_##SFX *v = (rc == VSIP_ROW) ? vsip_mbind_##SFX(b, 0, (vsip_stride)n, m, 1, n)     \
                                               : vsip_mbind_##SFX(b, 0, 1, m, (vsip_stride)m, n);    \
        if (!v) vsip_blockdestroy_##SFX(b);                                                          \
        return v;                                                                                    \
    }                                                                                                \
    extern "C" vsip_cblock_##SFX *vsip_cmdestroy_##SFX(vsip_cmview_##SFX *v) {                      \
        if (!v) return NULL;                                                                         \
        vsip_cblock_##SFX *b = v->block;                                                             \
        v->markings = JV_FREED_OBJECT;                                                               \
        free(v);                                                                                     \
        return b;                                                                                    \
    }                                                                                                \
    extern "C" vsip_block_##SFX *vsip_mdestroy_##SFX(vsip_mview_##SFX *v) {                         \
        if (!v) return NULL;                                                                         \
        vsip_block_##SFX *b = v->block;                                                              \
        v->markings = JV_FREED_OBJECT;                                                               \
        free(v);                                                                                     \
        return b;                                                                                    \
    }                                                                                                \
    extern "C" void vsip_cmalldestroy_##SFX(vsip_cmview_##SFX *v) {                                 \
        vsip_cblockdestroy_##SFX(vsip_cmdestroy_##SFX(v));                                           \
    }                                                                                                \
    extern "C" void vsip_malldestroy_##SFX(vsip_mview_##SFX *v) {                                   \
        vsip_blockdestroy_##SFX(vsip_mdestroy_##SFX(v));                                             \
    }

JV_BLOCK_API(f, vsip_scalar_f, vsip_cscalar_f)
JV_BLOCK_API(d, vsip_scalar_d, vsip_cscalar_d)

// Vector views of the single-FFT calls (c_VSIP_src/vsip_cvbind_f.c,
// vsip_vbind_f.c, vsip_cvcreate_f.c, vsip_vcreate_f.c, vsip_cvdestroy_f.c,
// vsip_vdestroy_f.c): the same objects as the reference's.
#define JV_VECTOR_API(SFX)                                                                           \
    extern "C" vsip_cvview_##SFX *vsip_cvbind_##SFX(const vsip_cblock_##SFX *b, vsip_offset o,      \
                                                  vsip_stride s, vsip_length n) {                    \
        vsip_cvview_##SFX *v = (vsip_cvview_##SFX *)malloc(sizeof(*v));                              \
        if (!v) return NULL;                                                                         \
        v->block = (vsip_cblock_##SFX *)b;                                                           \
        v->offset = o;                                                                               \
        v->stride = s;                                                                               \
        v->length = n;                                                                               \
        v->markings = JV_VALID_OBJECT;                                                               \
        return v;                                                                                    \
    }                                                                                                \
    extern "C" vsip_vview_##SFX *vsip_vbind_##SFX(const vsip_block_##SFX *b, vsip_offset o,         \
                                                vsip_stride s, vsip_length n) {                      \
        vsip_vview_##SFX *v = (vsip_vview_##SFX *)malloc(sizeof(*v));                                \
        if (!v) return NULL;                                                                         \
        v->block = (vsip_block_##SFX *)b;                                                            \
        v->offset = o;                                                                               \
        v->stride = s;                                                                               \
        v->length = n;                                                                               \
        v->markings = JV_VALID_OBJECT;                                                               \
        return v;                                                                                    \
    }                                                                                                \
    extern "C" vsip_cvview_##SFX *vsip_cvcreate_##SFX(vsip_length n, vsip_memory_hint h) {          \
        vsip_cblock_##SFX *b = vsip_cblockcreate_##SFX(n, h);                                        \
        if (!b) return NULL;                                                                         \
        vsip_cvview_##SFX *v = vsip_cvbind_##SFX(b, 0, 1, n);                                        \
        if (!v) vsip_cblockdestroy_##SFX(b);                                                         \
        return v;                                                                                    \
    }                                                                                                \
    extern "C" vsip_vview_##SFX *vsip_vcreate_##SFX(vsip_length n, vsip_memory_hint h) {            \
        vsip_block_##SFX *b = vsip_blockcreate_##SFX(n, h);                                          \
        if (!b) return NULL;                                                                         \
        vsip_vview_##SFX *v = vsip_vbind_##SFX(b, 0, 1, n);                                          \
        if (!v) vsip_blockdestroy_##SFX(b);                                                          \
        return v;                                                                                    \
    }                                                                                                \
    extern "C" vsip_cblock_##SFX *vsip_cvdestroy_##SFX(vsip_cvview_##SFX *v) {                      \
        if (!v) return NULL;                                                                         \
        vsip_cblock_##SFX *b = v->block;                                                             \
        v->markings = JV_FREED_OBJECT;                                                               \
        free(v);                                                                                     \
        return b;                                                                                    \
    }                                                                                                \
    extern "C" vsip_block_##SFX *vsip_vdestroy_##SFX(vsip_vview_##SFX *v) {                         \
        if (!v) return NULL;                                                                         \
        vsip_block_##SFX *b = v->block;                                                              \
        v->markings = JV_FREED_OBJECT;                                                               \
        free(v);                                                                                     \
        return b;                                                                                    \
    }                                                                                                \
    extern "C" void vsip_cvalldestroy_##SFX(vsip_cvview_##SFX *v) {                                 \
        vsip_cblockdestroy_##SFX(vsip_cvdestroy_##SFX(v));                                           \
    }                                                                                                \
    extern "C" void vsip_valldestroy_##SFX(vsip_vview_##SFX *v) {                                   \
        vsip_blockdestroy_##SFX(vsip_vdestroy_##SFX(v));                                             \
    }

JV_VECTOR_API(f)
JV_VECTOR_API(d)

// The library's CUDA stream (as a void*), so callers can order their own work
// and CUDA events after the fftm calls.
extern "C" void *jvsip_gpu_stream(void) {
    Device *d = device();
    return d ? (void *)d->stream : nullptr;
}

// Number of kernels this library has launched since it was loaded.
extern "C" unsigned long jvsip_gpu_kernel_launches(void) { return (unsigned long)g_launches.load(); }
