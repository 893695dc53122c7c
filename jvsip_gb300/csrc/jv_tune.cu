// jv_tune.cu -- autotuner for the batching form.
//
// For a transform length N, precision and stride class (transforms adjacent
// in memory -- column transforms -- or not) it times the persistent batch
// kernel on scratch data with each candidate number of FFTs per tile (powers
// of two up to the 16384-point tile limit) and keeps the fastest.  Results
// live in memory and in a versioned text cache, one line per key, keyed also
// by the GPU name, in $JVSIP_GPU_TUNE_CACHE or ~/.cache/jvsip_gb300/tune-v2.txt
// (safe to delete).  Lengths that were never tuned use the heuristic below.
#include <errno.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>
#include <sys/types.h>

#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "jv_core.h"

namespace jv {

static std::mutex g_tune_mu;
static std::map<std::tuple<long, int, int>, long> g_tuned;
static bool g_loaded = false;
static std::string g_gpu;

static std::string cache_path() {
    const char *e = getenv("JVSIP_GPU_TUNE_CACHE");
    if (e && *e) return e;
    const char *h = getenv("HOME");
    return std::string(h ? h : "/tmp") + "/.cache/jvsip_gb300/tune-v2.txt";
}

static void load_cache() {
    if (g_loaded) return;
    g_loaded = true;
    Device *d = device();
    if (d) {
        cudaDeviceProp prop;
        if (cudaGetDeviceProperties(&prop, d->id) == cudaSuccess) g_gpu = prop.name;
    }
    for (char &c : g_gpu)
        if (c == ' ') c = '_';
    FILE *f = fopen(cache_path().c_str(), "r");
    if (!f) return;
    char gpu[256];
    long N, per;
    int prec, vf;
    while (fscanf(f, "%255s %ld %d %d %ld", gpu, &N, &prec, &vf, &per) == 5)
        if (g_gpu == gpu && per > 0) g_tuned[std::make_tuple(N, prec, vf)] = per;
    fclose(f);
}

// every directory of `dir` that does not exist yet, created in turn (mode
// 0755); true when the whole path exists as a directory afterwards
static bool make_dirs(const std::string &dir) {
    if (dir.empty()) return true;
    for (size_t i = 1; i <= dir.size(); i++) {
        if (i < dir.size() && dir[i] != '/') continue;
        const std::string part = dir.substr(0, i);
        if (mkdir(part.c_str(), 0755) != 0 && errno != EEXIST) return false;
    }
    struct stat st;
    return stat(dir.c_str(), &st) == 0 && S_ISDIR(st.st_mode);
}

static void save_entry(long N, int prec, int vf, long per) {
    std::string p = cache_path();
    const size_t slash = p.find_last_of('/');
    if (slash != std::string::npos && !make_dirs(p.substr(0, slash))) return;
    FILE *f = fopen(p.c_str(), "a");
    if (!f) return;
    fprintf(f, "%s %ld %d %d %ld\n", g_gpu.empty() ? "gpu" : g_gpu.c_str(), N, prec, vf, per);
    fclose(f);
}

// heuristic: about 4096 points per tile for row transforms (a 256-thread CTA,
// four per SM), 16 columns per tile for column transforms (one 128-byte
// segment per row of the tile)
static long heuristic(long N, bool vf, long rows) {
    long per = vf ? 16 : std::max(1L, 4096 / N);
    while (per > 1 && per * N > 16384) per--;
    if (per > rows) per = rows;
    return std::max(1L, per);
}

long batch_fft_per_tile(long N, bool vf, long rows) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    load_cache();
    auto it = g_tuned.find(std::make_tuple(N, (int)P_F32, vf ? 1 : 0));
    long per = (it != g_tuned.end()) ? it->second : heuristic(N, vf, rows);
    while (per > 1 && per * N > 16384) per--;
    if (per > rows) per = rows;
    return std::max(1L, per);
}

long tuned_entries() {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    load_cache();
    return (long)g_tuned.size();
}

void tune_store(long N, int prec, int vf, long per) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    load_cache();
    g_tuned[std::make_tuple(N, prec, vf)] = per;
    save_entry(N, prec, vf, per);
}

}  // namespace jv

using namespace jv;

extern "C" {

// Tune the batch kernel's FFTs per tile for each of the n lengths (single
// precision; vf = 1 for column transforms).  Times candidates with the
// library's own batch call on scratch blocks; returns 0 on success.
int jvsip_fftm_autotune_f(size_t n, const unsigned long *lengths, int vf) {
    Device *d = device();
    if (!d) return E_NODEVICE;
    for (size_t i = 0; i < n; i++) {
        long N = (long)lengths[i];
        if (N < 2 || N > 16384) continue;
        // about 32 MiB of data per candidate run
        long rows = std::max(1L, (32L << 20) / (16 * N));
        size_t cplx = (size_t)rows * N;
        std::vector<float> host(2 * cplx, 0.5f);
        vsip_cblock_f *bx = vsip_cblockbind_f(host.data(), NULL, cplx, VSIP_MEM_NONE);
        if (!bx) return E_ALLOC;
        if (vsip_cblockadmit_f(bx, 1)) {
            vsip_cblockdestroy_f(bx);
            return jvsip_gpu_last_error();
        }
        vsip_cmview_f *v = vf ? vsip_cmbind_f(bx, 0, rows, N, 1, rows) : vsip_cmbind_f(bx, 0, N, rows, 1, N);
        vsip_fftm_f *p = vf ? vsip_ccfftmip_create_f(N, rows, 1.0f, VSIP_FFT_FWD, VSIP_COL, 0, VSIP_ALG_TIME)
                            : vsip_ccfftmip_create_f(rows, N, 1.0f, VSIP_FFT_FWD, VSIP_ROW, 0, VSIP_ALG_TIME);
        if (!p || !v) {
            if (v) vsip_cmdestroy_f(v);
            if (p) vsip_fftm_destroy_f(p);
            vsip_cblockdestroy_f(bx);
            return jvsip_gpu_last_error() ? jvsip_gpu_last_error() : E_ALLOC;
        }
        cudaEvent_t e0, e1;
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        long best = -1;
        float best_ms = 1e30f;
        for (long per = 1; per * N <= 16384 && per <= rows; per *= 2) {
            {
                std::lock_guard<std::mutex> lk(g_tune_mu);
                load_cache();
                g_tuned[std::make_tuple(N, (int)P_F32, vf ? 1 : 0)] = per;
            }
            const vsip_fftm_f *pl[1] = {p};
            const vsip_cmview_f *vi[1] = {v};
            jvsip_fftm_batch_f(1, pl, vi, vi);  // warm-up
            cudaEventRecord(e0, d->stream);
            for (int r = 0; r < 3; r++) jvsip_fftm_batch_f(1, pl, vi, vi);
            cudaEventRecord(e1, d->stream);
            cudaEventSynchronize(e1);
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            if (ms < best_ms) {
                best_ms = ms;
                best = per;
            }
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        if (best > 0) tune_store(N, P_F32, vf ? 1 : 0, best);
        vsip_cmdestroy_f(v);
        vsip_fftm_destroy_f(p);
        vsip_cblockrelease_f(bx, 0, NULL, NULL);
        vsip_cblockdestroy_f(bx);
    }
    return jvsip_gpu_last_error();
}

// Number of (length, precision, stride class) entries the tuner holds.
long jvsip_fftm_autotune_entries(void) { return tuned_entries(); }

}  // extern "C"
