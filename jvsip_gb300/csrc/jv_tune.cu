// jv_tune.cu -- autotuner of the c2c paths.
//
// Two kinds of entries, both per (transform length N, precision, stride class:
// 0 = transforms along contiguous rows, 1 = adjacent transforms):
//  * the batching form's FFTs per tile (jvsip_fftm_autotune_f): each candidate
//    (powers of two up to the 16384-point tile limit) timed through the batch
//    call on scratch data;
//  * the plain calls' kernel choice (jvsip_fftm_autotune_plain_f): residency
//    (the register-resident kernel where an instance exists, or the
//    shared-memory kernel), the shared-memory kernel's radix schedule, its
//    transforms per CTA and its complex values per thread and pass (which sets
//    the threads per transform), each candidate timed through vsip_ccfftmip_f
//    on scratch data.  Plans created afterwards take the entry of their length,
//    precision and major (VSIP_ROW: class 0, VSIP_COL: class 1).
// Results live in memory and in a versioned text cache, one line per entry,
// keyed also by the GPU name, in $JVSIP_GPU_TUNE_CACHE or
// ~/.cache/jvsip_gb300/tune-v3.txt (safe to delete):
//   B <gpu> N prec vf per
//   P <gpu> N prec cls res vpb emax npasses r1 ... rn
// Lengths that were never tuned use the heuristics.
#include <errno.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>
#include <sys/types.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "jv_core.h"

namespace jv {

static std::mutex g_tune_mu;
static std::map<std::tuple<long, int, int>, long> g_tuned;        // batch: FFTs per tile
static std::map<std::tuple<long, int, int>, PlainTune> g_plain;   // plain calls: kernel choice
static bool g_loaded = false;
static std::string g_gpu;
static thread_local const PlainTune *t_force = nullptr;

static std::string cache_path() {
    const char *e = getenv("JVSIP_GPU_TUNE_CACHE");
    if (e && *e) return e;
    const char *h = getenv("HOME");
    return std::string(h ? h : "/tmp") + "/.cache/jvsip_gb300/tune-v3.txt";
}

static void parse_line(const char *ln) {
    char tag[4], gpu[256];
    int used = 0;
    if (sscanf(ln, "%3s %255s %n", tag, gpu, &used) != 2 || g_gpu != gpu) return;
    const char *q = ln + used;
    if (!strcmp(tag, "B")) {
        long N, per;
        int prec, vf;
        if (sscanf(q, "%ld %d %d %ld", &N, &prec, &vf, &per) == 4 && per > 0)
            g_tuned[std::make_tuple(N, prec, vf)] = per;
    } else if (!strcmp(tag, "P")) {
        long N;
        int prec, cls, np, n = 0;
        PlainTune t;
        if (sscanf(q, "%ld %d %d %d %d %d %d%n", &N, &prec, &cls, &t.res, &t.vpb, &t.emax, &np, &n) != 7 || np < 1 ||
            np > 40)
            return;
        q += n;
        for (int i = 0; i < np; i++) {
            int r;
            if (sscanf(q, "%d%n", &r, &n) != 1) return;
            q += n;
            t.radix.push_back(r);
        }
        g_plain[std::make_tuple(N, prec, cls)] = t;
    }
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
    if (g_gpu.empty()) g_gpu = "gpu";
    FILE *f = fopen(cache_path().c_str(), "r");
    if (!f) return;
    char ln[1024];
    while (fgets(ln, sizeof ln, f)) parse_line(ln);
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

static void append_line(const std::string &line) {
    std::string p = cache_path();
    const size_t slash = p.find_last_of('/');
    if (slash != std::string::npos && !make_dirs(p.substr(0, slash))) return;
    FILE *f = fopen(p.c_str(), "a");
    if (!f) return;
    fputs(line.c_str(), f);
    fclose(f);
}

static void save_entry(long N, int prec, int vf, long per) {
    char b[512];
    snprintf(b, sizeof b, "B %s %ld %d %d %ld\n", g_gpu.c_str(), N, prec, vf, per);
    append_line(b);
}

static void save_plain(long N, int prec, int cls, const PlainTune &t) {
    std::string ln = "P " + g_gpu + " " + std::to_string(N) + " " + std::to_string(prec) + " " + std::to_string(cls) +
                     " " + std::to_string(t.res) + " " + std::to_string(t.vpb) + " " + std::to_string(t.emax) + " " +
                     std::to_string(t.radix.size());
    for (int r : t.radix) ln += " " + std::to_string(r);
    append_line(ln + "\n");
}

void plain_tune_force(const PlainTune *t) { t_force = t; }

bool plain_tuned(long N, int prec, int cls, PlainTune *out) {
    if (t_force) {
        *out = *t_force;
        return true;
    }
    std::lock_guard<std::mutex> lk(g_tune_mu);
    load_cache();
    auto it = g_plain.find(std::make_tuple(N, prec, cls));
    if (it == g_plain.end()) return false;
    *out = it->second;
    return true;
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
    return (long)(g_tuned.size() + g_plain.size());
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

// Tune the plain c2c calls for each of the n lengths (single precision, 2 to
// 16384 points of 2^a 3^b 5^c 7^d; cls 0: rows, 1: adjacent transforms):
// residency, radix schedule, transforms per CTA and values per thread, each
// candidate timed through vsip_ccfftmip_f on about 32 MiB of scratch data.
int jvsip_fftm_autotune_plain_f(size_t n, const unsigned long *lengths, int cls) {
    Device *d = device();
    if (!d) return E_NODEVICE;
    if (n && !lengths) {
        set_error(E_ARG, "autotune: null length array");
        return E_ARG;
    }
    cls = cls ? 1 : 0;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (!cuda_ok(cudaEventCreate(&e0), "tuner event") || !cuda_ok(cudaEventCreate(&e1), "tuner event")) return E_CUDA;
    int rc = 0;
    for (size_t i = 0; i < n && rc == 0; i++) {
        const long N = (long)lengths[i];
        if (N < 2 || N > 16384) continue;
        // adjacent columns that run as the two steps never use the tiles
        // searched here
        if (cls && N >= kColStepsMin && !fast_step_len(N)) continue;
        const std::vector<std::vector<int>> scheds = schedule_candidates(N, 1024, 6);
        if (scheds.empty()) continue;
        const long cnt = std::max(8L, (32L << 20) / (16 * N));
        const size_t cplx = (size_t)cnt * N;
        std::vector<float> host(2 * cplx, 0.5f);
        vsip_cblock_f *bx = vsip_cblockbind_f(host.data(), NULL, cplx, VSIP_MEM_NONE);
        if (!bx || vsip_cblockadmit_f(bx, 1)) {
            if (bx) vsip_cblockdestroy_f(bx);
            rc = jvsip_gpu_last_error() ? jvsip_gpu_last_error() : E_ALLOC;
            break;
        }
        vsip_cmview_f *v = cls ? vsip_cmbind_f(bx, 0, cnt, N, 1, cnt) : vsip_cmbind_f(bx, 0, N, cnt, 1, N);
        // candidates: the default plan (register-resident kernel where one
        // exists), then the shared-memory kernel over schedules x transforms
        // per CTA x values per thread
        std::vector<PlainTune> cands;
        {
            PlainTune t;
            t.radix = scheds[0];
            cands.push_back(t);
        }
        std::vector<int> vpbs;
        if (cls) vpbs = {2, 4, 8, 16};
        else {
            vpbs.push_back(0);
            for (int vv = 1; vv <= 8 && vv * N <= 16384; vv *= 2) vpbs.push_back(vv);
        }
        for (const std::vector<int> &sc : scheds)
            for (int vv : vpbs)
                for (int em : {8, 16}) {
                    if (em == 8 && vv > 0 && (long)vv * N > 8L * 1024) continue;  // would run with 16 anyway
                    PlainTune t;
                    t.res = 1;
                    t.radix = sc;
                    t.vpb = vv;
                    t.emax = em;
                    cands.push_back(t);
                }
        int best = -1;
        float best_ms = 1e30f;
        std::vector<vsip_fftm_f *> plans;
        for (size_t c = 0; c < cands.size(); c++) {
            plain_tune_force(&cands[c]);
            // scale 1/N keeps the repeated in-place transforms of the scratch bounded
            vsip_fftm_f *p = cls ? vsip_ccfftmip_create_f(N, cnt, 1.0f / N, VSIP_FFT_FWD, VSIP_COL, 1, VSIP_ALG_TIME)
                                 : vsip_ccfftmip_create_f(cnt, N, 1.0f / N, VSIP_FFT_FWD, VSIP_ROW, 1, VSIP_ALG_TIME);
            plain_tune_force(nullptr);
            if (!p) {
                jvsip_gpu_clear_error();
                continue;
            }
            plans.push_back(p);  // kept until the length is done: its tables serve later candidates
            vsip_ccfftmip_f(p, v);  // warm-up
            cudaEventRecord(e0, d->stream);
            for (int r = 0; r < 3; r++) vsip_ccfftmip_f(p, v);
            cudaEventRecord(e1, d->stream);
            cudaEventSynchronize(e1);
            if (jvsip_gpu_last_error()) {
                jvsip_gpu_clear_error();
                continue;
            }
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            if (ms < best_ms) {
                best_ms = ms;
                best = (int)c;
            }
        }
        for (vsip_fftm_f *p : plans) vsip_fftm_destroy_f(p);
        if (best >= 0) {
            std::lock_guard<std::mutex> lk(g_tune_mu);
            load_cache();
            g_plain[std::make_tuple(N, (int)P_F32, cls)] = cands[best];
            save_plain(N, P_F32, cls, cands[best]);
        }
        if (v) vsip_cmdestroy_f(v);
        vsip_cblockrelease_f(bx, 0, NULL, NULL);
        vsip_cblockdestroy_f(bx);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return rc ? rc : jvsip_gpu_last_error();
}

// The entry the plain-call tuner holds for (N, single precision, cls):
// writes residency, transforms per CTA, values per thread and up to maxr
// radices (out may be NULL); returns the number of passes, 0 when untuned.
int jvsip_fftm_autotune_plain_entry_f(unsigned long N, int cls, int *res, int *vpb, int *emax, int *radices,
                                      int maxr) {
    PlainTune t;
    if (!plain_tuned((long)N, P_F32, cls ? 1 : 0, &t)) return 0;
    if (res) *res = t.res;
    if (vpb) *vpb = t.vpb;
    if (emax) *emax = t.emax;
    for (int i = 0; radices && i < (int)t.radix.size() && i < maxr; i++) radices[i] = t.radix[i];
    return (int)t.radix.size();
}

// Number of (length, precision, stride class) entries the tuner holds.
long jvsip_fftm_autotune_entries(void) { return tuned_entries(); }

}  // extern "C"
