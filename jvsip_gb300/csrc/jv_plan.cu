// jv_plan.cu -- multiple-FFT plans: vsip_{cc,rc,cr}fftm{op,ip}_create_{f,d},
// vsip_fftm_destroy_{f,d}, vsip_fftm_getattr_{f,d}; single-FFT plans:
// vsip_{cc,rc,cr}fft{op,ip}_create_{f,d}, vsip_fft_destroy_{f,d},
// vsip_fft_getattr_{f,d}.
//
// A plan is the reference's plan object (layout of
// c_VSIP_src/vsip_fftmattributes_f.h:8-38, attributes filled with the
// reference's meaning, c_VSIP_src/VI_ccfftmop_create_f_def.h:23-88,
// VI_rcfftmop_create_f_def.h:26-99, VI_crfftmop_create_f_def.h:24-96) whose
// ext_fftm_obj points to the device plan: the pass schedule of the kernels,
// the device twiddle tables (generated in FP64, rounded to the plan's type)
// and, for real transforms, the half-angle table exp(-+ i pi k/MN).
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <functional>
#include <map>
#include <mutex>
#include <new>
#include <set>
#include <string>
#include <tuple>

#include "jv_core.h"

namespace jv {

unsigned long ref_factor(unsigned long N, unsigned long *pn, unsigned long *p0, unsigned long *pF) {
    // c_VSIP_src/VI_nuV.h:22-136: radices in the order 3, 5, 7, 8, 4, 2; the
    // cofactor left after a radix is that stage's final radix.
    static const unsigned long order[6] = {3, 5, 7, 8, 4, 2};
    unsigned long n = N, k = 0;
    if (N == 0) return 0;
    for (int r = 0; r < 6; r++) {
        unsigned long q = order[r], c = 0;
        while (n % q == 0) {
            n /= q;
            c++;
        }
        if (c) {
            p0[k] = q;
            pF[k] = (n != 1) ? n : q;
            pn[k] = (n != 1) ? c + 1 : c;
            k++;
        }
    }
    if (n != 1 && k == 0) {
        p0[0] = 1;
        pF[0] = n;
        pn[0] = 1;
        k = 1;
    }
    return k;
}

static unsigned long ref_jofk(unsigned long k, const unsigned long *pn, const unsigned long *p0,
                              unsigned long pF, unsigned long ns) {
    // c_VSIP_src/VI_jofk.h:21-48
    unsigned long j = 0, m = k;
    for (unsigned long q = 0; q < ns; q++)
        for (unsigned long i = 1; i < pn[q]; i++) {
            unsigned long s = m / p0[q];
            j = p0[q] * j + (m - s * p0[q]);
            m = s;
        }
    unsigned long s = m / pF;
    return pF * j + (m - s * pF);
}

// Exponents of 2, 3, 5, 7 in each radix of kRadixList (same order).
static const int kRadE[kRadices][4] = {{4, 0, 0, 0}, {0, 1, 1, 0}, {1, 0, 0, 1}, {2, 1, 0, 0}, {1, 0, 1, 0},
                                 {0, 2, 0, 0}, {3, 0, 0, 0}, {0, 0, 0, 1}, {1, 1, 0, 0}, {0, 0, 1, 0},
                                 {2, 0, 0, 0}, {0, 1, 0, 0}, {1, 0, 0, 0}};

// Fewest passes for 2^a 3^b 5^c 7^d using radices whose R * pass_k(16, R)
// (points a thread holds in that pass with 16-point registers) is at least
// `need`; ties go to the schedule with the larger radices first.  Returns
// false when no schedule exists.
static bool best_schedule(int a, int b, int c, int d, long need, std::vector<int> &out,
                          std::map<std::tuple<int, int, int, int>, std::vector<int>> &memo,
                          std::map<std::tuple<int, int, int, int>, bool> &ok) {
    auto key = std::make_tuple(a, b, c, d);
    auto it = ok.find(key);
    if (it != ok.end()) {
        if (it->second) out = memo[key];
        return it->second;
    }
    if (a == 0 && b == 0 && c == 0 && d == 0) {
        out.clear();
        ok[key] = true;
        memo[key] = out;
        return true;
    }
    bool found = false;
    std::vector<int> best;
    for (int i = 0; i < kRadices; i++) {
        const int R = kRadixList[i];
        const long K = pass_k(16, R);
        if ((long)R * K < need) continue;
        const int *e = kRadE[i];
        if (e[0] > a || e[1] > b || e[2] > c || e[3] > d) continue;
        std::vector<int> sub;
        if (!best_schedule(a - e[0], b - e[1], c - e[2], d - e[3], need, sub, memo, ok)) continue;
        sub.push_back(R);
        std::sort(sub.begin(), sub.end(), std::greater<int>());
        if (!found || sub.size() < best.size() || (sub.size() == best.size() && sub > best)) {
            best = sub;
            found = true;
        }
    }
    ok[key] = found;
    if (found) memo[key] = best;
    out = best;
    return found;
}

std::vector<int> pass_radices(long N, bool *smooth, long maxt) {
    std::vector<int> r;
    *smooth = true;
    if (N <= 1) return r;
    {
        // 2^a 3^b 5^c 7^d: the searched schedule (every pass fits maxt threads
        // for one transform of N points)
        long n = N;
        int ex[4] = {0, 0, 0, 0};
        const int pr[4] = {2, 3, 5, 7};
        for (int i = 0; i < 4; i++)
            while (n % pr[i] == 0) {
                n /= pr[i];
                ex[i]++;
            }
        if (n == 1) {
            std::map<std::tuple<int, int, int, int>, std::vector<int>> memo;
            std::map<std::tuple<int, int, int, int>, bool> ok;
            const long need = (N + maxt - 1) / maxt;
            if (best_schedule(ex[0], ex[1], ex[2], ex[3], need, r, memo, ok)) return r;
            r.clear();
        }
    }
    long n = N;
    int twos = 0;
    while (n % 2 == 0) {
        n /= 2;
        twos++;
    }
    // powers of two: radix-8 passes, the remainder as one radix-4 or radix-2 pass
    while (twos >= 3) {
        r.push_back(8);
        twos -= 3;
    }
    if (twos == 2) r.push_back(4);
    if (twos == 1) r.push_back(2);
    for (int p : {3, 5, 7}) {
        while (n % p == 0) {
            n /= p;
            r.push_back(p);
        }
    }
    for (long p = 11; n > 1 && p * p <= n; p += 2) {
        while (n % p == 0) {
            n /= p;
            r.push_back((int)p);
            *smooth = false;
        }
    }
    if (n > 1) {
        r.push_back((int)n);
        *smooth = false;
    }
    return r;
}

bool schedule_valid(const std::vector<int> &r, long N, long maxt) {
    if (N < 2 || r.empty()) return false;
    const long need = (N + maxt - 1) / maxt;
    long prod = 1;
    for (size_t i = 0; i < r.size(); i++) {
        const int R = r[i];
        // the shared-memory kernel runs its codelets largest first
        if (i && R > r[i - 1]) return false;
        if (!gpass_codelet_host(R) || (long)R * pass_k(16, R) < need) return false;
        prod *= R;
        if (prod > N) return false;
    }
    return prod == N;
}

// every multiset of usable codelet radices with product N and at most `maxp`
// passes, each as a descending list
static void schedules_rec(long n, int from, long need, int maxp, std::vector<int> &cur,
                          std::vector<std::vector<int>> &out) {
    if (n == 1) {
        out.push_back(cur);
        return;
    }
    if ((int)cur.size() >= maxp) return;
    for (int i = from; i < kRadices; i++) {
        const int R = kRadixList[i];
        if (n % R || (long)R * pass_k(16, R) < need) continue;
        cur.push_back(R);
        schedules_rec(n / R, i, need, maxp, cur, out);
        cur.pop_back();
    }
}

std::vector<std::vector<int>> schedule_candidates(long N, long maxt, size_t limit) {
    std::vector<std::vector<int>> out;
    bool smooth = true;
    std::vector<int> def = pass_radices(N, &smooth, maxt);
    if (!smooth || !schedule_valid(def, N, maxt)) return out;
    out.push_back(def);
    std::vector<std::vector<int>> sets;
    std::vector<int> cur;
    schedules_rec(N, 0, (N + maxt - 1) / maxt, (int)def.size() + 1, cur, sets);
    // fewer passes first; within a pass count larger radices first
    std::stable_sort(sets.begin(), sets.end(), [](const std::vector<int> &a, const std::vector<int> &b) {
        return a.size() != b.size() ? a.size() < b.size() : a > b;
    });
    auto add = [&](const std::vector<int> &c) {
        if (out.size() < limit && std::find(out.begin(), out.end(), c) == out.end()) out.push_back(c);
    };
    for (const std::vector<int> &m : sets) {
        add(m);  // descending: the kernel's codelet order
        if (out.size() >= limit) break;
    }
    return out;
}

// exp(-2 pi i m/N) in double with the angle reduced to [0, pi] by symmetry
static void unit_root(long m, long N, double *c, double *s) {
    bool flip = false;
    if (2 * m > N) {
        m = N - m;
        flip = true;
    }
    double x = (double)m / (double)N;
    double a = 2.0 * 3.14159265358979323846264338327950288 * x;
    *c = cos(a);
    double sn = sin(a);
    *s = flip ? sn : -sn;
}

// Device tables are shared by all plans of one (length, precision, kind):
// a batch of thousands of plans over a few hundred lengths keeps one copy.
struct TableSet {
    void *tw = nullptr, *thalf = nullptr, *twp = nullptr, *twg = nullptr, *pc = nullptr;
    int refs = 0;
};
static std::mutex g_tab_mu;
static std::map<std::tuple<long, int, int, std::string>, TableSet> g_tabs;

// the per-pass tables depend on the pass schedule: plans of one length with
// different (tuned) schedules keep separate tables
static std::string sched_key(const std::vector<int> &r) {
    std::string k;
    for (int R : r) k += std::to_string(R) + ",";
    return k;
}

static int table_kind(int type) { return type == JV_RCFFTOP ? 1 : type == JV_CRFFTOP ? 2 : 0; }

template <typename T>
static bool build_tables(Plan *p);

template <typename T>
static bool make_tables(Plan *p) {
    auto key = std::make_tuple(p->MN, p->prec, table_kind(p->type), sched_key(p->radix));
    std::lock_guard<std::mutex> lk(g_tab_mu);
    auto it = g_tabs.find(key);
    if (it != g_tabs.end()) {
        it->second.refs++;
        p->d_tw = it->second.tw;
        p->d_thalf = it->second.thalf;
        p->d_twp = it->second.twp;
        p->d_twg = it->second.twg;
        p->d_pc = it->second.pc;
        return true;
    }
    if (!build_tables<T>(p)) return false;
    TableSet ts;
    ts.tw = p->d_tw;
    ts.thalf = p->d_thalf;
    ts.twp = p->d_twp;
    ts.twg = p->d_twg;
    ts.pc = p->d_pc;
    ts.refs = 1;
    g_tabs[key] = ts;
    return true;
}

static void release_tables(Plan *p) {
    std::lock_guard<std::mutex> lk(g_tab_mu);
    auto key = std::make_tuple(p->MN, p->prec, table_kind(p->type), sched_key(p->radix));
    auto it = g_tabs.find(key);
    if (it != g_tabs.end() && it->second.tw == p->d_tw) {
        if (--it->second.refs > 0) return;
        g_tabs.erase(it);
    }
    dfree(p->d_tw);
    dfree(p->d_thalf);
    dfree(p->d_twp);
    dfree(p->d_twg);
    dfree(p->d_pc);
}

template <typename T>
static bool build_tables(Plan *p) {
    long MN = p->MN;
    size_t n = (size_t)(MN > 0 ? MN : 1);
    std::vector<T> tw(2 * n, (T)0);
    for (long m = 0; m < MN; m++) {
        double c, s;
        unit_root(m, MN, &c, &s);
        tw[2 * m] = (T)c;
        tw[2 * m + 1] = (T)s;
    }
    Device *d = device();
    if (!d) return false;
    p->d_tw = dmalloc(2 * n * sizeof(T));
    if (!p->d_tw) return false;
    if (!cuda_ok(cudaMemcpy(p->d_tw, tw.data(), 2 * n * sizeof(T), cudaMemcpyHostToDevice), "twiddle upload"))
        return false;
    // per-pass tables: the pass with radix R after radices of product Ns holds
    // exp(-2 pi i r m/(Ns R)) at r*Ns + m
    auto pass_tables = [&](const std::vector<int> &radices, void **dst) -> bool {
        std::vector<T> tp;
        long Ns = 1;
        for (int R : radices) {
            for (long r = 0; r < R; r++)
                for (long m = 0; m < Ns; m++) {
                    double c, s;
                    unit_root((r * m) % (Ns * R), Ns * R, &c, &s);
                    tp.push_back((T)c);
                    tp.push_back((T)s);
                }
            Ns *= R;
        }
        if (tp.empty()) tp.assign(2, (T)0);
        *dst = dmalloc(tp.size() * sizeof(T));
        if (!*dst) return false;
        return cuda_ok(cudaMemcpy(*dst, tp.data(), tp.size() * sizeof(T), cudaMemcpyHostToDevice),
                       "pass twiddle upload");
    };
    if (p->smooth && !pass_tables(p->radix, &p->d_twg)) return false;
    if (p->smooth) {
        std::vector<PassConst> pc(std::max<size_t>(1, p->radix.size()));
        unsigned long Ns = 1;
        for (size_t i = 0; i < p->radix.size(); i++) {
            const unsigned long NR = (unsigned long)MN / (unsigned long)p->radix[i];
            pc[i].NR = (unsigned)NR;
            pc[i].mNR = magic_host(NR);
            pc[i].Ns = (unsigned)Ns;
            pc[i].mNs = magic_host(Ns);
            Ns *= (unsigned long)p->radix[i];
        }
        p->d_pc = dmalloc(pc.size() * sizeof(PassConst));
        if (!p->d_pc) return false;
        if (!cuda_ok(cudaMemcpy(p->d_pc, pc.data(), pc.size() * sizeof(PassConst), cudaMemcpyHostToDevice),
                     "pass constants upload"))
            return false;
    }
    if (sizeof(T) == 4) {
        std::vector<int> fr = fast_radices(MN);
        if (!fr.empty() && !pass_tables(fr, &p->d_twp)) return false;
    }
    if (p->type == JV_RCFFTOP || p->type == JV_CRFFTOP) {
        // exp(-i pi k/MN) for R2C, exp(+i pi k/MN) for C2R, k = 0..MN
        // (c_VSIP_src/VI_rcfftmop_create_f_def.h:75-86, VI_crfftmop_create_f_def.h:72-83)
        std::vector<T> th(2 * (n + 1));
        for (long k = 0; k <= MN; k++) {
            double c, s;
            unit_root(k, 2 * MN, &c, &s);  // exp(-i pi k/MN)
            th[2 * k] = (T)c;
            th[2 * k + 1] = (T)((p->type == JV_RCFFTOP) ? s : -s);
        }
        p->d_thalf = dmalloc(2 * (n + 1) * sizeof(T));
        if (!p->d_thalf) return false;
        if (!cuda_ok(cudaMemcpy(p->d_thalf, th.data(), 2 * (n + 1) * sizeof(T), cudaMemcpyHostToDevice),
                     "half-angle table upload"))
            return false;
    }
    return true;
}

// ---------------------------------------------------------------- long transforms
static void long_free(LongPlan *lp) {
    if (!lp) return;
    for (Plan *q : {lp->p1, lp->p2})
        if (q) {
            release_tables(q);
            delete q;
        }
    for (Plan *q : lp->sp_plans)
        if (q) {
            release_tables(q);
            delete q;
        }
    dfree(lp->d_lo);
    dfree(lp->d_hi);
    dfree(lp->scratch);
    delete lp;
}

// A c2c plan of n points for one step of a long transform (tables from the
// shared cache); nullptr when n has no codelet schedule.
template <typename T>
static Plan *step_plan(long n, int prec) {
    Plan *q = new (std::nothrow) Plan();
    if (!q) return nullptr;
    q->type = JV_CCFFTOP;
    q->prec = prec;
    q->M = 1;
    q->N = q->MN = n;
    q->mN = 1;
    q->radix = pass_radices(n, &q->smooth, prec == P_F32 ? 1024 : 512);
    if (!q->smooth || q->radix.empty() || !make_tables<T>(q)) {
        if (q->smooth && !q->radix.empty()) {
            dfree(q->d_tw);
            dfree(q->d_thalf);
            dfree(q->d_twp);
            dfree(q->d_twg);
            dfree(q->d_pc);
        }
        delete q;
        return nullptr;
    }
    return q;
}

// The two-step decomposition N = N1 * N2 of a length longer than one CTA
// takes: N1 <= N2 as close to sqrt(N) as the codelet schedules allow, both
// within the shared-memory kernel.  Leaves p->lp null (the multi-pass global
// path) when there is none.  Returns false only on allocation failure.
template <typename T>
static bool build_long(Plan *p) {
    const long N = p->MN;
    const long lim = smem_max_len(p->prec, K_C2C);
    // lengths one CTA takes get the decomposition too when the plan has few
    // transforms (one CTA per transform would leave most SMs idle), and
    // single-precision c2c column plans from kColStepsMin points that the
    // register-resident column tiles do not take (their adjacent columns run
    // as two steps, faster than the shared-memory kernel's column tiles)
    const bool few = p->mN * 2 < (long)device()->sms && N >= kLongFewMin;
    const bool cols = p->major == 1 && p->prec == P_F32 && (p->type == JV_CCFFTOP || p->type == JV_CCFFTIP) &&
                      N >= kColStepsMin && !fast_step_len(N);
    if ((N <= lim && !few && !cols) || N >= (1L << 31)) return true;
    const long maxt = p->prec == P_F32 ? 1024 : 512;
    long best = 0;
    for (long d = 2; d * d <= N; d++) {
        if (N % d) continue;
        const long e = N / d;
        if (d > lim || e > lim) continue;
        bool s1 = false, s2 = false;
        pass_radices(d, &s1, maxt);
        pass_radices(e, &s2, maxt);
        if (s1 && s2) best = d;
    }
    if (!best) return true;
    LongPlan *lp = new (std::nothrow) LongPlan();
    if (!lp) return false;
    lp->N1 = best;
    lp->N2 = N / best;
    lp->p1 = step_plan<T>(lp->N1, p->prec);
    lp->p2 = step_plan<T>(lp->N2, p->prec);
    if (!lp->p1 || !lp->p2) {
        long_free(lp);
        return !jvsip_gpu_last_error();
    }
    // W_N^m = lo[m mod L] * hi[m / L], L = 2^sh about sqrt(N)
    unsigned bits = 0;
    while ((1L << bits) < N) bits++;
    lp->sh = (bits + 1) / 2;
    const long L = 1L << lp->sh, H = (N + L - 1) / L;
    lp->mask = (unsigned)(L - 1);
    std::vector<T> lo(2 * L), hi(2 * H);
    for (long r = 0; r < L; r++) {
        double c, s;
        unit_root(r % N, N, &c, &s);
        lo[2 * r] = (T)c;
        lo[2 * r + 1] = (T)s;
    }
    for (long q = 0; q < H; q++) {
        double c, s;
        unit_root((q * L) % N, N, &c, &s);
        hi[2 * q] = (T)c;
        hi[2 * q + 1] = (T)s;
    }
    lp->d_lo = dmalloc(lo.size() * sizeof(T));
    lp->d_hi = dmalloc(hi.size() * sizeof(T));
    if (!lp->d_lo || !lp->d_hi ||
        !cuda_ok(cudaMemcpy(lp->d_lo, lo.data(), lo.size() * sizeof(T), cudaMemcpyHostToDevice), "twiddle upload") ||
        !cuda_ok(cudaMemcpy(lp->d_hi, hi.data(), hi.size() * sizeof(T), cudaMemcpyHostToDevice), "twiddle upload")) {
        long_free(lp);
        return false;
    }
    // single vectors of 2^n points, n >= 13 (single precision): large-radix
    // Stockham passes of 2^6..2^12 points each, larger first -- two up to
    // 2^23 points (fewer launches for short vectors), else ceil(n/9)
    if (p->prec == P_F32 && (N & (N - 1)) == 0 && bits >= 13 && bits <= 31) {
        const unsigned k = bits <= 23 ? 2 : (bits + 8) / 9;
        std::vector<long> rad;
        for (unsigned i = 0; i < k; i++) rad.push_back(1L << (bits / k + (i < bits % k ? 1 : 0)));
        bool ok = true;
        for (long R : rad) ok = ok && R >= 64 && R <= 4096;
        for (size_t i = 0; ok && i < rad.size(); i++) {
            Plan *q = step_plan<T>(rad[i], p->prec);
            if (!q || !q->d_twp) {
                if (q) {
                    release_tables(q);
                    delete q;
                }
                ok = false;
                break;
            }
            lp->sp_plans.push_back(q);
        }
        if (ok) lp->sp_radix = rad;
        else {
            for (Plan *q : lp->sp_plans) {
                release_tables(q);
                delete q;
            }
            lp->sp_plans.clear();
            jvsip_gpu_clear_error();
        }
    }
    p->lp = lp;
    return true;
}

static void plan_free(Plan *p) {
    if (!p) return;
    Device *d = device();
    if (d) cudaStreamSynchronize(d->stream);
    for (CallGraph &g : p->graphs)
        if (g.exec) cudaGraphExecDestroy(g.exec);
    long_free(p->lp);
    release_tables(p);
    dfree(p->d_twdd);
    delete p;
}

Plan *plan_of(const void *vp) {
    if (!vp) return nullptr;
    // both precisions share the layout up to ext_fftm_obj
    const vsip_fftm_f *f = (const vsip_fftm_f *)vp;
    Plan *p = (Plan *)f->ext_fftm_obj;
    return (p && !p->single) ? p : nullptr;
}

// Addresses of the live single-FFT plan objects, so the introspection calls
// that take either kind of plan (as const void *) can tell them apart.
static std::mutex g_single_mu;
static std::set<const void *> g_single;

static bool is_single(const void *vp) {
    std::lock_guard<std::mutex> lk(g_single_mu);
    return g_single.count(vp) != 0;
}

Plan *plan_of_v(const void *vp) {
    if (!vp) return nullptr;
    // both precisions share the layout up to ext_fft_obj
    const vsip_fft_f *f = (const vsip_fft_f *)vp;
    Plan *p = (Plan *)f->ext_fft_obj;
    return (p && p->single) ? p : nullptr;
}

// Radices above 7 that are not codelets are primes taken as a direct sum of
// R multiply-adds per output point.  A plan whose direct sums would keep the
// GPU busy for seconds per call (a long prime length, the reference's
// O(L^2) VI_dftm_f case, c_VSIP_src/VI_fftm_building_blocks_f.h:95-155) is
// refused at creation: at most 2^38 complex multiply-adds per call in single
// precision and 2^35 in double (FP64 runs at a small fraction of FP32 here).
constexpr double kDirectSumMaxF = 274877906944.0;  // 2^38
constexpr double kDirectSumMaxD = 34359738368.0;   // 2^35

static bool direct_sum_ok(const Plan *p) {
    double per_point = 0;
    for (int R : p->radix)
        if (R > 7 && !gpass_codelet_host(R)) per_point += (double)R;
    const double work = per_point * (double)p->MN * (double)p->mN;
    const double lim = p->prec == P_F32 ? kDirectSumMaxF : kDirectSumMaxD;
    if (work > lim) {
        char msg[256];
        snprintf(msg, sizeof msg,
                 "plan refused: lengths with large prime factors are direct sums; this plan needs %.3g complex "
                 "multiply-adds per call, above the limit %.3g (%s)",
                 work, lim, p->prec == P_F32 ? "single precision" : "double precision");
        set_error(E_UNSUPPORTED, msg);
        return false;
    }
    return true;
}

// The device plan of M x N transforms (a single FFT is M = 1, VSIP_ROW);
// *ns and *dft receive the reference's factor count and DFT flag.  Returns
// nullptr (error recorded, nothing left allocated) on failure.
template <typename T>
static Plan *new_plan(int type, vsip_length M, vsip_length N, double scale, int dir, vsip_major major,
                      unsigned ntimes, vsip_alg_hint hint, unsigned long *ns_out, int *dft_out) {
    Plan *p = new (std::nothrow) Plan();
    if (!p) {
        set_error(E_ALLOC, "plan allocation");
        return nullptr;
    }
    p->type = type;
    p->prec = sizeof(T) == 4 ? P_F32 : P_F64;
    p->M = (long)M;
    p->N = (long)N;
    p->major = (major == VSIP_COL) ? 1 : 0;
    if (type == JV_RCFFTOP || type == JV_CRFFTOP) {
        p->MN = (long)(p->major == 0 ? N / 2 : M / 2);
        p->mN = (long)(p->major == 0 ? M : N);
        p->dir = (type == JV_RCFFTOP) ? -1 : 1;
    } else {
        p->MN = (long)(p->major == 1 ? M : N);
        p->mN = (long)(p->major == 1 ? N : M);
        p->dir = dir;
    }
    p->scale = scale;
    p->no_fast = getenv("JVSIP_GPU_NO_FAST") != nullptr;
    p->no_pipeline = getenv("JVSIP_GPU_NO_PIPELINE") != nullptr;
    {
        const char *t = getenv("JVSIP_GPU_TMA_COLUMNS");
        p->tma_columns = t ? (atoi(t) != 0 ? 1 : 0) : -1;
    }
    p->ntimes = ntimes;
    p->hint = (int)hint;
    const long maxt = p->prec == P_F32 ? 1024 : 512;
    p->radix = pass_radices(p->MN, &p->smooth, maxt);
    {
        // the autotuner's choice for this length, precision and stride class
        PlainTune t;
        if ((type == JV_CCFFTOP || type == JV_CCFFTIP) && p->smooth &&
            plain_tuned(p->MN, p->prec, p->major, &t)) {
            if (schedule_valid(t.radix, p->MN, maxt)) p->radix = t.radix;
            if (t.res == 1) p->no_fast = true;
            p->tuned_vpb = t.vpb;
            p->tuned_emax = t.emax;
            p->tuned = true;
        }
    }
    if (!direct_sum_ok(p)) {
        delete p;
        return nullptr;
    }
    if (!device()) {
        delete p;
        return nullptr;
    }
    unsigned long pn[8], p0[8], pF[8];
    unsigned long ns = ref_factor((unsigned long)p->MN, pn, p0, pF);
    if (ns > 0) {
        p->jofk.resize(p->MN);
        for (long i = 0; i < p->MN; i++) p->jofk[i] = ref_jofk((unsigned long)i, pn, p0, pF[ns - 1], ns);
    }
    if (!make_tables<T>(p)) {
        dfree(p->d_tw);
        dfree(p->d_thalf);
        dfree(p->d_twp);
        dfree(p->d_twg);
        dfree(p->d_pc);
        delete p;
        return nullptr;
    }
    if (!build_long<T>(p)) {
        release_tables(p);
        delete p;
        return nullptr;
    }
    *ns_out = ns;
    *dft_out = (ns > 0 && p0[0] == 1 && pF[0] == (unsigned long)p->MN) ? 1 : 0;
    return p;
}

template <typename VP, typename T>
static VP *create(int type, vsip_length M, vsip_length N, double scale, int dir, vsip_major major,
                  unsigned ntimes, vsip_alg_hint hint) {
    VP *vp = (VP *)calloc(1, sizeof(VP));
    if (!vp) {
        set_error(E_ALLOC, "plan allocation");
        return NULL;
    }
    unsigned long ns = 0;
    int dft = 0;
    Plan *p = new_plan<T>(type, M, N, scale, dir, major, ntimes, hint, &ns, &dft);
    if (!p) {
        free(vp);
        return NULL;
    }
    // attributes with the reference's meaning (c_VSIP_src/vsip_fftmattributes_f.h)
    vp->scale = (T)scale;
    vp->N = N;
    vp->M = M;
    vp->MN = (vsip_length)p->MN;
    vp->mN = (vsip_length)p->mN;
    vp->major = major;
    vp->length = ns;
    vp->d = (vsip_fft_dir)p->dir;
    vp->type = type;
    vp->dft = dft;
    vp->ntimes = ntimes;
    vp->hint = hint;
    vp->ext_fftm_obj = p;
    return vp;
}

// A single-FFT plan (c_VSIP_src/vsip_fftattributes_f.h:8-31): the device plan
// of one row of N points.  fft->N is the transform length, the half length for
// rcfftop / crfftop (c_VSIP_src/VI_rcfftop_create_f_def.h:35,
// VI_crfftop_create_f_def.h:32); the reference's work arrays are not needed.
template <typename FP, typename T>
static FP *create_v(int type, vsip_length N, double scale, int dir, unsigned ntimes, vsip_alg_hint hint) {
    FP *fp = (FP *)calloc(1, sizeof(FP));
    if (!fp) {
        set_error(E_ALLOC, "plan allocation");
        return NULL;
    }
    unsigned long ns = 0;
    int dft = 0;
    Plan *p = new_plan<T>(type, 1, N, scale, dir, VSIP_ROW, ntimes, hint, &ns, &dft);
    if (!p) {
        free(fp);
        return NULL;
    }
    p->single = true;
    fp->scale = (T)scale;
    fp->N = (vsip_length)p->MN;
    fp->length = ns;
    fp->d = (vsip_fft_dir)p->dir;
    fp->type = type;
    fp->dft = dft;
    fp->ntimes = ntimes;
    fp->hint = hint;
    fp->stage = 0;
    fp->ext_fft_obj = p;
    {
        std::lock_guard<std::mutex> lk(g_single_mu);
        g_single.insert(fp);
    }
    return fp;
}

template <typename VP>
static int destroy(VP *vp) {
    if (vp) {
        plan_free((Plan *)vp->ext_fftm_obj);
        free(vp);
    }
    return 0;
}

template <typename FP>
static int destroy_v(FP *fp) {
    if (fp) {
        {
            std::lock_guard<std::mutex> lk(g_single_mu);
            g_single.erase(fp);
        }
        plan_free((Plan *)fp->ext_fft_obj);
        free(fp);
    }
    return 0;
}

template <typename FP, typename A>
static void getattr_v(const FP *fft, A *attr) {
    // c_VSIP_src/vsip_fft_getattr_f.c:18-57: lengths of the input and output
    // vectors (real lengths 2N for rcfftop / crfftop, N + 1 for the half spectrum)
    if (!fft || !attr) return;
    attr->input = fft->N;
    attr->output = fft->N;
    attr->place = VSIP_FFT_OP;
    switch (fft->type) {
        case JV_CCFFTIP: attr->place = VSIP_FFT_IP; break;
        case JV_RCFFTOP:
            attr->input = fft->N * 2;
            attr->output = fft->N + 1;
            break;
        case JV_CRFFTOP:
            attr->input = fft->N + 1;
            attr->output = fft->N * 2;
            break;
        default: break;
    }
    attr->dir = fft->d;
    attr->scale = fft->scale;
}

template <typename VP, typename A>
static void getattr(const VP *fft, A *attr) {
    // c_VSIP_src/vsip_fftm_getattr_f.c:18-69
    if (!fft || !attr) return;
    attr->input.r = fft->M;
    attr->input.c = fft->N;
    attr->output.r = fft->M;
    attr->output.c = fft->N;
    attr->place = VSIP_FFT_OP;
    switch (fft->type) {
        case JV_CCFFTIP: attr->place = VSIP_FFT_IP; break;
        case JV_RCFFTOP:
            attr->output.r = (fft->major == VSIP_ROW) ? fft->mN : (fft->MN + 1);
            attr->output.c = (fft->major == VSIP_ROW) ? (fft->MN + 1) : fft->mN;
            break;
        case JV_CRFFTOP:
            attr->input.r = (fft->major == VSIP_ROW) ? fft->mN : (fft->MN + 1);
            attr->input.c = (fft->major == VSIP_ROW) ? (fft->MN + 1) : fft->mN;
            break;
        default: break;
    }
    attr->dir = fft->d;
    attr->scale = fft->scale;
    attr->major = fft->major;
}

}  // namespace jv

using namespace jv;

extern "C" {

vsip_fftm_f *vsip_ccfftmop_create_f(vsip_length M, vsip_length N, vsip_scalar_f scale, vsip_fft_dir dir,
                                    vsip_major major, unsigned int ntimes, vsip_alg_hint hint) {
    return create<vsip_fftm_f, float>(JV_CCFFTOP, M, N, scale, dir, major, ntimes, hint);
}
vsip_fftm_f *vsip_ccfftmip_create_f(vsip_length M, vsip_length N, vsip_scalar_f scale, vsip_fft_dir dir,
                                    vsip_major major, unsigned int ntimes, vsip_alg_hint hint) {
    return create<vsip_fftm_f, float>(JV_CCFFTIP, M, N, scale, dir, major, ntimes, hint);
}
vsip_fftm_f *vsip_rcfftmop_create_f(vsip_length M, vsip_length N, vsip_scalar_f scale, vsip_major major,
                                    unsigned int ntimes, vsip_alg_hint hint) {
    return create<vsip_fftm_f, float>(JV_RCFFTOP, M, N, scale, VSIP_FFT_FWD, major, ntimes, hint);
}
vsip_fftm_f *vsip_crfftmop_create_f(vsip_length M, vsip_length N, vsip_scalar_f scale, vsip_major major,
                                    unsigned int ntimes, vsip_alg_hint hint) {
    return create<vsip_fftm_f, float>(JV_CRFFTOP, M, N, scale, VSIP_FFT_INV, major, ntimes, hint);
}
vsip_fftm_d *vsip_ccfftmop_create_d(vsip_length M, vsip_length N, vsip_scalar_d scale, vsip_fft_dir dir,
                                    vsip_major major, unsigned int ntimes, vsip_alg_hint hint) {
    return create<vsip_fftm_d, double>(JV_CCFFTOP, M, N, scale, dir, major, ntimes, hint);
}
vsip_fftm_d *vsip_ccfftmip_create_d(vsip_length M, vsip_length N, vsip_scalar_d scale, vsip_fft_dir dir,
                                    vsip_major major, unsigned int ntimes, vsip_alg_hint hint) {
    return create<vsip_fftm_d, double>(JV_CCFFTIP, M, N, scale, dir, major, ntimes, hint);
}
vsip_fftm_d *vsip_rcfftmop_create_d(vsip_length M, vsip_length N, vsip_scalar_d scale, vsip_major major,
                                    unsigned int ntimes, vsip_alg_hint hint) {
    return create<vsip_fftm_d, double>(JV_RCFFTOP, M, N, scale, VSIP_FFT_FWD, major, ntimes, hint);
}
vsip_fftm_d *vsip_crfftmop_create_d(vsip_length M, vsip_length N, vsip_scalar_d scale, vsip_major major,
                                    unsigned int ntimes, vsip_alg_hint hint) {
    return create<vsip_fftm_d, double>(JV_CRFFTOP, M, N, scale, VSIP_FFT_INV, major, ntimes, hint);
}

vsip_fft_f *vsip_ccfftop_create_f(vsip_length N, vsip_scalar_f scale, vsip_fft_dir dir, unsigned int ntimes,
                                  vsip_alg_hint hint) {
    return create_v<vsip_fft_f, float>(JV_CCFFTOP, N, scale, dir, ntimes, hint);
}
vsip_fft_f *vsip_ccfftip_create_f(vsip_length N, vsip_scalar_f scale, vsip_fft_dir dir, unsigned int ntimes,
                                  vsip_alg_hint hint) {
    return create_v<vsip_fft_f, float>(JV_CCFFTIP, N, scale, dir, ntimes, hint);
}
vsip_fft_f *vsip_rcfftop_create_f(vsip_length N, vsip_scalar_f scale, unsigned int ntimes, vsip_alg_hint hint) {
    return create_v<vsip_fft_f, float>(JV_RCFFTOP, N, scale, VSIP_FFT_FWD, ntimes, hint);
}
vsip_fft_f *vsip_crfftop_create_f(vsip_length N, vsip_scalar_f scale, unsigned int ntimes, vsip_alg_hint hint) {
    return create_v<vsip_fft_f, float>(JV_CRFFTOP, N, scale, VSIP_FFT_INV, ntimes, hint);
}
vsip_fft_d *vsip_ccfftop_create_d(vsip_length N, vsip_scalar_d scale, vsip_fft_dir dir, unsigned int ntimes,
                                  vsip_alg_hint hint) {
    return create_v<vsip_fft_d, double>(JV_CCFFTOP, N, scale, dir, ntimes, hint);
}
vsip_fft_d *vsip_ccfftip_create_d(vsip_length N, vsip_scalar_d scale, vsip_fft_dir dir, unsigned int ntimes,
                                  vsip_alg_hint hint) {
    return create_v<vsip_fft_d, double>(JV_CCFFTIP, N, scale, dir, ntimes, hint);
}
vsip_fft_d *vsip_rcfftop_create_d(vsip_length N, vsip_scalar_d scale, unsigned int ntimes, vsip_alg_hint hint) {
    return create_v<vsip_fft_d, double>(JV_RCFFTOP, N, scale, VSIP_FFT_FWD, ntimes, hint);
}
vsip_fft_d *vsip_crfftop_create_d(vsip_length N, vsip_scalar_d scale, unsigned int ntimes, vsip_alg_hint hint) {
    return create_v<vsip_fft_d, double>(JV_CRFFTOP, N, scale, VSIP_FFT_INV, ntimes, hint);
}
int vsip_fft_destroy_f(vsip_fft_f *p) { return destroy_v(p); }
int vsip_fft_destroy_d(vsip_fft_d *p) { return destroy_v(p); }
void vsip_fft_getattr_f(const vsip_fft_f *p, vsip_fft_attr_f *a) { getattr_v(p, a); }
void vsip_fft_getattr_d(const vsip_fft_d *p, vsip_fft_attr_d *a) { getattr_v(p, a); }

int vsip_fftm_destroy_f(vsip_fftm_f *p) { return destroy(p); }
int vsip_fftm_destroy_d(vsip_fftm_d *p) { return destroy(p); }
void vsip_fftm_getattr_f(const vsip_fftm_f *p, vsip_fftm_attr_f *a) { getattr(p, a); }
void vsip_fftm_getattr_d(const vsip_fftm_d *p, vsip_fftm_attr_d *a) { getattr(p, a); }

int jvsip_fftm_setform_f(vsip_fftm_f *vp, int form) {
    Plan *p = plan_of(vp);
    if (!p || form < JVSIP_FORM_AUTO || form > JVSIP_FORM_SPLIT_FP16) return E_ARG;
    p->form = form;
    return 0;
}
int jvsip_fftm_getform_f(const vsip_fftm_f *vp) {
    Plan *p = plan_of(vp);
    return p ? p->form : -1;
}

// The FP64 form of a c2c _d plan: double-float twiddles of its radix-8/4/2
// schedule, [r][m] per pass as in the single-precision tables.
int jvsip_fftm_setform_d(vsip_fftm_d *vp, int form) {
    Plan *p = plan_of(vp);
    if (!p || (form != JVSIP_FORM_AUTO && form != JVSIP_FORM_PLAIN && form != JVSIP_FORM_DF64)) return E_ARG;
    std::lock_guard<std::mutex> lk(p->mu);
    if (form == JVSIP_FORM_DF64 && !p->d_twdd) {
        const std::vector<int> rad = dd_radices(p->MN);
        if (rad.empty() || (p->type != JV_CCFFTOP && p->type != JV_CCFFTIP)) {
            set_error(E_UNSUPPORTED, "the FP64 form takes c2c plans of 64 to 8192 points (powers of two)");
            return E_UNSUPPORTED;
        }
        std::vector<float> tb;
        long Ns = 1;
        for (int R : rad) {
            for (long r = 0; r < R; r++)
                for (long m = 0; m < Ns; m++) {
                    double c, sn;
                    unit_root((r * m) % (Ns * R), Ns * R, &c, &sn);
                    for (double x : {c, sn}) {
                        const float hi = (float)x;
                        tb.push_back(hi);
                        tb.push_back((float)(x - (double)hi));
                    }
                }
            Ns *= R;
        }
        void *d = dmalloc(tb.size() * sizeof(float));
        if (!d) return E_ALLOC;
        if (!cuda_ok(cudaMemcpy(d, tb.data(), tb.size() * sizeof(float), cudaMemcpyHostToDevice),
                     "FP64-form twiddle upload")) {
            dfree(d);
            return E_CUDA;
        }
        p->d_twdd = d;
    }
    p->form = form;
    return 0;
}
int jvsip_fftm_getform_d(const vsip_fftm_d *vp) {
    Plan *p = plan_of(vp);
    return p ? p->form : -1;
}

// Plan introspection for tests and tools: the device pass radices and the
// reference digit-reversal map.  Returns the count written (or needed).
static Plan *any_plan(const void *vp) { return is_single(vp) ? plan_of_v(vp) : plan_of(vp); }

int jvsip_fftm_passes(const void *vp, int *radix, int cap) {
    Plan *p = any_plan(vp);
    if (!p) return -1;
    int n = (int)p->radix.size();
    for (int i = 0; i < n && i < cap; i++) radix[i] = p->radix[i];
    return n;
}
int jvsip_fftm_graphs(const void *vp) {
    Plan *p = any_plan(vp);
    if (!p) return -1;
    std::lock_guard<std::mutex> lk(p->mu);
    int n = 0;
    for (const CallGraph &g : p->graphs) n += g.exec ? 1 : 0;
    return n;
}
long jvsip_fftm_jofk(const void *vp, unsigned long *out, long cap) {
    Plan *p = any_plan(vp);
    if (!p) return -1;
    long n = (long)p->jofk.size();
    for (long i = 0; i < n && i < cap; i++) out[i] = p->jofk[i];
    return n;
}

}  // extern "C"
