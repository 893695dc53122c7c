// jv_exec.cu -- vsip_ccfftmop/ccfftmip/rcfftmop/crfftmop in _f and _d, and
// the single-FFT calls vsip_ccfftop/ccfftip/rcfftop/crfftop on vector views.
//
// Semantics follow the reference (c_VSIP_src/VI_ccfftmop_f_def.h:20-29,
// VI_ccfftmip_f_def.h:17-23, VI_rcfftmop_f_def.h:24-120,
// VI_crfftmop_f_def.h:25-126): plan.mN transforms of length plan.MN along the
// rows (VSIP_ROW) or columns (VSIP_COL) of the views, y = scale * DFT_dir(x),
// the scale applied only when it is not 1, any signed strides and offsets,
// interleaved or split complex blocks, and x may alias y.
//
// Each view is resolved to device memory: a block admitted through this
// library is used in place in its device mirror; any other block is staged --
// the span of the block the view touches is copied to the device before the
// kernels and (for outputs) back after them, inside the call.
#include <string.h>

#include <algorithm>
#include <vector>

#include "jv_core.h"

namespace jv {

long smem_max_len_f32(int kind);
long smem_max_len_f64(int kind);

long smem_max_len(int prec, int kind) { return prec == P_F32 ? smem_max_len_f32(kind) : smem_max_len_f64(kind); }

static bool run_job(Job &j, cudaStream_t st);

// ---------------------------------------------------------------- staging of host blocks
// One staged region: scalars [lo*cst, (hi+1)*cst) of a host array (and of its
// imaginary array for split blocks) copied to one device buffer.
struct Region {
    const void *key = nullptr;   // block identity
    char *h_re = nullptr, *h_im = nullptr;
    size_t esz = 0;              // bytes per scalar
    long cst = 1;                // scalars per element index step
    long lo = 0, hi = -1;        // element index range
    bool read = false, write = false;
    void *d_re = nullptr, *d_im = nullptr;
};

struct Staging {
    std::vector<Region> regs;
    Region *find(const void *key) {
        for (auto &r : regs)
            if (r.key == key) return &r;
        return nullptr;
    }
    void add(const void *key, char *h_re, char *h_im, size_t esz, long cst, long lo, long hi, bool rd, bool wr) {
        Region *r = find(key);
        if (r) {
            r->lo = std::min(r->lo, lo);
            r->hi = std::max(r->hi, hi);
            r->read = r->read || rd;
            r->write = r->write || wr;
            return;
        }
        Region n;
        n.key = key;
        n.h_re = h_re;
        n.h_im = h_im;
        n.esz = esz;
        n.cst = cst;
        n.lo = lo;
        n.hi = hi;
        n.read = rd;
        n.write = wr;
        regs.push_back(n);
    }
    size_t bytes(const Region &r) const { return (size_t)(r.hi - r.lo + 1) * r.cst * r.esz; }
    bool upload(cudaStream_t st) {
        for (auto &r : regs) {
            size_t b = bytes(r);
            r.d_re = dmalloc(b);
            if (!r.d_re) return false;
            if (r.h_im) {
                r.d_im = dmalloc(b);
                if (!r.d_im) return false;
            }
            if (r.read) {
                size_t o = (size_t)r.lo * r.cst * r.esz;
                if (!cuda_ok(cudaMemcpyAsync(r.d_re, r.h_re + o, b, cudaMemcpyHostToDevice, st), "stage in"))
                    return false;
                if (r.h_im && !cuda_ok(cudaMemcpyAsync(r.d_im, r.h_im + o, b, cudaMemcpyHostToDevice, st), "stage in"))
                    return false;
            }
        }
        return true;
    }
    bool download(cudaStream_t st) {
        bool ok = true;
        for (auto &r : regs) {
            if (!r.write || !r.d_re) continue;
            size_t b = bytes(r), o = (size_t)r.lo * r.cst * r.esz;
            ok = ok && cuda_ok(cudaMemcpyAsync(r.h_re + o, r.d_re, b, cudaMemcpyDeviceToHost, st), "stage out");
            if (r.h_im) ok = ok && cuda_ok(cudaMemcpyAsync(r.h_im + o, r.d_im, b, cudaMemcpyDeviceToHost, st), "stage out");
        }
        return ok;
    }
    ~Staging() {
        for (auto &r : regs) {
            dfree(r.d_re);
            dfree(r.d_im);
        }
    }
};

// ---------------------------------------------------------------- view geometry
struct Geo {
    long off, es, vs, len, nvec;
    long lo() const { return off + std::min(0L, (nvec - 1) * vs) + std::min(0L, (len - 1) * es); }
    long hi() const { return off + std::max(0L, (nvec - 1) * vs) + std::max(0L, (len - 1) * es); }
    // covers its span exactly once (no gaps), so an output needs no copy-in
    bool dense() const {
        long span = hi() - lo() + 1;
        if (span != len * nvec) return false;
        return (labs(es) == 1 && (nvec == 1 || labs(vs) == len)) || (labs(vs) == 1 && (len == 1 || labs(es) == nvec));
    }
};

template <typename CMV>
static Geo cgeo(const CMV *v, int major, long len, long nvec) {
    Geo g;
    g.off = (long)v->offset;
    if (major == 0) {
        g.es = v->row_stride;
        g.vs = v->col_stride;
    } else {
        g.es = v->col_stride;
        g.vs = v->row_stride;
    }
    g.len = len;
    g.nvec = nvec;
    return g;
}

template <typename CMV>
static bool view_ok(const CMV *v, int major, long len, long nvec) {
    if (!v || !v->block) return false;
    long vl = (long)(major == 0 ? v->row_length : v->col_length);
    long vn = (long)(major == 0 ? v->col_length : v->row_length);
    return vl >= len && vn >= nvec;
}

// Resolve a complex view: device mirror in place, or a staged region.
template <typename T, typename CB>
struct CRes {
    const CB *blk;
    Geo g;
    Mirror *m;
};

template <typename T, typename CB>
static void stage_c(Staging &s, const CRes<T, CB> &r, bool rd, bool wr) {
    if (r.m) return;
    const CB *b = r.blk;
    bool split = (b->cstride == 1);
    char *h_re = (char *)b->R->array;
    char *h_im = split ? (char *)b->I->array : nullptr;
    s.add(b, h_re, h_im, sizeof(T), split ? 1 : 2, r.g.lo(), r.g.hi(), rd, wr);
}

template <typename T, typename CB>
static CView dev_c(Staging &s, const CRes<T, CB> &r) {
    CView v;
    v.es = r.g.es;
    v.vs = r.g.vs;
    bool split = (r.blk->cstride == 1);
    v.cst = split ? 1 : 2;
    if (r.m) {
        v.re = r.m->d;
        v.im = split ? r.m->d_im : (void *)((T *)r.m->d + 1);
        v.off = r.g.off;
    } else {
        Region *g = s.find(r.blk);
        v.re = g->d_re;
        v.im = split ? g->d_im : (void *)((T *)g->d_re + 1);
        v.off = r.g.off - g->lo;
    }
    return v;
}

// Real views: the block may be a user/VSIPL real block or the real/imaginary
// part of a complex block (its parent).
template <typename T, typename RB>
struct RRes {
    const RB *blk;
    Geo g;
    void *dbase;  // device address of the block's array (mirrored), else nullptr
    long rst;
};

template <typename T, typename RB>
static RRes<T, RB> resolve_r(const RB *b, const Geo &g) {
    RRes<T, RB> r;
    r.blk = b;
    r.g = g;
    r.dbase = nullptr;
    r.rst = b->rstride > 0 ? b->rstride : 1;
    Mirror *m = mirror_find(b);
    if (m) {
        r.dbase = m->d;
    } else if (b->parent) {
        Mirror *pm = mirror_find(b->parent);
        if (pm) {
            bool split = (b->parent->cstride == 1);
            if (b == b->parent->R) r.dbase = pm->d;
            else r.dbase = split ? pm->d_im : (void *)((T *)pm->d + 1);
        }
    }
    return r;
}

template <typename T, typename RB>
static void stage_r(Staging &s, const RRes<T, RB> &r, bool rd, bool wr) {
    if (r.dbase) return;
    s.add(r.blk, (char *)r.blk->array, nullptr, sizeof(T), r.rst, r.g.lo(), r.g.hi(), rd, wr);
}

template <typename T, typename RB>
static RView dev_r(Staging &s, const RRes<T, RB> &r) {
    RView v;
    v.rst = r.rst;
    v.es = r.g.es;
    v.vs = r.g.vs;
    if (r.dbase) {
        v.a = r.dbase;
        v.off = r.g.off;
    } else {
        Region *g = s.find(r.blk);
        v.a = g->d_re;
        v.off = r.g.off - g->lo;
    }
    return v;
}

static void mark_written(const void *blk) {
    Mirror *m = mirror_find(blk);
    if (m) m->device_newer = true;
}

// ---------------------------------------------------------------- dispatch
// true when the call runs in one of the shared-memory / register kernels (no
// scratch allocation); false for the multi-pass global path
static bool job_in_smem(const Job &j) {
    long lim = smem_max_len(j.prec, j.kind);
    bool smooth = true;
    for (int i = 0; i < j.npass; i++) {
        bool codelet = false;
        for (int r = 0; r < kRadices; r++) codelet = codelet || (j.radix[i] == kRadixList[r]);
        if (!codelet) smooth = false;
    }
    if (!j.twg || !j.pc) smooth = false;
    long need = j.N + (j.kind == K_C2R ? 1 : 0);
    return smooth && need <= lim;
}

// The two steps of a long c2c transform (LongPlan): interleaved views only;
// returns false with *handled unset when the views do not qualify.
static bool interleaved(const CView &v, size_t esz) {
    return v.cst == 2 && (const char *)v.im == (const char *)v.re + esz && ((uintptr_t)v.re % (2 * esz)) == 0;
}

static bool step_job(Job &q, const Job &j, const Plan *sp) {
    q.kind = K_C2C;
    q.prec = j.prec;
    q.N = sp->MN;
    q.tw = sp->d_tw;
    q.twg = sp->d_twg;
    q.pc = sp->d_pc;
    q.twp = sp->d_twp;
    q.thalf = nullptr;
    q.form = 0;
    q.no_fast = true;
    q.tma_columns = j.tma_columns;
    q.npass = (int)sp->radix.size();
    if (q.npass > 40) return false;
    for (int i = 0; i < q.npass; i++) q.radix[i] = sp->radix[i];
    q.inplace = 0;
    q.lp = nullptr;
    return true;
}

// The two steps of one c2c transform family: N-point transforms of the view
// `in` (nv of them) into the view `out`; conj_in / conj_out / scale as given.
static bool two_steps(const Job &j, LongPlan *lp, const CView &in, const CView &out, long nv, int conj_in,
                      int conj_out, int has_scale, double scale, char *sc, size_t esz, cudaStream_t st) {
    const long N = j.N, N1 = lp->N1, N2 = lp->N2;
    CView scv;
    scv.re = sc;
    scv.im = sc + esz;
    scv.cst = 2;
    scv.off = 0;
    // transforms of a vector far apart in memory ("rows": |vs| != 1 or one
    // vector): groups are the vectors, transforms inside a group are n1 (step
    // A) / k2 (step B).  Adjacent vectors ("columns", |vs| == 1): groups are
    // n1 / k2 and the transforms inside a group are the vectors, adjacent in
    // memory; the scratch then holds [n1][k2][v].
    const bool cols = nv > 1 && (in.vs == 1 || in.vs == -1);
    Job a = j, b = j;
    a.nvec = b.nvec = nv;
    if (!step_job(a, j, lp->p2) || !step_job(b, j, lp->p1)) return false;
    // step A: transform over n2 (N2 points, element n1 + N1*n2 of x).  With
    // equal conjugations (c2c, R2C) each step conjugates on its own load and
    // store -- an inverse transform of its own, the twiddle applied in the
    // conjugated domain; otherwise (C2R: forward transform of conjugated data,
    // conjugated at the end) step A conjugates the load and step B the store.
    const bool same = conj_in == conj_out;
    a.cin = in;
    a.cout = scv;
    a.conj_in = conj_in;
    a.conj_out = same ? conj_in : 0;
    if (same) a.inv = b.inv = conj_in;
    a.has_scale = 0;
    a.scale = 1.0;
    a.tw_lo = lp->d_lo;
    a.tw_hi = lp->d_hi;
    a.tw_mask = lp->mask;
    a.tw_sh = lp->sh;
    // step B: transform over n1 (N1 points) of the scratch, k1 to y[k2 + N2*k1]
    b.cin = scv;
    b.cout = out;
    b.conj_in = same ? conj_out : 0;
    b.conj_out = conj_out;
    b.has_scale = has_scale;
    b.scale = scale;
    if (!cols) {
        a.nvec = N1;
        a.nbatch = nv;
        a.cin.es = in.es * N1;
        a.cin.vs = in.es;
        a.bvs_in = in.vs;
        a.cout.es = 1;
        a.cout.vs = N2;
        a.bvs_out = N;
        a.tw_ts = 1;
        a.tw_ys = 0;
        b.nvec = N2;
        b.nbatch = nv;
        b.cin.es = N2;
        b.cin.vs = 1;
        b.bvs_in = N;
        b.cout.es = out.es * N2;
        b.cout.vs = out.es;
        b.bvs_out = out.vs;
    } else {
        a.nvec = nv;
        a.nbatch = N1;
        a.cin.es = in.es * N1;
        a.cin.vs = in.vs;
        a.bvs_in = in.es;
        a.cout.es = nv;
        a.cout.vs = 1;
        a.bvs_out = N2 * nv;
        a.tw_ts = 0;
        a.tw_ys = 1;
        b.nvec = nv;
        b.nbatch = N2;
        b.cin.es = N2 * nv;
        b.cin.vs = 1;
        b.bvs_in = nv;
        b.cout.es = out.es * N2;
        b.cout.vs = out.vs;
        b.bvs_out = out.es;
    }
    if (j.prec == P_F32) {
        // steps of lengths the register-resident kernel takes as column tiles
        // (groups along the grid's y)
        const bool fa = launch_fast_step_f32(a, st);
        if (!fa && jvsip_gpu_last_error()) return false;
        if (!fa && !launch_smem_f32(a, st)) return false;
        const bool fb = launch_fast_step_f32(b, st);
        if (!fb && jvsip_gpu_last_error()) return false;
        return fb || launch_smem_f32(b, st);
    }
    return launch_smem_f64(a, st) && launch_smem_f64(b, st);
}

// A single vector of 2^n points (single precision, interleaved, unit stride)
// as large-radix Stockham passes (LongPlan::sp_radix): pass p reads element n
// of transform j at j + n*N/R_p, multiplies it by W_N^(n*m*N/(Ns*R_p)),
// m = j mod Ns, and writes output k at (j - m)*R_p + m + k*Ns, Ns = R_0...R_{p-1};
// the passes alternate between two scratch halves and the last one writes y.
static bool sp_passes(const Job &j, LongPlan *lp, const CView &vin, const CView &vout, int inv, int has_scale,
                      double scale, char *sc, size_t esz, cudaStream_t st) {
    const long N = j.N;
    const int k = (int)lp->sp_radix.size();
    const size_t one = (size_t)N * 2 * esz;
    unsigned long Ns = 1;
    for (int p = 0; p < k; p++) {
        const long R = lp->sp_radix[p];
        Job q = j;
        q.kind = K_C2C;
        q.N = R;
        q.nvec = N / R;
        q.nbatch = 1;
        q.lp = nullptr;
        q.twp = lp->sp_plans[p]->d_twp;
        q.twg = lp->sp_plans[p]->d_twg;
        q.pc = lp->sp_plans[p]->d_pc;
        q.npass = 0;
        q.tw_lo = lp->d_lo;
        q.tw_hi = lp->d_hi;
        q.tw_mask = lp->mask;
        q.tw_sh = lp->sh;
        q.sp_ns = (unsigned)Ns;
        unsigned lg = 0;
        while ((1UL << lg) < Ns) lg++;
        q.sp_lgns = lg;
        q.sp_twstride = (unsigned)((unsigned long)N / (Ns * (unsigned long)R));
        q.sp_mask = (unsigned)(N - 1);
        q.inv = inv;
        q.has_scale = (p == k - 1) ? has_scale : 0;
        q.scale = scale;
        CView in = vin, out = vout;
        if (p > 0) {
            char *b = sc + (size_t)((p - 1) % 2) * one;
            in.re = b;
            in.im = b + esz;
            in.off = 0;
        }
        if (p < k - 1) {
            char *b = sc + (size_t)(p % 2) * one;
            out.re = b;
            out.im = b + esz;
            out.off = 0;
        }
        in.es = N / R;
        in.vs = 1;
        q.cin = in;
        q.cout = out;
        if (!launch_fast_sp_f32(q, st)) return false;
        Ns *= (unsigned long)R;
    }
    return true;
}

// A real view of unit stride, even offset and pitch, 2-element aligned, as
// the interleaved complex view of its pairs (x_2n + i x_2n+1).
static bool real_as_complex(const RView &r, long nvec, size_t esz, CView *c) {
    if (r.rst != 1 || r.es != 1 || r.off % 2 != 0 || (nvec > 1 && r.vs % 2 != 0) ||
        ((uintptr_t)r.a % (2 * esz)) != 0)
        return false;
    c->re = r.a;
    c->im = (char *)r.a + esz;
    c->cst = 2;
    c->off = r.off / 2;
    c->es = 1;
    c->vs = r.vs / 2;
    return true;
}

// The long-transform path (LongPlan): c2c on interleaved views; R2C from a
// real view of unit stride into an interleaved spectrum (steps into the
// output, then the in-place split); C2R from any spectrum view (un-split into
// scratch, steps into the real output as complex pairs, or into scratch and
// the final store).  Returns with *handled unset when the call does not
// qualify (the multi-pass global path takes it).
// Bytes of scratch a long call needs: its data once for the two steps of a
// c2c call of several vectors, twice otherwise (the single-vector passes and
// C2R use two halves).
static size_t long_scratch_need(const Job &j) {
    const size_t esz = j.prec == P_F32 ? sizeof(float) : sizeof(double);
    const size_t one = (size_t)j.nvec * j.N * 2 * esz;
    return (j.kind == K_C2C && j.nvec > 1) ? one : 2 * one;
}

// The plan's scratch of at least `need` bytes (held by the plan: a captured
// call replays into it).  quiet: a failed allocation records no error (the
// caller has another path).
static bool long_scratch(LongPlan *lp, size_t need, bool quiet) {
    if (lp->scratch_bytes >= need) return true;
    const int err0 = jvsip_gpu_last_error();
    dfree(lp->scratch);
    lp->scratch = dmalloc(need);
    lp->scratch_bytes = lp->scratch ? need : 0;
    if (lp->scratch) return true;
    if (quiet) {
        if (err0 == 0 && jvsip_gpu_last_error() != 0) jvsip_gpu_clear_error();
    } else if (!jvsip_gpu_last_error()) {
        set_error(E_ALLOC, "scratch of a long transform");
    }
    return false;
}

// few transforms of a length with a decomposition: two steps over many CTAs
// instead of one CTA per transform
static bool long_few(const Job &j) {
    return j.lp && j.nvec * 2 < (long)device()->sms && j.N >= kLongFewMin;
}
// single-precision c2c columns (adjacent vectors on both sides) of a length
// with a decomposition from kColStepsMin points, not taken by the
// register-resident column tiles: two steps whatever their count.  Measured
// against the shared-memory kernel's column tiles: 16384 x 1024: 3001 against
// 1013 GB/s (1799 before the steps ran on the register-resident column tiles);
// 10000 x 1024: 1840 against 917; 8192 x 2048: 2980 against 1436; 7000 x 512:
// 1319 against 782; 3000 x 1024: 1164 against 874 (and slower than the
// register-resident tiles themselves: 4096 x 1024: 1457 against 2283).
static bool long_columns(const Job &j) {
    return j.lp && j.kind == K_C2C && j.prec == P_F32 && j.nvec > 1 && j.N >= kColStepsMin && !fast_step_len(j.N) &&
           labs(j.cin.vs) == 1 && labs(j.cout.vs) == 1;
}

static bool run_long(Job &j, cudaStream_t st, bool *handled) {
    *handled = false;
    LongPlan *lp = j.lp;
    const size_t esz = j.prec == P_F32 ? sizeof(float) : sizeof(double);
    if (!lp) return false;
    CView zin;
    if (j.kind == K_C2C && !(interleaved(j.cin, esz) && interleaved(j.cout, esz))) return false;
    if (j.kind == K_R2C && !(interleaved(j.cout, esz) && real_as_complex(j.rin, j.nvec, esz, &zin))) return false;
    const long N = j.N, nv = j.nvec;
    const size_t one = (size_t)nv * N * 2 * esz;
    // single vectors of unit stride take the Stockham passes when planned:
    // c2c, and R2C (the half-length transform of the pairs, then the split)
    // when it has three passes or more (measured: R2C of 2^24 points 892 GB/s
    // in the two steps, 815 in two passes; 2^26 points 715 against 891)
    const bool sp = !lp->sp_radix.empty() && nv == 1 && j.prec == P_F32 && j.cout.es == 1 &&
                    ((j.kind == K_C2C && j.cin.es == 1) || (j.kind == K_R2C && lp->sp_radix.size() >= 3));
    // the plan's call shape is fixed, so the scratch is sized once: a captured
    // call's graph holds its address, and it is never reallocated while the
    // plan lives
    *handled = true;
    if (!long_scratch(lp, long_scratch_need(j), false)) return false;
    char *sc = (char *)lp->scratch;
    if (sp && j.kind == K_C2C) return sp_passes(j, lp, j.cin, j.cout, j.inv, j.has_scale, j.scale, sc, esz, st);
    if (j.kind == K_C2C)
        return two_steps(j, lp, j.cin, j.cout, nv, j.inv, j.inv, j.has_scale, j.scale, sc, esz, st);
    if (j.kind == K_R2C) {
        // Z = F(z) into the first N elements of each output vector, then the split
        const bool ok = sp ? sp_passes(j, lp, zin, j.cout, 0, 0, 1.0, sc, esz, st)
                           : two_steps(j, lp, zin, j.cout, nv, 0, 0, 0, 1.0, sc, esz, st);
        if (!ok) return false;
        void *z = (char *)j.cout.re + (size_t)j.cout.off * 2 * esz;
        return j.prec == P_F32
                   ? launch_r2c_pairs_f32(z, j.cout.es, j.cout.vs, N, nv, j.has_scale, j.scale, j.thalf, st)
                   : launch_r2c_pairs_f64(z, j.cout.es, j.cout.vs, N, nv, j.has_scale, j.scale, j.thalf, st);
    }
    // C2R: conj(Y) dense in the second half of the scratch, the steps, conj back
    char *ys = sc + one;
    CView yv;
    yv.re = ys;
    yv.im = ys + esz;
    yv.cst = 2;
    yv.off = 0;
    yv.es = 1;
    yv.vs = N;
    bool ok = j.prec == P_F32 ? launch_c2r_unsplit_f32(j, ys, st) : launch_c2r_unsplit_f64(j, ys, st);
    if (!ok) return false;
    CView xo;
    if (real_as_complex(j.rout, nv, esz, &xo))
        return two_steps(j, lp, yv, xo, nv, 0, 1, j.has_scale, j.scale, sc, esz, st);
    // other real views: the steps back into the second half, then the final store
    if (!two_steps(j, lp, yv, yv, nv, 0, 0, 0, 1.0, sc, esz, st)) return false;
    return j.prec == P_F32 ? launch_c2r_unpack_f32(j, ys, st) : launch_c2r_unpack_f64(j, ys, st);
}

static bool run_job(Job &j, cudaStream_t st) {
    if (j.nvec <= 0 || j.N <= 0) return true;
    if (j.form == JVSIP_FORM_SPLIT_BF16 || j.form == JVSIP_FORM_SPLIT_FP16) {
        if (launch_split_f32(j, st)) return jvsip_gpu_last_error() == 0;
    }
    if (j.form == JVSIP_FORM_DF64 && j.twdd) {
        if (launch_fast_dd(j, st)) return jvsip_gpu_last_error() == 0;
    }
    // columns take the two steps when the plan's scratch can be had, the
    // tile kernels otherwise
    const bool two = long_few(j) || (long_columns(j) && long_scratch(j.lp, long_scratch_need(j), true));
    if (job_in_smem(j) && !two) {
        if (j.prec == P_F32) {
            if (launch_fast_f32(j, st)) return true;
            return launch_smem_f32(j, st);
        }
        return launch_smem_f64(j, st);
    }
    if (j.lp) {
        bool handled = false;
        const bool ok = run_long(j, st, &handled);
        if (handled) return ok;
    }
    if (job_in_smem(j)) {
        if (j.prec == P_F32) {
            if (launch_fast_f32(j, st)) return true;
            return launch_smem_f32(j, st);
        }
        return launch_smem_f64(j, st);
    }
    return j.prec == P_F32 ? launch_global_f32(j, st) : launch_global_f64(j, st);
}

// ---------------------------------------------------------------- plan graphs
static bool same_cview(const CView &a, const CView &b) {
    return a.re == b.re && a.im == b.im && a.cst == b.cst && a.off == b.off && a.es == b.es && a.vs == b.vs;
}
static bool same_rview(const RView &a, const RView &b) {
    return a.a == b.a && a.rst == b.rst && a.off == b.off && a.es == b.es && a.vs == b.vs;
}
static bool same_call(const Job &a, const Job &b) {
    return a.kind == b.kind && a.form == b.form && a.no_fast == b.no_fast && a.tma_columns == b.tma_columns &&
           a.inplace == b.inplace &&
           a.nvec == b.nvec && same_cview(a.cin, b.cin) && same_cview(a.cout, b.cout) && same_rview(a.rin, b.rin) &&
           same_rview(a.rout, b.rout);
}

// A device-resident call of a plan created with ntimes == 0: the first call
// with these views runs directly (and creates every lazily built resource),
// the second is captured into a CUDA graph, later ones replay it.  Calls on
// the multi-pass global path (scratch allocations) always run directly.
static constexpr size_t kPlanGraphs = 8;

static bool run_job_planned(Plan *p, Job &j, cudaStream_t st) {
    if (p->ntimes != 0 || j.nvec <= 0 || j.N <= 0) return run_job(j, st);
    const bool split = (j.form == JVSIP_FORM_SPLIT_BF16 || j.form == JVSIP_FORM_SPLIT_FP16);
    // a long transform captures once its plan holds the scratch for this call
    const size_t esz = j.prec == P_F32 ? sizeof(float) : sizeof(double);
    CView tmpv;
    const bool long_job = j.lp && (!job_in_smem(j) || long_few(j) || long_columns(j)) &&
                          ((j.kind == K_C2C && interleaved(j.cin, esz) && interleaved(j.cout, esz)) ||
                           (j.kind == K_R2C && interleaved(j.cout, esz) && real_as_complex(j.rin, j.nvec, esz, &tmpv)) ||
                           j.kind == K_C2R);
    const bool long_ready = long_job && j.lp->scratch_bytes >= long_scratch_need(j);
    if (!split && !job_in_smem(j) && !long_job) return run_job(j, st);
    CallGraph *e = nullptr;
    for (CallGraph &g : p->graphs)
        if (same_call(g.key, j)) e = &g;
    if (!e) {
        if (p->graphs.size() >= kPlanGraphs) {
            if (p->graphs.front().exec) cudaGraphExecDestroy(p->graphs.front().exec);
            p->graphs.erase(p->graphs.begin());
        }
        CallGraph g;
        g.key = j;
        p->graphs.push_back(g);
        return run_job(j, st);
    }
    if (!e->exec && !e->failed && (!long_job || long_ready)) {
        cudaStream_t cs = nullptr;
        cudaGraph_t graph = nullptr;
        const int err0 = jvsip_gpu_last_error();
        const unsigned long n0 = jvsip_gpu_kernel_launches();
        bool ok = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) == cudaSuccess &&
                  cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
        bool ran = false;
        if (ok) {
            ran = run_job(j, cs);
            ok = (cudaStreamEndCapture(cs, &graph) == cudaSuccess) && ran && graph;
        }
        const unsigned long n1 = jvsip_gpu_kernel_launches();
        count_launch_undo(n1 - n0);  // recorded, not run
        if (ok) ok = cudaGraphInstantiate(&e->exec, graph, 0) == cudaSuccess;
        if (graph) cudaGraphDestroy(graph);
        if (cs) cudaStreamDestroy(cs);
        e->kernels = (unsigned)(n1 - n0);
        if (!ok) {
            cudaGetLastError();
            if (e->exec) cudaGraphExecDestroy(e->exec);
            e->exec = nullptr;
            e->failed = true;
            // an error recorded by the refused capture is not the caller's
            if (err0 == 0 && jvsip_gpu_last_error() != 0) jvsip_gpu_clear_error();
        }
    }
    if (!e->exec) return run_job(j, st);
    if (!cuda_ok(cudaGraphLaunch(e->exec, st), "plan graph launch")) return false;
    count_launch(e->kernels);
    return true;
}

// Staged (host) views: copy results back and wait, so the host data is
// current when the call returns.  All-resident calls return asynchronously;
// work on the library stream is ordered, and release / sync wait for it.
static bool finish(Staging &stg, cudaStream_t st, bool ok) {
    // a failed step that did not say why still leaves a status for the caller
    if (!ok && !jvsip_gpu_last_error()) set_error(E_UNSUPPORTED, "fft execution path refused the call");
    if (stg.regs.empty()) return ok;
    ok = ok && stg.download(st);
    return cuda_ok(cudaStreamSynchronize(st), "fftm execution") && ok;
}

static void fill_job(Job &j, const Plan *p, int kind) {
    j.kind = kind;
    j.prec = p->prec;
    j.N = p->MN;
    j.nvec = p->mN;
    j.inv = (p->dir == 1) ? 1 : 0;
    j.has_scale = (p->scale != 1.0) ? 1 : 0;
    j.scale = p->scale;
    j.tw = p->d_tw;
    j.thalf = p->d_thalf;
    j.twp = p->d_twp;
    j.twg = p->d_twg;
    j.pc = p->d_pc;
    j.twdd = p->d_twdd;
    j.form = p->form;
    j.no_fast = p->no_fast;
    j.no_pipeline = p->no_pipeline;
    j.tma_columns = p->tma_columns;
    j.tuned_vpb = p->tuned_vpb;
    j.tuned_emax = p->tuned_emax;
    j.npass = (int)p->radix.size();
    for (int i = 0; i < j.npass && i < 40; i++) j.radix[i] = p->radix[i];
    j.lp = p->lp;
}

// Host-resident c2c call whose views are rows of unit element stride and
// positive pitch (the common dense case): the transforms are cut into chunks
// that flow host -> device (copy stream), kernel (library stream), device ->
// host (second copy stream), so both copy directions and the kernels overlap.
// Each chunk is copied with a 2-D copy of exactly its rows, so pitched views
// need no read-back of the gaps.  Returns false (nothing done) when the views
// do not qualify.
template <typename T, typename CB>
static bool pipelined_cc(Job &j, const CRes<T, CB> &rx, const CRes<T, CB> &ry, bool same_view, bool *ok) {
    if (j.no_pipeline) return false;
    if (rx.m || ry.m) return false;
    if (rx.blk->cstride != 2 || ry.blk->cstride != 2) return false;
    const long len = j.N, nv = j.nvec;
    if (rx.g.es != 1 || ry.g.es != 1 || rx.g.vs < len || ry.g.vs < len || nv < 2) return false;
    if (!same_view && rx.blk == ry.blk) return false;  // overlapping spans are handled by the general path
    const size_t esz = 2 * sizeof(T);
    const size_t row_b = (size_t)len * esz;
    const size_t total = row_b * (size_t)nv;
    if (total < ((size_t)64 << 20)) return false;       // small calls: one copy each way is as good
    Device *d = device();
    long chunks = (long)(total / ((size_t)128 << 20));
    if (chunks < 4) chunks = 4;
    if (chunks > 32) chunks = 32;
    if (chunks > nv) chunks = nv;
    const long rpc = (nv + chunks - 1) / chunks;
    chunks = (nv + rpc - 1) / rpc;
    char *din = (char *)dmalloc(total);
    char *dout = same_view ? din : (char *)dmalloc(total);
    if (!din || !dout) {
        dfree(din);
        if (!same_view) dfree(dout);
        *ok = false;
        return true;
    }
    const char *hx = (const char *)rx.blk->R->array + (size_t)rx.g.off * esz;
    char *hy = (char *)ry.blk->R->array + (size_t)ry.g.off * esz;
    bool good = true;
    // the copy-in of a chunk must not overtake earlier library work that may
    // still read the pool buffers it reuses
    cudaEvent_t *ev = d->ev;
    good = good && cuda_ok(cudaEventRecord(ev[0], d->stream), "event");
    good = good && cuda_ok(cudaStreamWaitEvent(d->h2d, ev[0], 0), "wait");
    for (long c = 0; c < chunks && good; c++) {
        long r0 = c * rpc, r1 = std::min(nv, r0 + rpc);
        cudaEvent_t ein = ev[1 + 2 * (c % 63)], eker = ev[2 + 2 * (c % 63)];
        good = cuda_ok(cudaMemcpy2DAsync(din + (size_t)r0 * row_b, row_b, hx + (size_t)r0 * rx.g.vs * esz,
                                         (size_t)rx.g.vs * esz, row_b, (size_t)(r1 - r0), cudaMemcpyHostToDevice,
                                         d->h2d), "pipelined copy in");
        good = good && cuda_ok(cudaEventRecord(ein, d->h2d), "event");
        good = good && cuda_ok(cudaStreamWaitEvent(d->stream, ein, 0), "wait");
        Job q = j;
        q.nvec = r1 - r0;
        q.cin.re = din + (size_t)r0 * row_b;
        q.cin.im = (T *)q.cin.re + 1;
        q.cin.cst = 2;
        q.cin.off = 0;
        q.cin.es = 1;
        q.cin.vs = len;
        q.cout = q.cin;
        q.cout.re = dout + (size_t)r0 * row_b;
        q.cout.im = (T *)q.cout.re + 1;
        q.inplace = same_view ? 1 : 0;
        good = good && run_job(q, d->stream);
        good = good && cuda_ok(cudaEventRecord(eker, d->stream), "event");
        good = good && cuda_ok(cudaStreamWaitEvent(d->d2h, eker, 0), "wait");
        good = good && cuda_ok(cudaMemcpy2DAsync(hy + (size_t)r0 * ry.g.vs * esz, (size_t)ry.g.vs * esz,
                                                 dout + (size_t)r0 * row_b, row_b, row_b, (size_t)(r1 - r0),
                                                 cudaMemcpyDeviceToHost, d->d2h), "pipelined copy out");
    }
    // later library work is ordered after the copy-out, then wait for it
    cuda_ok(cudaEventRecord(ev[127], d->d2h), "event");
    cuda_ok(cudaStreamWaitEvent(d->stream, ev[127], 0), "wait");
    good = cuda_ok(cudaStreamSynchronize(d->d2h), "pipelined fftm") && good;
    good = cuda_ok(cudaStreamSynchronize(d->stream), "pipelined fftm") && good;
    dfree(din);
    if (!same_view) dfree(dout);
    *ok = good;
    return true;
}

template <typename T, typename CMV, typename CB>
static void exec_cc(Plan *p, const CMV *x, const CMV *y, bool ip) {
    if (!p) {
        set_error(E_ARG, "invalid fft plan");
        return;
    }
    if (p->type != JV_CCFFTOP && p->type != JV_CCFFTIP) {
        set_error(E_ARG, "plan is not a complex-to-complex plan");
        return;
    }
    Device *d = device();
    if (!d) return;
    std::lock_guard<std::mutex> lk(p->mu);
    if (!view_ok(x, p->major, p->MN, p->mN) || (!ip && !view_ok(y, p->major, p->MN, p->mN))) {
        set_error(E_ARG, "view smaller than the plan");
        return;
    }
    Job j;
    fill_job(j, p, K_C2C);
    CRes<T, CB> rx{x->block, cgeo(x, p->major, p->MN, p->mN), mirror_find(x->block)};
    CRes<T, CB> ry = rx;
    bool same_view = ip;
    if (!ip) {
        ry = CRes<T, CB>{y->block, cgeo(y, p->major, p->MN, p->mN), mirror_find(y->block)};
        same_view = (x->block == y->block && rx.g.off == ry.g.off && rx.g.es == ry.g.es && rx.g.vs == ry.g.vs);
    }
    {
        bool pok = false;
        if (pipelined_cc<T, CB>(j, rx, ry, same_view, &pok)) return;
    }
    Staging stg;
    cudaStream_t st = d->stream;
    stage_c(stg, rx, true, same_view);
    if (!same_view) stage_c(stg, ry, !ry.g.dense() || (y->block == x->block), true);
    if (!stg.upload(st)) return;
    j.cin = dev_c(stg, rx);
    j.cout = same_view ? j.cin : dev_c(stg, ry);
    j.inplace = same_view ? 1 : 0;
    void *tmp = nullptr;
    if (!same_view && x->block == y->block) {
        long xl = rx.g.lo(), xh = rx.g.hi(), yl = ry.g.lo(), yh = ry.g.hi();
        if (!(xh < yl || yh < xl)) {
            // x and y overlap in one block: transform from a private copy of x
            // (the reference copies x into y first, VI_ccfftmop_f_def.h:26)
            size_t n = (size_t)(xh - xl + 1);
            bool split = (x->block->cstride == 1);
            size_t b = n * (split ? 1 : 2) * sizeof(T);
            tmp = dmalloc(split ? 2 * b : b);
            if (!tmp) return;
            Geo gd = rx.g;
            gd.off = j.cin.off;  // x's geometry in device index space
            xl = gd.lo();
            char *src_re = (char *)j.cin.re + (size_t)xl * j.cin.cst * sizeof(T);
            if (!split) {
                if (!cuda_ok(cudaMemcpyAsync(tmp, src_re, b, cudaMemcpyDeviceToDevice, st), "alias copy")) return;
                j.cin.re = tmp;
                j.cin.im = (T *)tmp + 1;
            } else {
                char *src_im = (char *)j.cin.im + (size_t)xl * sizeof(T);
                if (!cuda_ok(cudaMemcpyAsync(tmp, src_re, b, cudaMemcpyDeviceToDevice, st), "alias copy") ||
                    !cuda_ok(cudaMemcpyAsync((char *)tmp + b, src_im, b, cudaMemcpyDeviceToDevice, st), "alias copy"))
                    return;
                j.cin.re = tmp;
                j.cin.im = (char *)tmp + b;
            }
            j.cin.off -= xl;
        }
    }
    bool ok = (stg.regs.empty() && !tmp) ? run_job_planned(p, j, st) : run_job(j, st);
    ok = finish(stg, st, ok);
    dfree(tmp);  // stream-ordered: the pool hands it out only to later work on this stream
    if (ok) mark_written(same_view ? (const void *)x->block : (const void *)y->block);
}

// The job of a c2c call of plan p on views of admitted interleaved blocks
// (both resident), or false.
static bool resident_job_f(Plan *p, const vsip_cmview_f *x, const vsip_cmview_f *y, Job &j) {
    if (!p || p->prec != P_F32 || (p->type != JV_CCFFTOP && p->type != JV_CCFFTIP) || !x || !y || !x->block ||
        !y->block)
        return false;
    if (!view_ok(x, p->major, p->MN, p->mN) || !view_ok(y, p->major, p->MN, p->mN)) return false;
    CRes<float, vsip_cblock_f> rx{x->block, cgeo(x, p->major, p->MN, p->mN), mirror_find(x->block)};
    CRes<float, vsip_cblock_f> ry{y->block, cgeo(y, p->major, p->MN, p->mN), mirror_find(y->block)};
    if (!rx.m || !ry.m) return false;
    const bool same = (x->block == y->block && rx.g.off == ry.g.off && rx.g.es == ry.g.es && rx.g.vs == ry.g.vs);
    if (x->block == y->block && !same) return false;
    fill_job(j, p, K_C2C);
    Staging stg;  // stays empty: both views are resident
    j.cin = dev_c(stg, rx);
    j.cout = same ? j.cin : dev_c(stg, ry);
    j.inplace = same ? 1 : 0;
    return true;
}

bool resident_long_columns_f(Plan *p, const vsip_cmview_f *x, const vsip_cmview_f *y) {
    if (!p) return false;
    std::lock_guard<std::mutex> lk(p->mu);
    Job j;
    return resident_job_f(p, x, y, j) && long_columns(j);
}

bool enqueue_resident_c2c_f(Plan *p, const vsip_cmview_f *x, const vsip_cmview_f *y, cudaStream_t st, bool prepare) {
    if (!p || !device()) return false;
    std::lock_guard<std::mutex> lk(p->mu);
    Job j;
    if (!resident_job_f(p, x, y, j)) {
        set_error(E_ARG, "resident c2c call: views of admitted interleaved blocks expected");
        return false;
    }
    if (prepare) return !j.lp || long_scratch(j.lp, long_scratch_need(j), false);
    return run_job(j, st);
}

template <typename T, typename RMV, typename CMV, typename RB, typename CB>
static void exec_rc(Plan *p, const RMV *x, const CMV *z) {
    if (!p || p->type != JV_RCFFTOP) {
        set_error(E_ARG, "invalid real-to-complex fftm plan");
        return;
    }
    Device *d = device();
    if (!d) return;
    std::lock_guard<std::mutex> lk(p->mu);
    if (!x || !z || !x->block || !z->block) {
        set_error(E_ARG, "null view");
        return;
    }
    Job j;
    fill_job(j, p, K_R2C);
    Geo gx;
    gx.off = (long)x->offset;
    gx.es = p->major == 0 ? x->row_stride : x->col_stride;
    gx.vs = p->major == 0 ? x->col_stride : x->row_stride;
    gx.len = 2 * p->MN;
    gx.nvec = p->mN;
    RRes<T, RB> rx = resolve_r<T, RB>(x->block, gx);
    CRes<T, CB> rz{z->block, cgeo(z, p->major, p->MN + 1, p->mN), mirror_find(z->block)};
    Staging stg;
    cudaStream_t st = d->stream;
    stage_r(stg, rx, true, false);
    stage_c(stg, rz, !rz.g.dense(), true);
    if (!stg.upload(st)) return;
    j.rin = dev_r(stg, rx);
    j.cout = dev_c(stg, rz);
    bool ok = stg.regs.empty() ? run_job_planned(p, j, st) : run_job(j, st);
    ok = finish(stg, st, ok);
    if (ok) mark_written(z->block);
}

template <typename T, typename CMV, typename RMV, typename CB, typename RB>
static void exec_cr(Plan *p, const CMV *z, const RMV *x) {
    if (!p || p->type != JV_CRFFTOP) {
        set_error(E_ARG, "invalid complex-to-real fftm plan");
        return;
    }
    Device *d = device();
    if (!d) return;
    std::lock_guard<std::mutex> lk(p->mu);
    if (!x || !z || !x->block || !z->block) {
        set_error(E_ARG, "null view");
        return;
    }
    Job j;
    fill_job(j, p, K_C2R);
    Geo gx;
    gx.off = (long)x->offset;
    gx.es = p->major == 0 ? x->row_stride : x->col_stride;
    gx.vs = p->major == 0 ? x->col_stride : x->row_stride;
    gx.len = 2 * p->MN;
    gx.nvec = p->mN;
    RRes<T, RB> rx = resolve_r<T, RB>(x->block, gx);
    CRes<T, CB> rz{z->block, cgeo(z, p->major, p->MN + 1, p->mN), mirror_find(z->block)};
    Staging stg;
    cudaStream_t st = d->stream;
    stage_c(stg, rz, true, false);
    stage_r(stg, rx, !rx.g.dense(), true);
    if (!stg.upload(st)) return;
    j.cin = dev_c(stg, rz);
    j.rout = dev_r(stg, rx);
    bool ok = stg.regs.empty() ? run_job_planned(p, j, st) : run_job(j, st);
    ok = finish(stg, st, ok);
    if (ok) {
        if (rx.blk->parent) mark_written(rx.blk->parent);
        mark_written(rx.blk);
    }
}

// A vector view as the one-row matrix view over the same elements (null-safe:
// a null vector gives a view without a block, which the checks reject).
static vsip_cmview_f row_of(const vsip_cvview_f *v) {
    vsip_cmview_f m;
    memset(&m, 0, sizeof(m));
    if (!v) return m;
    m.block = v->block;
    m.offset = v->offset;
    m.row_stride = v->stride;
    m.row_length = v->length;
    m.col_stride = (vsip_stride)v->length * v->stride;
    m.col_length = 1;
    m.markings = v->markings;
    return m;
}
static vsip_cmview_d row_of(const vsip_cvview_d *v) {
    vsip_cmview_d m;
    memset(&m, 0, sizeof(m));
    if (!v) return m;
    m.block = v->block;
    m.offset = v->offset;
    m.row_stride = v->stride;
    m.row_length = v->length;
    m.col_stride = (vsip_stride)v->length * v->stride;
    m.col_length = 1;
    m.markings = v->markings;
    return m;
}
static vsip_mview_f row_of(const vsip_vview_f *v) {
    vsip_mview_f m;
    memset(&m, 0, sizeof(m));
    if (!v) return m;
    m.block = v->block;
    m.offset = v->offset;
    m.row_stride = v->stride;
    m.row_length = v->length;
    m.col_stride = (vsip_stride)v->length * v->stride;
    m.col_length = 1;
    m.markings = v->markings;
    return m;
}
static vsip_mview_d row_of(const vsip_vview_d *v) {
    vsip_mview_d m;
    memset(&m, 0, sizeof(m));
    if (!v) return m;
    m.block = v->block;
    m.offset = v->offset;
    m.row_stride = v->stride;
    m.row_length = v->length;
    m.col_stride = (vsip_stride)v->length * v->stride;
    m.col_length = 1;
    m.markings = v->markings;
    return m;
}

}  // namespace jv

using namespace jv;

extern "C" {

void vsip_ccfftmop_f(const vsip_fftm_f *p, const vsip_cmview_f *x, const vsip_cmview_f *y) {
    exec_cc<float, vsip_cmview_f, vsip_cblock_f>(plan_of(p), x, y, false);
}
void vsip_ccfftmip_f(const vsip_fftm_f *p, const vsip_cmview_f *xy) {
    exec_cc<float, vsip_cmview_f, vsip_cblock_f>(plan_of(p), xy, xy, true);
}
void vsip_ccfftmop_d(const vsip_fftm_d *p, const vsip_cmview_d *x, const vsip_cmview_d *y) {
    exec_cc<double, vsip_cmview_d, vsip_cblock_d>(plan_of(p), x, y, false);
}
void vsip_ccfftmip_d(const vsip_fftm_d *p, const vsip_cmview_d *xy) {
    exec_cc<double, vsip_cmview_d, vsip_cblock_d>(plan_of(p), xy, xy, true);
}
void vsip_rcfftmop_f(const vsip_fftm_f *p, const vsip_mview_f *x, const vsip_cmview_f *z) {
    exec_rc<float, vsip_mview_f, vsip_cmview_f, vsip_block_f, vsip_cblock_f>(plan_of(p), x, z);
}
void vsip_rcfftmop_d(const vsip_fftm_d *p, const vsip_mview_d *x, const vsip_cmview_d *z) {
    exec_rc<double, vsip_mview_d, vsip_cmview_d, vsip_block_d, vsip_cblock_d>(plan_of(p), x, z);
}
void vsip_crfftmop_f(const vsip_fftm_f *p, const vsip_cmview_f *z, const vsip_mview_f *x) {
    exec_cr<float, vsip_cmview_f, vsip_mview_f, vsip_cblock_f, vsip_block_f>(plan_of(p), z, x);
}
void vsip_crfftmop_d(const vsip_fftm_d *p, const vsip_cmview_d *z, const vsip_mview_d *x) {
    exec_cr<double, vsip_cmview_d, vsip_mview_d, vsip_cblock_d, vsip_block_d>(plan_of(p), z, x);
}

// Single FFTs (c_VSIP_src/VI_ccfftop_f_def.h:19-28, VI_ccfftip_f.h,
// VI_rcfftop_f_def.h:22-101, VI_crfftop_f_def.h:20-87): a vector view of
// `length` elements `stride` apart is the one-row matrix view with that row
// stride, so the single FFT runs the multiple-FFT path with one transform.
void vsip_ccfftop_f(const vsip_fft_f *p, const vsip_cvview_f *x, const vsip_cvview_f *y) {
    vsip_cmview_f mx = row_of(x), my = row_of(y);
    exec_cc<float, vsip_cmview_f, vsip_cblock_f>(plan_of_v(p), x ? &mx : nullptr, y ? &my : nullptr, false);
}
void vsip_ccfftip_f(const vsip_fft_f *p, const vsip_cvview_f *xy) {
    vsip_cmview_f m = row_of(xy);
    exec_cc<float, vsip_cmview_f, vsip_cblock_f>(plan_of_v(p), xy ? &m : nullptr, xy ? &m : nullptr, true);
}
void vsip_ccfftop_d(const vsip_fft_d *p, const vsip_cvview_d *x, const vsip_cvview_d *y) {
    vsip_cmview_d mx = row_of(x), my = row_of(y);
    exec_cc<double, vsip_cmview_d, vsip_cblock_d>(plan_of_v(p), x ? &mx : nullptr, y ? &my : nullptr, false);
}
void vsip_ccfftip_d(const vsip_fft_d *p, const vsip_cvview_d *xy) {
    vsip_cmview_d m = row_of(xy);
    exec_cc<double, vsip_cmview_d, vsip_cblock_d>(plan_of_v(p), xy ? &m : nullptr, xy ? &m : nullptr, true);
}
void vsip_rcfftop_f(const vsip_fft_f *p, const vsip_vview_f *x, const vsip_cvview_f *z) {
    vsip_mview_f mx = row_of(x);
    vsip_cmview_f mz = row_of(z);
    exec_rc<float, vsip_mview_f, vsip_cmview_f, vsip_block_f, vsip_cblock_f>(plan_of_v(p), x ? &mx : nullptr,
                                                                            z ? &mz : nullptr);
}
void vsip_rcfftop_d(const vsip_fft_d *p, const vsip_vview_d *x, const vsip_cvview_d *z) {
    vsip_mview_d mx = row_of(x);
    vsip_cmview_d mz = row_of(z);
    exec_rc<double, vsip_mview_d, vsip_cmview_d, vsip_block_d, vsip_cblock_d>(plan_of_v(p), x ? &mx : nullptr,
                                                                             z ? &mz : nullptr);
}
void vsip_crfftop_f(const vsip_fft_f *p, const vsip_cvview_f *z, const vsip_vview_f *x) {
    vsip_cmview_f mz = row_of(z);
    vsip_mview_f mx = row_of(x);
    exec_cr<float, vsip_cmview_f, vsip_mview_f, vsip_cblock_f, vsip_block_f>(plan_of_v(p), z ? &mz : nullptr,
                                                                            x ? &mx : nullptr);
}
void vsip_crfftop_d(const vsip_fft_d *p, const vsip_cvview_d *z, const vsip_vview_d *x) {
    vsip_cmview_d mz = row_of(z);
    vsip_mview_d mx = row_of(x);
    exec_cr<double, vsip_cmview_d, vsip_mview_d, vsip_cblock_d, vsip_block_d>(plan_of_v(p), z ? &mz : nullptr,
                                                                             x ? &mx : nullptr);
}

const char *jvsip_gpu_build_info(void) {
    static thread_local char buf[256];  // valid until the calling thread's next call
    Device *d = device();
    snprintf(buf, sizeof(buf), "jvsip_gb300 fftm: sm_103a kernels; device %d, %d SMs, %zu B smem/block",
             d ? d->id : -1, d ? d->sms : 0, d ? d->smem_optin : (size_t)0);
    return buf;
}

}  // extern "C"
