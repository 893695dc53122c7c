/*
 * fftm_oracle_body.h -- type-generic body of the CPU oracle (TEST INFRASTRUCTURE
 * ONLY; see fftm_oracle.h).  Included twice by fftm_oracle.c with
 *   T = float,  SFX = _f   and   T = double, SFX = _d.
 *
 * Each function names the reference routine whose algorithm and arithmetic
 * order it restates (paths relative to the jvsip repository).  Additions are
 * grouped exactly as in the reference so that results agree bit for bit when
 * compiled without floating-point contraction (-ffp-contract=off).
 */
#define ORC_CAT2(a, b) a##b
#define ORC_CAT(a, b) ORC_CAT2(a, b)
#define FN(name) ORC_CAT(name, SFX)
#define PLAN FN(orc_fftm)
#define CMV FN(orc_cmview)
#define RMV FN(orc_mview)
#define CTX FN(orc_ctx)

struct PLAN {
    int kind, major, dir, dft;
    unsigned long M, N, MN, mN, nstage;
    unsigned long pn[6], p0[6], pF[6];
    T scale;
    T *wr, *wi;          /* exp(dir*2*pi*i*k/MN), k < MN  (create: VI_ccfftmop_create_f_def.h:64-75) */
    T *er, *ei;          /* exp(-+pi*i*k/MN), k <= MN      (VI_rcfftmop_create_f_def.h:75-86)  */
    unsigned long *index;/* jofk digit reversal             (VI_ccfftmop_create_f_def.h:82-86) */
    T *tr, *ti;          /* DFT / sort scratch, MN entries                                       */
    T *mr, *mi;          /* real-transform mirror vector, MN+1 entries                           */
    T *yr, *yi;          /* C2R row-major work matrix, mN x (MN+1) (VI_crfftmop_create_f_def.h:45) */
};

/* In-place execution state: base points at element 0 of vector 0 (in scalar
 * units); elements of a vector are xst scalars apart, vectors ypst apart
 * (VI_init_fftm_f, VI_fftm_building_blocks_f.h:1044-1060). */
typedef struct {
    const struct PLAN *p;
    T *re, *im;
    long xst, ypst;
    unsigned long len;   /* length of the top-level vector view */
} CTX;

/* ---------------- small Winograd DFTs (VI_fft{2,3,4,5,7,8}m_f / VI_ifft*m_f,
 * VI_fftm_building_blocks_f.h:162-836).  Each call transforms one butterfly
 * position in every vector: element e of the butterfly is at offset e*es from
 * (re,im)+off, vectors are c->ypst apart. ---------------- */
#define LD(k, v) do { v##r = pr[(k) * es]; v##i = pi[(k) * es]; } while (0)
#define ST(k, xr, xi) do { pr[(k) * es] = (xr); pi[(k) * es] = (xi); } while (0)

static void FN(orc_b2)(const CTX *c, long off, long es)
{
    unsigned long v;
    for (v = 0; v < c->p->mN; v++) {
        T *pr = c->re + off + (long)v * c->ypst, *pi = c->im + off + (long)v * c->ypst;
        T a0r, a0i, a1r, a1i;
        LD(0, a0); LD(1, a1);
        ST(1, a0r - a1r, a0i - a1i);
        ST(0, a0r + a1r, a0i + a1i);
    }
}

static void FN(orc_b3)(const CTX *c, long off, long es, int inv)
{
    const T k1 = (T)-1.5;                                       /* -(1 + cos(2pi/3)) */
    const T k2 = (T)0.866025403784438646763723170752936183;     /* sin(2pi/3) */
    unsigned long v;
    for (v = 0; v < c->p->mN; v++) {
        T *pr = c->re + off + (long)v * c->ypst, *pi = c->im + off + (long)v * c->ypst;
        T a0r, a0i, a1r, a1i, a2r, a2i;
        T sr, si, dr, di, tr, ti, hr, hi, qr, qi, ur, ui;
        LD(0, a0); LD(1, a1); LD(2, a2);
        sr = a1r + a2r; si = a1i + a2i;       /* a1 + a2 */
        dr = a1r - a2r; di = a1i - a2i;       /* a1 - a2 */
        tr = a0r + sr;  ti = a0i + si;        /* y0 */
        hr = k1 * sr;   hi = k1 * si;
        if (!inv) { qr = k2 * di; qi = k2 * dr; }
        else      { qr = -k2 * di; qi = -k2 * dr; }
        ur = tr + hr;   ui = ti + hi;
        ST(2, ur - qr, ui + qi);
        ST(1, ur + qr, ui - qi);
        ST(0, tr, ti);
    }
}

static void FN(orc_b4)(const CTX *c, long off, long es, int inv)
{
    unsigned long v;
    for (v = 0; v < c->p->mN; v++) {
        T *pr = c->re + off + (long)v * c->ypst, *pi = c->im + off + (long)v * c->ypst;
        T a0r, a0i, a1r, a1i, a2r, a2i, a3r, a3i;
        T s02r, s02i, d02r, d02i, s13r, s13i, d13r, d13i;
        LD(0, a0); LD(1, a1); LD(2, a2); LD(3, a3);
        s02r = a0r + a2r; s02i = a0i + a2i;
        d02r = a0r - a2r; d02i = a0i - a2i;
        s13r = a1r + a3r; s13i = a1i + a3i;
        d13r = a1r - a3r; d13i = a1i - a3i;
        if (!inv) {
            ST(3, d02r - d13i, d02i + d13r);
            ST(2, s02r - s13r, s02i - s13i);
            ST(1, d02r + d13i, d02i - d13r);
        } else {
            ST(3, d02r + d13i, d02i - d13r);
            ST(2, s02r - s13r, s02i - s13i);
            ST(1, d02r - d13i, d02i + d13r);
        }
        ST(0, s02r + s13r, s02i + s13i);
    }
}

static void FN(orc_b5)(const CTX *c, long off, long es, int inv)
{
    const T k1 = (T)-1.25;                                      /* (cos u + cos 2u)/2 - 1, u = 2pi/5 */
    const T k2 = (T)0.559016994374947424102293417182819059;     /* (cos u - cos 2u)/2 */
    const T k3 = (T)0.587785252292473129168705954639072769;     /* sin 2u */
    const T k4 = (T)1.53884176858762670128514528801845491;      /* sin u + sin 2u */
    const T k5 = (T)0.363271264002680442947733378740309375;     /* sin u - sin 2u */
    unsigned long v;
    for (v = 0; v < c->p->mN; v++) {
        T *pr = c->re + off + (long)v * c->ypst, *pi = c->im + off + (long)v * c->ypst;
        T a0r, a0i, a1r, a1i, a2r, a2i, a3r, a3i, a4r, a4i;
        T s14r, s14i, d14r, d14i, s23r, s23i, d32r, d32i;
        T ssr, ssi, sdr, sdi, ddr, ddi, y0r, y0i;
        T m1r, m1i, m2r, m2i, m3r, m3i, m4r, m4i, m5r, m5i;
        T e1r, e1i, g1r, g1i, g2r, g2i, g3r, g3i, g4r, g4i;
        LD(0, a0); LD(1, a1); LD(2, a2); LD(3, a3); LD(4, a4);
        s14r = a1r + a4r; s14i = a1i + a4i;
        d14r = a1r - a4r; d14i = a1i - a4i;
        s23r = a2r + a3r; s23i = a2i + a3i;
        d32r = a3r - a2r; d32i = a3i - a2i;
        ssr = s14r + s23r; ssi = s14i + s23i;
        sdr = s14r - s23r; sdi = s14i - s23i;
        ddr = d14r + d32r; ddi = d14i + d32i;
        y0r = ssr + a0r;   y0i = ssi + a0i;
        m1r = ssr * k1;    m1i = ssi * k1;
        m3r = sdr * k2;    m3i = sdi * k2;
        if (!inv) {
            m5r = ddr * k3;     m5i = ddi * k3;
            m2r = d14i * k4;    m2i = -(d14r * k4);
            m4r = -(d32i * k5); m4i = d32r * k5;
        } else {
            m5r = -(ddr * k3);  m5i = -(ddi * k3);
            m2r = -(d14i * k4); m2i = d14r * k4;
            m4r = d32i * k5;    m4i = -(d32r * k5);
        }
        e1r = m1r + y0r;   e1i = m1i + y0i;
        g1r = e1r + m3r;   g1i = e1i + m3i;
        g2r = m2r - m5i;   g2i = m2i + m5r;
        g3r = e1r - m3r;   g3i = e1i - m3i;
        g4r = m4r - m5i;   g4i = m4i + m5r;
        ST(4, g1r - g2r, g1i - g2i);
        ST(3, g3r + g4r, g3i + g4i);
        ST(2, g3r - g4r, g3i - g4i);
        ST(1, g1r + g2r, g1i + g2i);
        ST(0, y0r, y0i);
    }
}

static void FN(orc_b7)(const CTX *c, long off, long es, int inv)
{
    /* u = 2pi/7 */
    const T k1 = (T)-1.16666666666666666666666666666666667;     /* -1 + (cos u + cos 2u + cos 3u)/3 */
    const T k2 = (T)0.790156468525400197191671550670906477;     /* (2cos u - cos 2u - cos 3u)/3 */
    const T k3 = (T)0.0558542672896477376222358978301280928;    /* (cos u - 2cos 2u + cos 3u)/3 */
    const T k4 = (T)0.734302201235752459569435652840778384;     /* (cos u + cos 2u - 2cos 3u)/3 */
    const T k5 = (T)0.440958551844098431750269292273210071;     /* (sin u + sin 2u - sin 3u)/3 */
    const T k6 = (T)0.340872930623931376958175234400847679;     /* (2sin u - sin 2u + sin 3u)/3 */
    const T k7 = (T)-0.533969360337725175267862390720721146;    /* (sin u - 2sin 2u - sin 3u)/3 */
    const T k8 = (T)0.874842290961656552226037625121568826;     /* (sin u + sin 2u + 2sin 3u)/3 */
    unsigned long v;
    for (v = 0; v < c->p->mN; v++) {
        T *pr = c->re + off + (long)v * c->ypst, *pi = c->im + off + (long)v * c->ypst;
        T a0r, a0i, a1r, a1i, a2r, a2i, a3r, a3i, a4r, a4i, a5r, a5i, a6r, a6i;
        T p16r, p16i, m16r, m16i, p43r, p43i, m43r, m43i, p25r, p25i, m25r, m25i;
        T q1r, q1i, q2r, q2i, q3r, q3i, q4r, q4i, q5r, q5i, q6r, q6i, q7r, q7i, q8r, q8i;
        T sr_, si_, tr_, ti_, y0r, y0i;
        T n1r, n1i, n2r, n2i, n3r, n3i, n4r, n4i, n5r, n5i, n6r, n6i, n7r, n7i, n8r, n8i;
        T f1r, f1i, f2r, f2i, f3r, f3i, f4r, f4i;
        T h1r, h1i, h2r, h2i, h3r, h3i, h4r, h4i, h5r, h5i, h6r, h6i;
        T o1r, o1i, o2r, o2i, o3r, o3i;
        LD(0, a0); LD(1, a1); LD(2, a2); LD(3, a3); LD(4, a4); LD(5, a5); LD(6, a6);
        p16r = a1r + a6r; p16i = a1i + a6i;
        m16r = a1r - a6r; m16i = a1i - a6i;
        p43r = a4r + a3r; p43i = a4i + a3i;
        m43r = a4r - a3r; m43i = a4i - a3i;
        p25r = a2r + a5r; p25i = a2i + a5i;
        m25r = a2r - a5r; m25i = a2i - a5i;
        q1r = p16r + p43r; q1i = p16i + p43i;
        q2r = p43r - p25r; q2i = p43i - p25i;
        q3r = p16r - p43r; q3i = p16i - p43i;
        q4r = p25r - p16r; q4i = p25i - p16i;
        q5r = m16r + m43r; q5i = m16i + m43i;
        q6r = m16r - m43r; q6i = m16i - m43i;
        q7r = m43r - m25r; q7i = m43i - m25i;
        q8r = m25r - m16r; q8i = m25i - m16i;
        sr_ = p25r + q1r;  si_ = p25i + q1i;
        tr_ = m25r + q5r;  ti_ = m25i + q5i;
        y0r = a0r + sr_;   y0i = a0i + si_;
        n1r = sr_ * k1;    n1i = si_ * k1;
        n2r = q3r * k2;    n2i = q3i * k2;
        n3r = q2r * k3;    n3i = q2i * k3;
        n4r = q4r * k4;    n4i = q4i * k4;
        if (!inv) {
            n5r = -(ti_ * k5); n5i = tr_ * k5;
            n6r = -(q6i * k6); n6i = q6r * k6;
            n7r = -(q7i * k7); n7i = q7r * k7;
            n8r = -(q8i * k8); n8i = q8r * k8;
        } else {
            n5r = ti_ * k5;    n5i = -(tr_ * k5);
            n6r = q6i * k6;    n6i = -(q6r * k6);
            n7r = q7i * k7;    n7i = -(q7r * k7);
            n8r = q8i * k8;    n8i = -(q8r * k8);
        }
        f1r = y0r + n1r;   f1i = y0i + n1i;
        f2r = n5r + n6r;   f2i = n5i + n6i;
        f3r = n5r - n6r;   f3i = n5i - n6i;
        f4r = n5r - n7r;   f4i = n5i - n7i;
        h1r = f1r + n2r;   h1i = f1i + n2i;
        h2r = f1r - n2r;   h2i = f1i - n2i;
        h3r = f1r - n3r;   h3i = f1i - n3i;
        h4r = f2r + n7r;   h4i = f2i + n7i;
        h5r = f3r - n8r;   h5i = f3i - n8i;
        h6r = f4r + n8r;   h6i = f4i + n8i;
        o1r = h1r + n3r;   o1i = h1i + n3i;
        o2r = h2r - n4r;   o2i = h2i - n4i;
        o3r = h3r + n4r;   o3i = h3i + n4i;
        ST(6, o1r + h4r, o1i + h4i);
        ST(5, o2r + h5r, o2i + h5i);
        ST(4, o3r - h6r, o3i - h6i);
        ST(3, o3r + h6r, o3i + h6i);
        ST(2, o2r - h5r, o2i - h5i);
        ST(1, o1r - h4r, o1i - h4i);
        ST(0, y0r, y0i);
    }
}

static void FN(orc_b8)(const CTX *c, long off, long es, int inv)
{
    const T h = (T)0.707106781186547524400844362104849039;      /* cos(pi/4) */
    unsigned long v;
    for (v = 0; v < c->p->mN; v++) {
        T *pr = c->re + off + (long)v * c->ypst, *pi = c->im + off + (long)v * c->ypst;
        T a0r, a0i, a1r, a1i, a2r, a2i, a3r, a3i, a4r, a4i, a5r, a5i, a6r, a6i, a7r, a7i;
        T s04r, s04i, d04r, d04i, s15r, s15i, d15r, d15i, s26r, s26i, d26r, d26i, s37r, s37i, d37r, d37i;
        T u0r, u0i, u1r, u1i, u2r, u2i, u3r, u3i, u4r, u4i, u5r, u5i;
        T e0r, e0i, e1r, e1i, e2r, e2i, e3r, e3i, e4r, e4i, e5r, e5i, e6r, e6i, e7r, e7i;
        LD(0, a0); LD(1, a1); LD(2, a2); LD(3, a3); LD(4, a4); LD(5, a5); LD(6, a6); LD(7, a7);
        s04r = a0r + a4r; s04i = a0i + a4i;
        d04r = a0r - a4r; d04i = a0i - a4i;
        s15r = a1r + a5r; s15i = a1i + a5i;
        d15r = a1r - a5r; d15i = a1i - a5i;
        s26r = a2r + a6r; s26i = a2i + a6i;
        d26r = a2r - a6r; d26i = a2i - a6i;
        s37r = a3r + a7r; s37i = a3i + a7i;
        d37r = a3r - a7r; d37i = a3i - a7i;
        u0r = s04r + s26r; u0i = s04i + s26i;
        u1r = s04r - s26r; u1i = s04i - s26i;
        u2r = s15r + s37r; u2i = s15i + s37i;
        u3r = s15r - s37r; u3i = s15i - s37i;
        u4r = d15r + d37r; u4i = d15i + d37i;
        u5r = d15r - d37r; u5i = d15i - d37i;
        u4r = u4r * h;     u4i = u4i * h;
        u5r = u5r * h;     u5i = u5i * h;
        e0r = u0r + u2r;   e0i = u0i + u2i;
        e4r = u0r - u2r;   e4i = u0i - u2i;
        e1r = d04r + u5r;  e1i = d04i + u5i;
        e5r = d04r - u5r;  e5i = d04i - u5i;
        if (!inv) {
            e2r = u1r + u3i;    e2i = u1i - u3r;
            e6r = u1r - u3i;    e6i = u1i + u3r;
            e3r = d26i + u4i;   e3i = d26r + u4r;
            e7r = u4i - d26i;   e7i = d26r - u4r;
        } else {
            e2r = u1r - u3i;    e2i = u1i + u3r;
            e6r = u1r + u3i;    e6i = u1i - u3r;
            e3r = -(d26i + u4i); e3i = -(d26r + u4r);
            e7r = d26i - u4i;   e7i = u4r - d26r;
        }
        ST(7, e1r - e3r, e1i + e3i);
        ST(6, e6r, e6i);
        ST(5, e5r - e7r, e5i - e7i);
        ST(4, e4r, e4i);
        ST(3, e5r + e7r, e5i + e7i);
        ST(2, e2r, e2i);
        ST(1, e1r + e3r, e1i - e3i);
        ST(0, e0r, e0i);
    }
}
#undef LD
#undef ST

/* Twiddle pass of VI_fft_wtm_f (VI_fftm_building_blocks_f.h:839-873): element
 * e (e < len) of every vector is multiplied by table entry e*wst. */
static void FN(orc_twiddle)(const CTX *c, long off, long es, unsigned long len, unsigned long wst)
{
    const struct PLAN *p = c->p;
    unsigned long v, e;
    for (v = 0; v < p->mN; v++) {
        T *pr = c->re + off + (long)v * c->ypst, *pi = c->im + off + (long)v * c->ypst;
        for (e = 0; e < len; e++) {
            T ar = pr[(long)e * es], ai = pi[(long)e * es];
            T br = p->wr[e * wst], bi = p->wi[e * wst];
            T t = ar * br - bi * ai;
            pi[(long)e * es] = ar * bi + ai * br;
            pr[(long)e * es] = t;
        }
    }
}

/* O(L^2) DFT of VI_dftm_f (VI_fftm_building_blocks_f.h:95-155): table entries
 * are taken at stride MN/L; results go through the scratch vector. */
static void FN(orc_dft)(const CTX *c, long off, long es, unsigned long L)
{
    const struct PLAN *p = c->p;
    unsigned long tstr = p->MN / L, v, j, n, k;
    for (v = 0; v < p->mN; v++) {
        T *pr = c->re + off + (long)v * c->ypst, *pi = c->im + off + (long)v * c->ypst;
        for (j = 0; j < L; j++) {
            T sr = 0, si = 0;
            sr += (pr[0] * p->wr[0] - pi[0] * p->wi[0]);
            si += (pi[0] * p->wr[0] + pr[0] * p->wi[0]);
            k = 0;
            for (n = 1; n < L; n++) {
                T br, bi;
                k += j;
                if (k > L - 1) k -= L;
                br = p->wr[k * tstr]; bi = p->wi[k * tstr];
                sr += (pr[(long)n * es] * br - pi[(long)n * es] * bi);
                si += (pi[(long)n * es] * br + pr[(long)n * es] * bi);
            }
            p->tr[j] = sr; p->ti[j] = si;
        }
        for (j = 0; j < L; j++) { pr[(long)j * es] = p->tr[j]; pi[(long)j * es] = p->ti[j]; }
    }
}

static void FN(orc_bfly)(const CTX *c, unsigned long r, long off, long es)
{
    int inv = (c->p->dir != -1);
    switch (r) {
    case 2: FN(orc_b2)(c, off, es); break;
    case 3: FN(orc_b3)(c, off, es, inv); break;
    case 4: FN(orc_b4)(c, off, es, inv); break;
    case 5: FN(orc_b5)(c, off, es, inv); break;
    case 7: FN(orc_b7)(c, off, es, inv); break;
    case 8: FN(orc_b8)(c, off, es, inv); break;
    default: break;
    }
}

/* Recursive decimation-in-frequency stage driver of VI_p0pFm_f
 * (VI_fftm_building_blocks_f.h:877-1042).  The sub-vector being transformed
 * starts at scalar offset off with elements es scalars apart and has length N. */
static void FN(orc_stage)(const CTX *c, unsigned long s, long off, long es, unsigned long N)
{
    const struct PLAN *p = c->p;
    unsigned long p0 = p->p0[s], pF = p->pF[s], passes = p->pn[s];
    unsigned long Ns = N, N1, wtstr = p->MN / N, seg = 1, wst, i, j, k;
    int last = (s + 1 == p->nstage);
    for (k = 0; k + 1 < passes; k++) {
        N1 = Ns;
        Ns = Ns / p0;
        wst = 0;
        FN(orc_bfly)(c, p0, off, es * (long)Ns);
        for (i = N1; i < N; i += N1) {
            FN(orc_bfly)(c, p0, off + es * (long)i, es * (long)Ns);
            FN(orc_twiddle)(c, off + es * (long)i, es * (long)Ns, p0, wst);
        }
        wst += seg * wtstr;
        for (j = 1; j < Ns; j++) {
            for (i = j; i < N; i += N1) {
                FN(orc_bfly)(c, p0, off + es * (long)i, es * (long)Ns);
                FN(orc_twiddle)(c, off + es * (long)i, es * (long)Ns, p0, wst);
            }
            wst += seg * wtstr;
        }
        seg *= p0;
    }
    N1 = Ns;
    Ns = Ns / pF;
    for (j = 0; j < Ns; j++) {
        for (i = j; i < N; i += N1) {
            long o = off + es * (long)i, e = es * (long)Ns;
            if (pF < 9) FN(orc_bfly)(c, pF, o, e);
            else if (last) FN(orc_dft)(c, o, e, pF);
            else FN(orc_stage)(c, s + 1, o, e, pF);
        }
    }
}

/* Digit-reversal gather of VI_sortm_copy_f (VI_fftm_building_blocks_f.h:47-88). */
static void FN(orc_sort)(const CTX *c)
{
    const struct PLAN *p = c->p;
    unsigned long v, n;
    for (v = 0; v < p->mN; v++) {
        T *pr = c->re + (long)v * c->ypst, *pi = c->im + (long)v * c->ypst;
        for (n = 0; n < p->MN; n++) {
            long q = (long)p->index[n] * c->xst;
            p->tr[n] = pr[q]; p->ti[n] = pi[q];
        }
        for (n = 0; n < p->MN; n++) { pr[(long)n * c->xst] = p->tr[n]; pi[(long)n * c->xst] = p->ti[n]; }
    }
}

/* VI_ccfftmip_f (VI_fftm_building_blocks_f.h:1064-1088) on the view y, with the
 * transform direction of `major`. */
static void FN(orc_ip)(const struct PLAN *p, const CMV *y, int major)
{
    CTX c;
    unsigned long v, n;
    c.p = p;
    c.re = y->re + y->cst * y->off;
    c.im = y->im + y->cst * y->off;
    if (major == 1) {             /* VSIP_COL: vectors are columns */
        c.xst = y->cst * y->col_stride; c.ypst = y->cst * y->row_stride; c.len = y->col_length;
    } else {
        c.xst = y->cst * y->row_stride; c.ypst = y->cst * y->col_stride; c.len = y->row_length;
    }
    if (p->MN > 1) {
        if (p->dft) {
            FN(orc_dft)(&c, 0, c.xst, c.len);
        } else {
            FN(orc_stage)(&c, 0, 0, c.xst, p->MN);
            FN(orc_sort)(&c);
        }
    }
    if (p->scale != 1) {          /* vsip_rscvmul_f per vector */
        for (v = 0; v < p->mN; v++) {
            T *pr = c.re + (long)v * c.ypst, *pi = c.im + (long)v * c.ypst;
            for (n = 0; n < c.len; n++) {
                pr[(long)n * c.xst] = p->scale * pr[(long)n * c.xst];
                pi[(long)n * c.xst] = p->scale * pi[(long)n * c.xst];
            }
        }
    }
}

/* ---------------- plan creation ---------------- */
static void FN(orc_ramp_exp)(T *re, T *im, unsigned long n, T inc)
{
    /* vsip_vramp_f + vsip_vsin_f + vsip_vcos_f (vsip_vramp_f.c:21-34,
     * vsip_scalars.h:30,36): the angle ramp is formed in T, sin/cos in double. */
    unsigned long i;
    for (i = 0; i < n; i++) {
        T a = (i == 0) ? (T)0 : (T)0 + (T)i * inc;
        im[i] = (T)sin((double)a);
        re[i] = (T)cos((double)a);
    }
}

struct PLAN *FN(orc_fftm_create)(int kind, unsigned long M, unsigned long N, T scale,
                                 int dir, int major)
{
    struct PLAN *p = (struct PLAN *)calloc(1, sizeof(struct PLAN));
    const T two_pi = (T)6.28318530717958647692528676655900577;
    const T pi_ = (T)3.14159265358979323846264338327950288;
    unsigned long i;
    if (!p) return NULL;
    p->kind = kind; p->M = M; p->N = N; p->major = major; p->scale = scale;
    if (kind == ORC_RCOP || kind == ORC_CROP) {
        p->MN = (major == 0) ? N / 2 : M / 2;
        p->mN = (major == 0) ? M : N;
        p->dir = (kind == ORC_RCOP) ? -1 : 1;
    } else {
        p->MN = (major == 1) ? M : N;
        p->mN = (major == 1) ? N : M;
        p->dir = dir;
    }
    p->wr = (T *)calloc(p->MN + 1, sizeof(T)); p->wi = (T *)calloc(p->MN + 1, sizeof(T));
    p->tr = (T *)calloc(p->MN + 1, sizeof(T)); p->ti = (T *)calloc(p->MN + 1, sizeof(T));
    p->index = (unsigned long *)calloc(p->MN + 1, sizeof(unsigned long));
    p->er = (T *)calloc(p->MN + 2, sizeof(T)); p->ei = (T *)calloc(p->MN + 2, sizeof(T));
    p->mr = (T *)calloc(p->MN + 2, sizeof(T)); p->mi = (T *)calloc(p->MN + 2, sizeof(T));
    if (kind == ORC_CROP) {
        p->yr = (T *)calloc((p->MN + 1) * (p->mN ? p->mN : 1), 2 * sizeof(T));
        p->yi = p->yr ? p->yr + 1 : NULL;
    }
    if (!p->wr || !p->wi || !p->tr || !p->ti || !p->index || !p->er || !p->ei || !p->mr ||
        !p->mi || (kind == ORC_CROP && !p->yr)) {
        FN(orc_fftm_destroy)(p);
        return NULL;
    }
    p->nstage = orc_factor(p->MN, p->pn, p->p0, p->pF);
    /* twiddle table: ramp step (-+2pi)/MN formed in T (VI_ccfftmop_create_f_def.h:66-72) */
    if (p->MN > 0) {
        T inc = (p->dir == -1) ? (-two_pi) / (T)p->MN : two_pi / (T)p->MN;
        FN(orc_ramp_exp)(p->wr, p->wi, p->MN, inc);
        if (kind == ORC_RCOP || kind == ORC_CROP) {
            T einc = (kind == ORC_RCOP) ? (-pi_) / (T)p->MN : pi_ / (T)p->MN;
            FN(orc_ramp_exp)(p->er, p->ei, p->MN + 1, einc);
        }
    }
    p->dft = (p->nstage > 0 && p->p0[0] == 1 && p->pF[0] == p->MN) ? 1 : 0;
    if (p->nstage > 0) {
        unsigned long pF = p->pF[p->nstage - 1];
        for (i = 0; i < p->MN; i++) p->index[i] = orc_jofk(i, p->pn, p->p0, pF, p->nstage);
    }
    return p;
}

void FN(orc_fftm_destroy)(struct PLAN *p)
{
    if (!p) return;
    free(p->wr); free(p->wi); free(p->tr); free(p->ti); free(p->index);
    free(p->er); free(p->ei); free(p->mr); free(p->mi); free(p->yr);
    free(p);
}

/* ---------------- execution entry points ---------------- */
/* VI_cmcopy_f_f (VI_cmcopy_f_f.h:22-68): traversal follows the output strides. */
static void FN(orc_cmcopy)(const CMV *a, const CMV *r)
{
    unsigned long nmj, nmn, i, j;
    long amj, amn, rmj, rmn;
    if (r->row_stride < r->col_stride) {
        nmj = r->row_length; nmn = r->col_length;
        rmj = r->row_stride; rmn = r->col_stride; amj = a->row_stride; amn = a->col_stride;
    } else {
        nmn = r->row_length; nmj = r->col_length;
        rmn = r->row_stride; rmj = r->col_stride; amn = a->row_stride; amj = a->col_stride;
    }
    for (i = 0; i < nmn; i++) {
        for (j = 0; j < nmj; j++) {
            long ai = a->cst * (a->off + (long)i * amn + (long)j * amj);
            long ri = r->cst * (r->off + (long)i * rmn + (long)j * rmj);
            r->re[ri] = a->re[ai];
            r->im[ri] = a->im[ai];
        }
    }
}

void FN(orc_ccfftmop)(const struct PLAN *p, const CMV *x, const CMV *y)
{
    FN(orc_cmcopy)(x, y);
    FN(orc_ip)(p, y, p->major);
}

void FN(orc_ccfftmip)(const struct PLAN *p, const CMV *y)
{
    FN(orc_ip)(p, y, p->major);
}

#define RIDX(v, i, j) ((v)->rst * ((v)->off + (long)(i) * (v)->col_stride + (long)(j) * (v)->row_stride))
#define CIDX(v, i, j) ((v)->cst * ((v)->off + (long)(i) * (v)->col_stride + (long)(j) * (v)->row_stride))

/* vsip_rcfftmop_f (VI_rcfftmop_f_def.h:24-120). */
void FN(orc_rcfftmop)(const struct PLAN *p, const RMV *x, const CMV *z)
{
    unsigned long MN = p->MN, v, k;
    CMV y = *z;
    if (p->major == 0) {
        for (v = 0; v < x->col_length; v++)
            for (k = 0; k < MN; k++) {
                y.im[CIDX(z, v, k)] = x->a[RIDX(x, v, 2 * k + 1)];
                y.re[CIDX(z, v, k)] = x->a[RIDX(x, v, 2 * k)];
            }
        y.row_length = MN;
    } else {
        for (v = 0; v < x->row_length; v++)
            for (k = 0; k < MN; k++) {
                y.im[CIDX(z, k, v)] = x->a[RIDX(x, 2 * k + 1, v)];
                y.re[CIDX(z, k, v)] = x->a[RIDX(x, 2 * k, v)];
            }
        y.col_length = MN;
    }
    FN(orc_ip)(p, &y, p->major);
    for (v = 0; v < p->mN; v++) {
        /* z: vector v of the output, element k at base + k*zs */
        long base = z->cst * (z->off + (long)v * (p->major == 0 ? z->col_stride : z->row_stride));
        long zs = z->cst * (p->major == 0 ? z->row_stride : z->col_stride);
        T *fr = z->re + base, *fi = z->im + base;
        fr[(long)MN * zs] = fr[0]; fi[(long)MN * zs] = fi[0];
        for (k = 0; k <= MN; k++) { p->mr[MN - k] = fr[(long)k * zs]; p->mi[MN - k] = fi[(long)k * zs]; }
        for (k = 0; k <= MN; k++) {
            T br = p->mr[k], bi = p->mi[k], wr = p->er[k], wi = p->ei[k];
            T Fr = fr[(long)k * zs], Fi = fi[(long)k * zs];
            T t = (T)0.5 * (br + Fr + wr * (bi + Fi) + wi * (Fr - br));
            fi[(long)k * zs] = (T)0.5 * (Fi - bi + wr * (br - Fr) + wi * (bi + Fi));
            fr[(long)k * zs] = t;
        }
    }
}

/* vsip_crfftmop_f (VI_crfftmop_f_def.h:25-126). */
void FN(orc_crfftmop)(const struct PLAN *p, const CMV *z, const RMV *x)
{
    unsigned long MN = p->MN, v, k;
    CMV y;
    for (v = 0; v < p->mN; v++) {
        long base = z->cst * (z->off + (long)v * (p->major == 0 ? z->col_stride : z->row_stride));
        long zs = z->cst * (p->major == 0 ? z->row_stride : z->col_stride);
        const T *fr = z->re + base, *fi = z->im + base;
        T *br = p->yr + 2 * (long)v * (long)(MN + 1), *bi = p->yi + 2 * (long)v * (long)(MN + 1);
        for (k = 0; k <= MN; k++) { br[2 * (long)(MN - k)] = fr[(long)k * zs]; bi[2 * (long)(MN - k)] = fi[(long)k * zs]; }
        for (k = 0; k <= MN; k++) {
            T Fr = fr[(long)k * zs], Fi = fi[(long)k * zs];
            T Br = br[2 * (long)k], Bi = bi[2 * (long)k], wr = p->er[k], wi = p->ei[k];
            T t = Fr + Br + wi * (Br - Fr) - wr * (Fi + Bi);
            bi[2 * (long)k] = Fi - Bi - wi * (Fi + Bi) + wr * (Fr - Br);
            br[2 * (long)k] = t;
        }
    }
    y.re = p->yr; y.im = p->yi; y.cst = 2; y.off = 0;
    y.row_stride = 1; y.col_stride = (long)(MN + 1);
    y.row_length = MN; y.col_length = p->mN;
    FN(orc_ip)(p, &y, 0);
    for (v = 0; v < p->mN; v++)
        for (k = 0; k < MN; k++) {
            long yi = 2 * ((long)v * (long)(MN + 1) + (long)k);
            if (p->major == 0) {
                x->a[RIDX(x, v, 2 * k)] = p->yr[yi];
                x->a[RIDX(x, v, 2 * k + 1)] = p->yi[yi];
            } else {
                x->a[RIDX(x, 2 * k, v)] = p->yr[yi];
                x->a[RIDX(x, 2 * k + 1, v)] = p->yi[yi];
            }
        }
}
#undef RIDX
#undef CIDX

/* all-cores baseline: each thread owns a plan and a disjoint slab of rows */
struct FN(orc_mt_arg) { unsigned long r0, nr, N; int dir; T scale; const T *x; T *y; int rc; };

static void *FN(orc_mt_worker)(void *vp)
{
    struct FN(orc_mt_arg) *a = (struct FN(orc_mt_arg) *)vp;
    struct PLAN *p;
    CMV xv, yv;
    a->rc = 0;
    if (a->nr == 0) return NULL;
    p = FN(orc_fftm_create)(ORC_CCOP, a->nr, a->N, a->scale, a->dir, 0);
    if (!p) { a->rc = 1; return NULL; }
    xv.re = (T *)a->x; xv.im = (T *)a->x + 1; xv.cst = 2;
    xv.off = (long)(a->r0 * a->N); xv.col_stride = (long)a->N; xv.row_stride = 1;
    xv.col_length = a->nr; xv.row_length = a->N;
    yv = xv; yv.re = a->y; yv.im = a->y + 1;
    FN(orc_ccfftmop)(p, &xv, &yv);
    FN(orc_fftm_destroy)(p);
    return NULL;
}

int FN(orc_ccfftmop_rows_mt)(unsigned long rows, unsigned long N, int dir, T scale,
                             const T *x, T *y, int threads)
{
    pthread_t th[256];
    struct FN(orc_mt_arg) args[256];
    int t, rc = 0;
    unsigned long per, r0 = 0;
    if (threads < 1) threads = 1;
    if (threads > 256) threads = 256;
    per = (rows + (unsigned long)threads - 1) / (unsigned long)threads;
    for (t = 0; t < threads; t++) {
        args[t].r0 = r0; args[t].nr = (r0 >= rows) ? 0 : ((rows - r0 < per) ? rows - r0 : per);
        args[t].N = N; args[t].dir = dir; args[t].scale = scale; args[t].x = x; args[t].y = y;
        r0 += args[t].nr;
        if (pthread_create(&th[t], NULL, FN(orc_mt_worker), &args[t]) != 0) { args[t].rc = 1; th[t] = 0; }
    }
    for (t = 0; t < threads; t++) {
        if (th[t]) pthread_join(th[t], NULL);
        rc |= args[t].rc;
    }
    return rc;
}

#undef FN
#undef PLAN
#undef CMV
#undef RMV
#undef CTX
#undef ORC_CAT
#undef ORC_CAT2
